"""Frequency sharding of a harmonic sweep over ranks (one process per GPU).

The frequencies of a sweep are independent systems (src/multifebe.f90 loops
over them, building and solving each in turn), so a sweep shards over ranks
with no data-path collective: rank r assembles, factorises and solves the
frequencies r, r + W, r + 2W, ... on its own GPU; the solution vectors are
gathered on the host of rank 0 afterwards (gloo or any backend that carries
CPU tensors). Nothing is exchanged between GPUs.
"""
from __future__ import annotations

import numpy as np


def frequency_shard(n_freq: int, rank: int, world: int) -> np.ndarray:
    """Indices of the frequencies rank `rank` of `world` owns (strided, so
    every rank gets low and high frequencies alike)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"invalid rank {rank} of {world}")
    return np.arange(rank, n_freq, world, dtype=np.int64)


def weak_scaled_frequencies(a0_lo: float, a0_hi: float, per_rank: int, world: int) -> np.ndarray:
    """Global dimensionless frequencies of a weak-scaled sweep: per_rank * world
    values linearly spaced in [a0_lo, a0_hi] (each rank then solves per_rank)."""
    return np.linspace(a0_lo, a0_hi, per_rank * world)


def gather_solutions(local: np.ndarray, idx: np.ndarray, n_freq: int, rank: int, world: int, dist=None):
    """Place every rank's solutions (local[i] belongs to frequency idx[i]) into
    one (n_freq, n) array on rank 0; other ranks get None. `dist` is
    torch.distributed (initialised), or None for a single process."""
    local = np.ascontiguousarray(local)
    if world == 1 or dist is None:
        out = np.zeros((n_freq,) + local.shape[1:], dtype=local.dtype)
        out[idx] = local
        return out
    parts = [None] * world if rank == 0 else None
    dist.gather_object((idx, local), parts, dst=0)
    if rank != 0:
        return None
    out = np.zeros((n_freq,) + local.shape[1:], dtype=local.dtype)
    seen = np.zeros(n_freq, dtype=bool)
    for ix, x in parts:
        if np.any(seen[ix]):
            raise RuntimeError("two ranks returned the same frequency")
        seen[ix] = True
        out[ix] = x
    if not seen.all():
        raise RuntimeError("a frequency of the sweep was not solved by any rank")
    return out


def sweep_sharded(region, material, omegas, precision="mixed", rank=0, world=1, dist=None):
    """Sweep `omegas` over `world` ranks; returns the full solution array on
    rank 0 (None elsewhere)."""
    omegas = np.asarray(omegas, dtype=np.float64)
    idx = frequency_shard(len(omegas), rank, world)
    local = region.sweep_harela(material, omegas[idx], precision=precision) if len(idx) else \
        np.zeros((0, region.n), dtype=np.complex128)
    return gather_solutions(local, idx, len(omegas), rank, world, dist)
