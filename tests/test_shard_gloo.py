"""Frequency sharding of a sweep over ranks: host logic on CPU, world_size 2
over gloo (the per-rank solver is a stand-in; the device sweep itself is
covered by the GPU tests)."""
import os
import socket

import numpy as np
import pytest

from multifebe_gb300 import shard


def test_frequency_shard_partitions_the_sweep():
    for n in (1, 5, 20, 21):
        for w in (1, 2, 3, 8):
            got = np.concatenate([shard.frequency_shard(n, r, w) for r in range(w)])
            assert np.array_equal(np.sort(got), np.arange(n))
    with pytest.raises(ValueError):
        shard.frequency_shard(4, 2, 2)


def test_weak_scaled_frequencies():
    a = shard.weak_scaled_frequencies(0.1, 2.0, 20, 1)
    assert len(a) == 20 and a[0] == 0.1 and a[-1] == 2.0
    assert len(shard.weak_scaled_frequencies(0.1, 2.0, 20, 4)) == 80


class _FakeRegion:
    """Solver stand-in: solution of frequency w is w * (1..n) + rank-independent."""
    n = 6

    def sweep_harela(self, material, omegas, precision="mixed"):
        return np.array([w * np.arange(1, self.n + 1) * (1 + 1j) for w in omegas])


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, omegas, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out = shard.sweep_sharded(_FakeRegion(), None, omegas, rank=rank, world=world, dist=dist)
        if rank == 0:
            q.put(out)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_sweep_sharded_gloo_world2():
    import torch.multiprocessing as mp
    omegas = np.linspace(0.1, 2.0, 7)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, omegas, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    ref = _FakeRegion().sweep_harela(None, omegas)
    assert np.array_equal(out, ref)
