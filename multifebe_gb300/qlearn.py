"""Learned quadrature order / subdivision for near-singular pairs.

The rule family and the network are described in csrc/mfbem_learned.cuh. This
module draws the seeded random training pairs (quad8 elements and collocation
points at distance / size ratios log-uniform in [1e-3, 2]), has the library
label them on the GPU (each candidate rule's relative error against a
converged rule, and the reference adaptive rule's error and point count),
trains the MLP with the library's own kernels and hands the weights to a mesh.

    feats, y, cost, valid = label_pairs(*random_pairs(4096, seed=1))
    w = init_weights(seed=0)
    loss = train(w, feats, y, valid, steps=3000)
    region.set_learned_quadrature(w, log10_tol=-6)
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from ._abi import check

_vp = ctypes.c_void_p

NF, NT, NG, NL = 8, 7, 9, 5
NC = NT + NG * NL
ORDERS = (3, 4, 6, 8, 10, 12, 16, 20, 30)
# candidate c < NT: the reference adaptive rule at qsi_relative_error 10^-(3+c)
# (the method's default 1e-6 is c = 3); c >= NT: graded depth (c-NT)//NG,
# order ORDERS[(c-NT)%NG]
REF_DEFAULT = 3


def _lib():
    L = _abi.load()
    if not getattr(L, "_ql_set", False):
        L.mfbem_qlearn_label.argtypes = [ctypes.c_int32, _vp, _vp, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp]
        L.mfbem_mlp_size.restype = ctypes.c_int32
        L.mfbem_mlp_forward.argtypes = [_vp, ctypes.c_int32, _vp, _vp]
        L.mfbem_mlp_loss_grad.argtypes = [_vp, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp]
        L.mfbem_mlp_train.argtypes = [_vp, ctypes.c_int32, _vp, _vp, _vp, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_float, ctypes.c_uint64, _vp]
        L.mfbem_set_learned_quadrature.argtypes = [_vp, _vp, ctypes.c_double, ctypes.c_int32, ctypes.c_double, _vp]
        L._ql_set = True
    return L


def n_weights() -> int:
    return int(_lib().mfbem_mlp_size())


# ------------------------------------------------------------------ pairs
_XI = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1], [0, -1], [1, 0], [0, 1], [-1, 0]], dtype=np.float64)


def _phi_q8(x1, x2):
    """quad8 shape functions and derivatives (node order of _XI)."""
    phi = np.empty(8)
    d1 = np.empty(8)
    d2 = np.empty(8)
    for k in range(4):
        a, b = _XI[k]
        phi[k] = 0.25 * (1 + a * x1) * (1 + b * x2) * (a * x1 + b * x2 - 1)
        d1[k] = 0.25 * a * (1 + b * x2) * (2 * a * x1 + b * x2)
        d2[k] = 0.25 * b * (1 + a * x1) * (a * x1 + 2 * b * x2)
    for k in range(4, 8):
        a, b = _XI[k]
        if a == 0:
            phi[k] = 0.5 * (1 - x1 * x1) * (1 + b * x2)
            d1[k] = -x1 * (1 + b * x2)
            d2[k] = 0.5 * b * (1 - x1 * x1)
        else:
            phi[k] = 0.5 * (1 + a * x1) * (1 - x2 * x2)
            d1[k] = 0.5 * a * (1 - x2 * x2)
            d2[k] = -x2 * (1 + a * x1)
    return phi, d1, d2


def random_pairs(n: int, seed: int, kernel: int = 0):
    """n seeded random (quad8 element, point) pairs: element size 10^U(-1,1),
    aspect ratio 10^U(0,0.6), curvature and mid-side jitter, random rigid
    motion; the point sits off a random parametric location in [-1.2,1.2]^2
    at distance / size log-uniform in [1e-3, 2]. kernel 1 adds |k| x size
    U(0, 0.5) per pair. Returns (elem [n,8,3], pts [n,3], kernel, kcl [n])."""
    rng = np.random.default_rng(seed)
    elem = np.empty((n, 8, 3))
    pts = np.empty((n, 3))
    for s in range(n):
        size = 10.0 ** rng.uniform(-1, 1)
        asp = 10.0 ** rng.uniform(0, 0.6)
        kap = rng.uniform(-0.3, 0.3)
        loc = _XI * np.array([0.5 * size * asp, 0.5 * size])
        loc[4:] += rng.uniform(-0.05, 0.05, (4, 2)) * size
        z = kap * (loc[:, 0] ** 2 + loc[:, 1] ** 2) / size
        x = np.column_stack([loc, z])
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        x = x @ q.T + rng.normal(size=3) * size
        elem[s] = x
        xi = rng.uniform(-1.2, 1.2, 2)
        phi, d1, d2 = _phi_q8(*xi)
        p0 = phi @ x
        nrm = np.cross(d1 @ x, d2 @ x)
        nrm /= np.linalg.norm(nrm)
        ratio = 10.0 ** rng.uniform(-3, np.log10(2.0))
        pts[s] = p0 + (1 if rng.uniform() < 0.5 else -1) * ratio * size * max(asp, 1.0) * nrm
    kcl = rng.uniform(0.0, 0.5, n) if kernel else np.zeros(n)
    return elem, pts, kernel, kcl


def label_pairs(elem, pts, kernel=0, kcl=None):
    """GPU labels: (features [n,NF], log10 candidate errors [n,NC], candidate
    quadrature points [n,NC] (-1: not available), valid [n])."""
    n = len(pts)
    elem = np.ascontiguousarray(elem, dtype=np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    kc = np.ascontiguousarray(kcl if kcl is not None else np.zeros(n), dtype=np.float64)
    f = np.zeros((n, NF), np.float32)
    y = np.zeros((n, NC), np.float32)
    c = np.zeros((n, NC), np.int32)
    v = np.zeros(n, np.int32)
    check(_lib().mfbem_qlearn_label(n, elem.ctypes.data, pts.ctypes.data, kernel, kc.ctypes.data, f.ctypes.data,
                                    y.ctypes.data, c.ctypes.data, v.ctypes.data))
    return f, y, c, v


# ------------------------------------------------------------------ network
def init_weights(seed: int = 0) -> np.ndarray:
    """Glorot-uniform weights, zero biases, in the library's layout."""
    rng = np.random.default_rng(seed)
    H = 64
    parts = []
    for fan_in, fan_out in ((NF, H), (H, H), (H, H), (H, NC)):
        a = np.sqrt(6.0 / (fan_in + fan_out))
        parts.append(rng.uniform(-a, a, fan_out * fan_in))
        parts.append(np.zeros(fan_out))
    w = np.concatenate(parts).astype(np.float32)
    assert w.size == n_weights()
    return w


def forward(w, feats):
    f = np.ascontiguousarray(feats, np.float32)
    out = np.zeros((len(f), NC), np.float32)
    check(_lib().mfbem_mlp_forward(np.ascontiguousarray(w, np.float32).ctypes.data, len(f), f.ctypes.data,
                                   out.ctypes.data))
    return out


def loss_grad(w, feats, y, valid=None):
    f = np.ascontiguousarray(feats, np.float32)
    yy = np.ascontiguousarray(y, np.float32)
    vv = np.ascontiguousarray(valid if valid is not None else np.ones(len(f)), np.int32)
    loss = np.zeros(1, np.float32)
    g = np.zeros(n_weights(), np.float32)
    check(_lib().mfbem_mlp_loss_grad(np.ascontiguousarray(w, np.float32).ctypes.data, len(f), f.ctypes.data,
                                     yy.ctypes.data, vv.ctypes.data, loss.ctypes.data, g.ctypes.data))
    return float(loss[0]), g


def train(w, feats, y, valid=None, steps=3000, batch=1024, lr=2e-3, seed=0):
    """Adam on device-drawn mini-batches; updates w in place, returns the
    per-step mini-batch loss."""
    assert w.dtype == np.float32 and w.flags.c_contiguous
    f = np.ascontiguousarray(feats, np.float32)
    yy = np.ascontiguousarray(y, np.float32)
    vv = np.ascontiguousarray(valid if valid is not None else np.ones(len(f)), np.int32)
    hist = np.zeros(steps, np.float32)
    check(_lib().mfbem_mlp_train(w.ctypes.data, len(f), f.ctypes.data, yy.ctypes.data, vv.ctypes.data, steps, batch,
                                 lr, seed, hist.ctypes.data))
    return hist


def choose(pred, cost, log10_tol, fallback=REF_DEFAULT):
    """Per pair the cheapest candidate (by `cost`, the quadrature points) whose
    predicted log10 error is <= log10_tol; `fallback` (the reference rule at
    the mesh's qsi_relative_error: candidate 3 for the default 1e-6, 4 for
    1e-7) when none qualifies -- the selection the library makes."""
    ok = (pred <= log10_tol) & (cost > 0)
    cc = np.where(ok, cost, np.iinfo(np.int32).max)
    c = cc.argmin(1)
    return np.where(ok.any(1), c, fallback)


def reference_candidate(qsi_relative_error):
    """Candidate index of the reference adaptive rule at a tolerance 10^-(3+c)."""
    c = int(round(-np.log10(qsi_relative_error))) - 3
    if not 0 <= c < NT:
        raise ValueError("no reference-rule candidate for this tolerance")
    return c


def mesh_adaptive_pairs(region):
    """The quasi-singular (adaptive) pairs of a mesh on the device: element
    node coordinates [n,8,3] and collocation points [n,3], as label_pairs
    takes them, and the element index of each pair."""
    L = _abi.load()
    if not getattr(L, "_ap_set", False):
        L.mfbem_internal_adaptive_pairs.argtypes = [_vp, _vp, _vp, _vp]
        L._ap_set = True
    n = np.zeros(1, np.int32)
    check(L.mfbem_internal_adaptive_pairs(region._h, n.ctypes.data, None, None))
    pts = np.zeros((int(n[0]), 3))
    el = np.zeros(int(n[0]), np.int32)
    check(L.mfbem_internal_adaptive_pairs(region._h, n.ctypes.data, pts.ctypes.data, el.ctypes.data))
    d = region.deck
    return d.nodes[d.conn[el]], pts, el
