"""Crack-like boundaries (dual BEM) on the device against the oracle, through
the C-ABI (mfbem_mesh_upload_dual with crack_el / ctype2 / cvalue2).

A crack node carries both faces' unknowns and two equations, SBIE and HBIE,
at the same points, in the reference's interleaved rows
(build_auxiliary_variables_mechanics_static.f90:146-207); face 2 takes -h, g,
-m, l of the element (build_lse_mechanics_bem_staela.f90:883-887) and the free
terms of staela.f90:195-204 / harela.f90:344-360. The oracle is pinned by
Sneddon's penny crack (tests/test_oracle_crack.py). Meshes: the pressurised
penny crack alone, and inside a clamped cube (ordinary rows after the six-row
crack nodes; ordinary points integrating the crack's faces and crack points
integrating the cube). The hypersingular cancellation makes vanishing
entries rounding residues, so the tolerance is max(floor, 4 x the oracle's
own change when the HBIE points move by one part in 4e-16), at most 2e-9.
"""
import ctypes

import numpy as np
import pytest

from multifebe_gb300 import meshgen as M, BemRegion, MfbemError
from multifebe_gb300 import _abi

pytestmark = pytest.mark.gpu

DELTA = 0.22540333
CASES = [("penny", lambda: M.penny_crack(1.0, 2, 2, 1.0)), ("penny_in_box", lambda: M.penny_crack_in_box(1.0, 2, 1, 2.0, 2))]


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def tol_of(sens, floor):
    return min(max(floor, 4.0 * sens), 2e-9)


def oracle_pair(oracle, d, crack, build):
    out = []
    for dl in (DELTA, DELTA * (1 + 4e-16)):
        P = oracle.Problem(d)
        P.set_formulation("sbie", delta=dl)
        P.set_crack(*crack)
        out.append((P, build(P)))
    (P, s0), (_, s1) = out
    return P, s0, s1


def hbie_counts(R):
    L = _abi.load()
    L.mfbem_internal_hbie_counts.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    out = np.zeros(21, dtype=np.int64)
    _abi.check(L.mfbem_internal_hbie_counts(R._h, out.ctypes.data))
    return out.reshape(3, 7)


@pytest.mark.parametrize("name,mk", CASES, ids=[c[0] for c in CASES])
def test_static_assembly_matches_oracle(oracle, name, mk):
    d, crack = mk()
    mat = M.elastic(1.0, 0.25)
    P, (Ao, bo), (A1, b1) = oracle_pair(oracle, d, crack, lambda P: P.assemble_staela(mat["mu"], mat["nu"]))
    tA, tb = tol_of(rel(A1, Ao), 1e-11), tol_of(rel(b1, bo), 1e-11)
    R = BemRegion(d, crack=crack)
    assert R.n == P.n
    A, b = R.build_lse_staela(mat["mu"], mat["nu"])
    c = hbie_counts(R)
    s = R.stats()
    print(name, "A", rel(A, Ao), "b", rel(b, bo), "tolerances", tA, tb, "HBIE pairs", c[0, :3], "oracle",
          P.stats[8:11])
    assert (c[0, 0], c[0, 1], c[0, 2]) == (P.stats[8], P.stats[9], P.stats[10])
    assert s["pairs_regular"] + c[1, 0] == P.stats[0]
    assert s["pairs_adaptive"] + c[1, 1] == P.stats[1]
    assert s["pairs_singular"] + c[1, 2] == P.stats[2]
    assert rel(A, Ao) <= tA and rel(b, bo) <= tb
    R.close()


@pytest.mark.parametrize("name,mk", CASES, ids=[c[0] for c in CASES])
def test_harmonic_assembly_matches_oracle(oracle, name, mk):
    d, crack = mk()
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    R = BemRegion(d, crack=crack)
    for om in (0.5, 2.0):
        P, (Ao, bo), (A1, b1) = oracle_pair(oracle, d, crack, lambda P: P.assemble_harela(mat, om))
        tA, tb = tol_of(rel(A1, Ao), 1e-11), tol_of(rel(b1, bo), 1e-11)
        A, b = R.build_lse_harela(mat, om)
        print(name, om, "A", rel(A, Ao), "b", rel(b, bo), "tolerances", tA, tb)
        assert rel(A, Ao) <= tA and rel(b, bo) <= tb
    c = hbie_counts(R)
    s = R.stats()
    assert (c[0, 0], c[0, 1], c[0, 2]) == (P.stats[8], P.stats[9], P.stats[10])
    # shbie_auto: the crack nodes' SBIE shares the HBIE's classification
    assert s["pairs_regular"] + c[2, 0] == P.stats[0]
    assert s["pairs_singular"] + c[2, 2] == P.stats[2]
    R.close()


@pytest.mark.parametrize("precision,tol", [("plain", 1e-10), ("mixed", 1e-8)])
def test_static_solve_sneddon(oracle, precision, tol):
    d, crack = M.penny_crack(1.0, 2, 2, 1.0)
    E, nu = 1.0, 0.25
    mat = M.elastic(E, nu)
    _, xo, x1 = oracle_pair(oracle, d, crack, lambda P: oracle.lu_solve(*P.assemble_staela(mat["mu"], mat["nu"])))
    R = BemRegion(d, crack=crack)
    x = R.solve_staela(mat["mu"], mat["nu"], precision=precision)
    assert rel(x, xo) <= tol_of(rel(x1, xo), tol)
    u1, t1, u2, t2 = R.solution_faces(x)
    c = np.argmin(np.linalg.norm(d.nodes, axis=1))
    ex = M.sneddon_opening(0.0, 1.0, 1.0, E, nu)
    assert abs(u2[c, 2] - u1[c, 2] - ex) < 2e-3 * ex
    assert np.allclose(t1[:, 2], -1.0) and np.allclose(t2[:, 2], 1.0)
    R.close()


@pytest.mark.parametrize("precision,tol", [("plain", 1e-10), ("mixed", 1e-8)])
def test_harmonic_sweep(oracle, precision, tol):
    d, crack = M.penny_crack_in_box(1.0, 2, 1, 2.0, 2)
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    oms = np.array([0.5, 1.5])
    R = BemRegion(d, crack=crack)
    X = R.sweep_harela(mat, oms, precision=precision)
    for i, om in enumerate(oms):
        _, xo, x1 = oracle_pair(oracle, d, crack, lambda P: oracle.lu_solve(*P.assemble_harela(mat, om)))
        t = tol_of(rel(x1, xo), tol)
        assert rel(X[i], xo) <= t, (precision, om, rel(X[i], xo), t)
    R.close()


def test_crack_errors():
    d, crack = M.penny_crack(1.0, 2, 1, 1.0)
    R = BemRegion(d, crack=crack)
    with pytest.raises(MfbemError) as e:
        R.set_halfspace(-3, -1.0, 1)
    assert e.value.code == _abi.MFBEM_EUNSUPPORTED
    # a crack node whose formulation flags are not the dual BEM's
    L = _abi.load()
    dd = L.mfbem_prep_dual(R._prep).contents
    nn = d.n_nodes
    du = np.ctypeslib.as_array(dd.dual, shape=(nn,))
    keep = du.copy()
    du[0] = 1
    h = ctypes.c_void_p()
    rc = L.mfbem_mesh_upload_dual(R.desc, ctypes.byref(dd), ctypes.byref(h))
    du[:] = keep
    assert rc == _abi.MFBEM_EARG and not h.value
    R.close()
    # a node shared by crack-like and ordinary elements
    ce = crack[0].copy()
    ce[0] = False
    with pytest.raises(ValueError):
        BemRegion(d, crack=(ce, crack[1], crack[2]))


@pytest.mark.parametrize("harmonic", [False, True])
def test_internal_points_with_both_faces(oracle, harmonic):
    """mfbem_internal_points_faces_*: face 2 integrated with the reversed
    element (calculate_internal_points_mechanics_static.f90:320-354,431-465),
    device against the oracle (<= 1e-10, max-norm relative) inside the cube
    around the crack, near it and far from it; the single-face entry points and
    a point at a crack node are refused."""
    d, crack = M.penny_crack_in_box(1.0, 2, 1, 2.0, 2)
    P = oracle.Problem(d)
    P.set_crack(*crack)
    R = BemRegion(d, crack=crack)
    xp = np.array([[0.3, 0.2, 0.4], [-0.5, 0.1, -0.3], [1.2, 0.0, 0.1], [0.0, 0.0, 0.05], [0.1, -1.5, 1.5]])
    if harmonic:
        mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
        om = 0.8
        x = R.sweep_harela(mat, [om], precision="plain")[0]
        kw = dict(mat=mat, omega=om)
    else:
        mat = M.elastic(1.0, 0.25)
        x = R.solve_staela(mat["mu"], mat["nu"], precision="plain")
        kw = dict(mu=mat["mu"], nu=mat["nu"])
    u1, t1, u2, t2 = R.solution_faces(x)
    ud, sd = R.internal_points(xp, u1, t1, u2=u2, t2=t2, **kw)
    uo, so = P.internal_points(xp, u1, t1, u2=u2, t2=t2, **kw)
    print("harmonic" if harmonic else "static", "u", rel(ud, uo), "sigma", rel(sd, so))
    assert rel(ud, uo) <= 1e-10 and rel(sd, so) <= 1e-10
    with pytest.raises(MfbemError) as e:
        R.internal_points(xp, u1, t1, **kw)
    assert e.value.code == _abi.MFBEM_EUNSUPPORTED
    c = np.nonzero(crack[0])[0][0]
    with pytest.raises(MfbemError) as e:
        R.internal_points(d.nodes[d.conn[c, :1]], u1, t1, u2=u2, t2=t2, **kw)
    assert e.value.code == _abi.MFBEM_EUNSUPPORTED
    R.close()
