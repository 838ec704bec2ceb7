"""HBIE collocation on the boundary ('hbie', 'dual_bm_same' and
'dual_bm_mixed' formulations) on the device against the oracle, through the
C-ABI (mfbem_mesh_upload_dual).

The oracle restates the builders' HBIE branches (build_lse_mechanics_bem_staela.f90:
783-842,938-997, build_lse_mechanics_bem_harela.f90:1144-1284), hbie_auto /
hbie_int (lib/fbem/src/bem_staela3d.f90:4307-5578, bem_harela3d.f90:3169-3697)
and shbie_auto (bem_harela3d.f90:4888-4957); it is pinned by the closed forms
of tests/test_oracle_hbie.py. Pair counts are identical. The hypersingular
integration cancels large polar and line integrals, so entries that vanish
in exact arithmetic carry rounding residues: moving the HBIE points by one
part in 4e-16 (delta_hbie * (1 + 4e-16)) changes the oracle's own A by ~2e-10
(max-norm relative) on these meshes. The tolerance of A, b and of the
solutions is therefore max(1e-11 | 1e-10, 4 x that sensitivity of the oracle),
measured in each test, and never above 2e-9.
"""
import ctypes

import numpy as np
import pytest

from multifebe_gb300 import meshgen as M, BemRegion, MfbemError
from multifebe_gb300 import _abi

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def hbie_counts(R):
    L = _abi.load()
    L.mfbem_internal_hbie_counts.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    out = np.zeros(21, dtype=np.int64)
    _abi.check(L.mfbem_internal_hbie_counts(R._h, out.ctypes.data))
    return out.reshape(3, 7)


def mixed_codes(d):
    """Per-node codes: SBIE, 'hbie', 'dual_bm_same' and 'dual_bm_mixed' nodes
    in one region."""
    f = np.full(d.n_nodes, 2, dtype=np.int32)
    f[d.nodes[:, 2] > 0.99] = 1
    f[d.nodes[:, 1] < 0.01] = 3
    f[d.nodes[:, 0] < 0.01] = 0
    return f


DELTA = 0.22540333


def sensitivity(d, f, alpha, build):
    """Oracle systems at delta_hbie and at delta_hbie * (1 + 4e-16): the
    reference system and its rounding-level sensitivity."""
    out = []
    for dl in (DELTA, DELTA * (1 + 4e-16)):
        P = oracle_mod().Problem(d)
        P.set_formulation(f, alpha=alpha, delta=dl)
        out.append((P, build(P)))
    (P, s0), (_, s1) = out
    return P, s0, s1


def oracle_mod():
    import oracle
    return oracle


def tol_of(sens, floor):
    return min(max(floor, 4.0 * sens), 2e-9)


DECKS = [("cube2", lambda: M.cube_clamped_top_traction(2)), ("kat2", lambda: M.cube_confined_kat(2)),
         ("patch", lambda: M.surface_patch(2.0, 4, 1.0))]
FORMS = ["hbie", "dual_bm", "dual_bm_mixed", "codes"]


def form_of(name, d):
    return mixed_codes(d) if name == "codes" else name


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("name,mk", DECKS, ids=[c[0] for c in DECKS])
def test_static_assembly_matches_oracle(oracle, name, mk, form):
    d = mk()
    mat = M.elastic(1.0, 0.25)
    f = form_of(form, d)
    alpha = 0.7
    P, (Ao, bo), (A1, b1) = sensitivity(d, f, alpha, lambda P: P.assemble_staela(mat["mu"], mat["nu"]))
    tA, tb = tol_of(rel(A1, Ao), 1e-11), tol_of(rel(b1, bo), 1e-11)
    R = BemRegion(d, formulation=f, alpha=alpha)
    A, b = R.build_lse_staela(mat["mu"], mat["nu"])
    c = hbie_counts(R)
    print(name, form, "HBIE pairs reg/adp/sing", c[0, :3], "oracle", P.stats[8:11], "A", rel(A, Ao), "b", rel(b, bo),
          "tolerances", tA, tb)
    assert (c[0, 0], c[0, 1], c[0, 2]) == (P.stats[8], P.stats[9], P.stats[10])
    # SBIE pairs: the SBIE nodes' points plus the Burton & Miller points (static classification)
    s = R.stats()
    assert s["pairs_regular"] + c[1, 0] == P.stats[0]
    assert s["pairs_adaptive"] + c[1, 1] == P.stats[1]
    assert s["pairs_singular"] + c[1, 2] == P.stats[2]
    assert rel(A, Ao) <= tA and rel(b, bo) <= tb
    R.close()


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("name,mk", DECKS[:2], ids=[c[0] for c in DECKS[:2]])
def test_harmonic_assembly_matches_oracle(oracle, name, mk, form):
    d = mk()
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    f = form_of(form, d)
    R = BemRegion(d, formulation=f, alpha=1.3)
    for a0 in (0.4, 1.7):
        om = float(M.omega_from_a0(a0, mat))
        P, (Ao, bo), (A1, b1) = sensitivity(d, f, 1.3, lambda P: P.assemble_harela(mat, om))
        tA, tb = tol_of(rel(A1, Ao), 1e-11), tol_of(rel(b1, bo), 1e-11)
        A, b = R.build_lse_harela(mat, om)
        print(name, form, a0, "A", rel(A, Ao), "b", rel(b, bo), "tolerances", tA, tb)
        assert rel(A, Ao) <= tA and rel(b, bo) <= tb
    c = hbie_counts(R)
    assert (c[0, 0], c[0, 1], c[0, 2]) == (P.stats[8], P.stats[9], P.stats[10])
    if form != "hbie":
        # shbie_auto: the SBIE part shares the HBIE's classification
        s = R.stats()
        assert s["pairs_regular"] + c[2, 0] == P.stats[0]
        assert s["pairs_singular"] + c[2, 2] == P.stats[2]
    R.close()


@pytest.mark.parametrize("precision,tol", [("plain", 1e-10), ("mixed", 1e-8)])
def test_static_solve_burton_miller(oracle, precision, tol):
    d = M.cube_confined_kat(2)
    mat = M.elastic(1.0, 0.25)
    _, xo, x1 = sensitivity(d, "dual_bm", 1.0,
                            lambda P: oracle.lu_solve(*P.assemble_staela(mat["mu"], mat["nu"])))
    R = BemRegion(d, formulation="dual_bm")
    x = R.solve_staela(mat["mu"], mat["nu"], precision=precision)
    assert rel(x, xo) <= tol_of(rel(x1, xo), tol)
    u, _ = R.solution(x)
    assert np.abs(u[:, 0] - (1.25 * 0.5 / 0.75) * d.nodes[:, 0]).max() < 2e-5
    R.close()


@pytest.mark.parametrize("precision,tol", [("plain", 1e-10), ("mixed", 1e-8)])
@pytest.mark.parametrize("form", ["hbie", "dual_bm", "dual_bm_mixed"])
def test_harmonic_sweep(oracle, form, precision, tol):
    """ME-TH-EL-001 column: the sweep's solutions equal the oracle's LU
    solutions and converge to the closed form like the oracle's."""
    d = M.cube_confined_kat(2)
    mat = M.viscoelastic(2.4, 0.2, 1.0, 0.02)
    oms = np.array([2.0, 5.0])
    R = BemRegion(d, formulation=form)
    X = R.sweep_harela(mat, oms, precision=precision)
    for i, om in enumerate(oms):
        _, xo, x1 = sensitivity(d, form, 1.0, lambda P: oracle.lu_solve(*P.assemble_harela(mat, om)))
        t = tol_of(rel(x1, xo), tol)
        assert rel(X[i], xo) <= t, (form, precision, om, rel(X[i], xo), t)
    R.close()


def test_hbie_errors():
    d = M.halfspace_footing(1.0, 2, 1.0)
    R = BemRegion(d, formulation="dual_bm")
    with pytest.raises(MfbemError) as e:
        R.set_halfspace(-3, 0.0, 1)
    assert e.value.code == _abi.MFBEM_EUNSUPPORTED
    R.close()
    # a combination outside the formulations (dual without the HBIE)
    R0 = BemRegion(d)
    L = _abi.load()
    nn, ne = d.n_nodes, d.n_elements
    keep = [np.zeros(nn, np.int32), np.ones(nn, np.int32), np.ones(nn, np.int32), np.ones(nn),
            np.zeros(16 * ne), np.zeros(24 * ne), np.zeros(24 * ne)]
    dd = _abi.DualDesc(*[k.ctypes.data_as(_abi._ip if k.dtype == np.int32 else _abi._dp) for k in keep])
    h = ctypes.c_void_p()
    rc = L.mfbem_mesh_upload_dual(R0.desc, ctypes.byref(dd), ctypes.byref(h))
    assert rc == _abi.MFBEM_EUNSUPPORTED and not h.value
    R0.close()
