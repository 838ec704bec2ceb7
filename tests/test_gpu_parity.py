"""GPU path against the CPU oracle, through the C-ABI (mfbem_* entry points).

Tolerances (max-norm relative):
  assembled A, b     <= 1e-11 (the near-singular integrands amplify FP64
                     rounding differences between an FMA device and the oracle)
  solutions          <= 1e-10 on well-conditioned systems; <= cond(A) * 1e-12
                     in general (the FP64 method's own sensitivity)
  pair classes       identical counts of regular / adaptive / singular pairs,
                     adaptive leaves and quadrature points
"""
import numpy as np
import pytest

from multifebe_gb300 import meshgen as M, BemRegion, solve_lse, MfbemError
from multifebe_gb300 import _abi

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


STATIC = [("cube4", lambda: M.cube_clamped_top_traction(4)), ("kat2", lambda: M.cube_confined_kat(2))]
HARMONIC = [("cube4", lambda: M.cube_clamped_top_traction(4)), ("patch8", lambda: M.surface_patch(10.0, 8, 1.0)),
            ("slab4", lambda: M.slab(4, 1))]


@pytest.mark.parametrize("name,mk", STATIC, ids=[s[0] for s in STATIC])
def test_assemble_staela_matches_oracle(oracle, name, mk):
    d = mk()
    R = BemRegion(d)
    P = oracle.Problem(d)
    mat = M.elastic(1.0, 0.25)
    A, b = R.build_lse_staela(mat["mu"], mat["nu"])
    Ao, bo = P.assemble_staela(mat["mu"], mat["nu"])
    st = R.stats()
    assert (st["pairs_regular"], st["pairs_adaptive"], st["pairs_singular"]) == tuple(P.stats[:3])
    assert st["adaptive_leaves"] == P.stats[3] and st["points_adaptive"] == P.stats[4]
    assert rel(A, Ao) < 1e-11 and rel(b, bo) < 1e-11
    # accumulate semantics: a second call adds the same contribution
    A2, b2 = R.build_lse_staela(mat["mu"], mat["nu"], A.copy(order="F"), b.copy())
    assert rel(A2, 2 * A) < 1e-15 and rel(b2, 2 * b) < 1e-15
    R.close()


@pytest.mark.parametrize("name,mk", HARMONIC, ids=[s[0] for s in HARMONIC])
def test_assemble_harela_matches_oracle(oracle, name, mk):
    d = mk()
    R = BemRegion(d)
    P = oracle.Problem(d)
    mat = M.viscoelastic(1.0, 0.3, 1.0, 0.05)
    for a0 in (0.2, 1.5):
        om = float(M.omega_from_a0(a0, mat))
        A, b = R.build_lse_harela(mat, om)
        Ao, bo = P.assemble_harela(mat, om)
        assert rel(A, Ao) < 1e-11, (a0, rel(A, Ao))
        assert rel(b, bo) < 1e-11
        st = R.stats()
        assert (st["pairs_regular"], st["pairs_adaptive"], st["pairs_singular"]) == tuple(P.stats[:3])
    R.close()


def test_assembly_is_deterministic():
    d = M.slab(4, 1)
    R = BemRegion(d)
    mat = M.viscoelastic(1.0, 0.3, 1.0, 0.05)
    A1, b1 = R.build_lse_harela(mat, 0.7)
    A2, b2 = R.build_lse_harela(mat, 0.7)
    assert np.array_equal(A1, A2) and np.array_equal(b1, b2)
    R.close()


@pytest.mark.parametrize("cplx", [False, True])
def test_solve_lse_lapack_semantics(cplx):
    """mfbem_solve_{r,c}: A overwritten by getrf's LU, 1-based ipiv, b by x;
    factorize=0 reuses the factors."""
    import scipy.linalg as sl
    rng = np.random.default_rng(3)
    n = 300
    A = rng.standard_normal((n, n)) + (1j * rng.standard_normal((n, n)) if cplx else 0)
    A = np.asfortranarray(A)
    b = np.asfortranarray(rng.standard_normal((n, 2)) + (1j * rng.standard_normal((n, 2)) if cplx else 0))
    lu, piv = sl.lu_factor(A)
    xr = sl.lu_solve((lu, piv), b)
    A1, b1 = A.copy(order="F"), b.copy(order="F")
    _, ipiv = solve_lse(A1, b1)
    assert np.array_equal(ipiv - 1, piv)
    assert rel(A1, lu) < 1e-12
    assert rel(b1, xr) < 1e-11
    b2 = b.copy(order="F")
    solve_lse(A1, b2, ipiv=ipiv, factorize=False)
    assert rel(b2, xr) < 1e-11


def test_solve_lse_singular_matrix_reports_info():
    n = 64
    A = np.asfortranarray(np.eye(n))
    A[:, 10] = 0.0
    b = np.ones((n, 1), order="F")
    with pytest.raises(MfbemError) as e:
        solve_lse(A, b)
    assert e.value.code == 11


def test_kat_confined_cube_on_gpu():
    """docs/examples/ME-ST-EL-002 closed form through the device path."""
    d = M.cube_confined_kat(2)
    R = BemRegion(d, qsi_relative_error=1e-10)
    mat = M.elastic(1.0, 0.25)
    x = R.solve_staela(mat["mu"], mat["nu"])
    u, _ = R.solution(x)
    assert np.abs(u[:, 0] - (1.25 * 0.5 / 0.75) * d.nodes[:, 0]).max() < 2e-9
    assert np.abs(u[:, 1:]).max() < 2e-9
    R.close()


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_kat_harmonic_p_wave_column_on_gpu(oracle, precision):
    """docs/examples/ME-TH-EL-001 through the device sweep: the closed form to
    the discretisation error of 4x4 quad8 per face, and the oracle's solution
    of the same mesh to the parity tolerance."""
    from test_oracle_kat import _p_wave_column
    d = M.cube_confined_kat(4)
    mat = M.viscoelastic(2.4, 0.2, 1.0, 0.02)
    om = np.array([1.0, 2.0, 5.0])
    R = BemRegion(d)
    X = R.sweep_harela(mat, om, precision=precision)
    P = oracle.Problem(d)
    for i, w in enumerate(om):
        u, _ = R.solution(X[i])
        ue = _p_wave_column(mat, w, d.nodes[:, 0])
        assert np.abs(u[:, 0] - ue).max() / np.abs(ue).max() < (3e-3 if w > 3 else 2e-4)
        Ao, bo = P.assemble_harela(mat, w)
        assert rel(X[i], oracle.lu_solve(Ao, bo)) < (1e-10 if precision == "plain" else 1e-8)
    R.close()


@pytest.mark.parametrize("precision,tol", [("plain", 1e-10), ("mixed", 1e-8)])
def test_sweep_matches_oracle_solution(oracle, precision, tol):
    d = M.cube_clamped_top_traction(4)
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    om = M.omega_from_a0(np.linspace(0.1, 2.0, 5), mat)
    R = BemRegion(d)
    P = oracle.Problem(d)
    X = R.sweep_harela(mat, om, precision=precision)
    for i, w in enumerate(om):
        Ao, bo = P.assemble_harela(mat, w)
        xo = oracle.lu_solve(Ao, bo)
        assert rel(X[i], xo) < tol, (precision, i, rel(X[i], xo))
    if precision == "mixed":
        assert R.last_stats["max_backward_error"] <= 1e-12
    R.close()


@pytest.mark.parametrize("name,mk", [("cube4", lambda: M.cube_clamped_top_traction(4)),
                                     ("footing6", lambda: M.halfspace_footing(1.0, 6, 1.0))],
                         ids=["cube4", "footing6-odd-n"])
def test_static_solve_mixed_matches_plain(name, mk):
    """footing6: 399 unknowns, an odd length for the FP32 work vectors of the
    real mixed path (the doubles after them stay aligned)."""
    d = mk()
    R = BemRegion(d)
    mat = M.elastic(1.0, 0.25)
    xp = R.solve_staela(mat["mu"], mat["nu"], precision="plain")
    xm = R.solve_staela(mat["mu"], mat["nu"], precision="mixed")
    assert rel(xm, xp) < 1e-9
    R.close()


def test_zexp_double_float_matches_fp64():
    """E_2..E_5 of the mixed regular-pair kernel (double-float, own exp/sincos
    with Cody-Waite reduction) against the binary64 path of the plain method."""
    import ctypes
    L = _abi.load()
    L.mfbem_internal_zexp.argtypes = [ctypes.c_int32] + [ctypes.c_void_p] * 3
    rng = np.random.default_rng(7)
    n = 20000
    mag = 10.0 ** rng.uniform(-4, np.log10(30.0), n)
    ang = rng.uniform(-np.pi, np.pi, n)
    z = mag * np.exp(1j * ang)
    z = np.where(z.real < -60, z.imag * 1j - 60, z)
    zz = np.ascontiguousarray(np.stack([z.real, z.imag], 1))
    e64 = np.zeros((n, 4, 2))
    eff = np.zeros((n, 4, 2))
    _abi.check(L.mfbem_internal_zexp(n, zz.ctypes.data, e64.ctypes.data, eff.ctypes.data))
    E = e64[..., 0] + 1j * e64[..., 1]
    F = eff[..., 0] + 1j * eff[..., 1]
    small = np.abs(z) <= 1.0
    # series branch: relative to each E_n
    rs = np.abs(F[small] - E[small]) / np.abs(E[small])
    assert rs.max() < 1e-13, rs.max()
    # exponential branch: E_n = e^z - sum_{k<n} z^k/k!, error relative to the
    # largest term (double-float carries ~2^-48 per operation; the exp/sincos
    # Horner chains and the cancellation against the leading terms stay below
    # 2e-13 of that scale)
    a = np.abs(z[~small])
    scale = np.maximum.reduce([np.exp(z[~small].real), np.ones_like(a), a, a ** 2 / 2, a ** 3 / 6, a ** 4 / 24])
    ra = np.abs(F[~small] - E[~small]).max(1) / scale
    assert ra.max() < 2e-13, (ra.max(), z[~small][ra.argmax()])


@pytest.mark.parametrize("gemm", ["simt", "tf32", "tc3"])
@pytest.mark.parametrize("name,mk", [("cube4", lambda: M.cube_clamped_top_traction(4)), ("slab4", lambda: M.slab(4, 1)),
                                     ("patch8", lambda: M.surface_patch(10.0, 8, 1.0))],
                         ids=["cube4", "slab4", "patch8"])
def test_mixed_sweep_trailing_update_modes(oracle, monkeypatch, gemm, name, mk):
    """Mixed sweep with SIMT FP32, cuBLAS TF32 and this library's tcgen05
    3xTF32 trailing updates: all reach the FP64 oracle solution to 1e-8 (TF32
    factors are refined in FP64 and escalate to SIMT FP32 when refinement
    stalls)."""
    monkeypatch.setenv("MFBEM_FP32_GEMM", gemm)
    d = mk()
    mat = M.viscoelastic(1.0, 0.3, 1.0, 0.05)
    om = M.omega_from_a0([0.3, 1.2], mat)
    R = BemRegion(d)
    P = oracle.Problem(d)
    X = R.sweep_harela(mat, om, precision="mixed")
    for i, w in enumerate(om):
        Ao, bo = P.assemble_harela(mat, w)
        xo = oracle.lu_solve(Ao, bo)
        assert rel(X[i], xo) < 1e-8, (gemm, name, i, rel(X[i], xo))
    assert R.last_stats["max_backward_error"] <= 1e-12
    R.close()


@pytest.mark.parametrize("gemm", ["simt", "tf32"])
@pytest.mark.parametrize("name,mk", [("cube4", lambda: M.cube_clamped_top_traction(4)), ("slab4", lambda: M.slab(4, 1))],
                         ids=["cube4", "slab4"])
def test_mixed_sweep_gmres_refinement(oracle, monkeypatch, gemm, name, mk):
    """GMRES-based refinement (precision 'mixed-gmres'): FP64 GMRES on the
    correction equation, left-preconditioned by the FP32 / TF32 LU factors,
    reaches the FP64 oracle solution to 1e-8."""
    monkeypatch.setenv("MFBEM_FP32_GEMM", gemm)
    d = mk()
    mat = M.viscoelastic(1.0, 0.3, 1.0, 0.05)
    om = M.omega_from_a0([0.3, 1.2], mat)
    R = BemRegion(d)
    P = oracle.Problem(d)
    X = R.sweep_harela(mat, om, precision="mixed-gmres")
    st = R.last_stats
    assert st["gmres_iterations"] > 0 and st["max_backward_error"] <= 1e-12
    for i, w in enumerate(om):
        Ao, bo = P.assemble_harela(mat, w)
        xo = oracle.lu_solve(Ao, bo)
        assert rel(X[i], xo) < 1e-8, (gemm, name, i, rel(X[i], xo))
    R.close()


def test_static_solve_gmres_refinement(oracle):
    d = M.cube_clamped_top_traction(4)
    mat = M.elastic(1.0, 0.25)
    R = BemRegion(d)
    xp = R.solve_staela(mat["mu"], mat["nu"], precision="plain")
    xg = R.solve_staela(mat["mu"], mat["nu"], precision="mixed-gmres")
    assert R.last_stats["gmres_iterations"] > 0
    assert rel(xg, xp) < 1e-10
    R.close()


def test_sweep_batch_of_uneven_meshes(oracle):
    """Sweeps of meshes of different size in one call (concurrent on the GPU)
    agree with each mesh's plain FP64 sweep to max(1e-8, 1e-14 / rcond) (mixed
    precision: double-float pair sums, entries within about 1e-14 of the
    binary64 assembly; the thin slab's 1/rcond reaches 6.7e6), and the cube's
    with the FP64 oracle."""
    from multifebe_gb300 import sweep_harela_batch
    decks = [M.cube_clamped_top_traction(2), M.cube_clamped_top_traction(3), M.slab(3, 1)]
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    oms = [M.omega_from_a0([0.3, 1.1], mat), M.omega_from_a0([0.5], mat), M.omega_from_a0([0.2, 0.9, 1.4], mat)]
    regions = [BemRegion(d) for d in decks]
    X, stats = sweep_harela_batch(regions, mat, oms, precision="mixed")
    for d, r, om, x, st in zip(decks, regions, oms, X, stats):
        xp = r.sweep_harela(mat, om, precision="plain")
        Po = oracle.Problem(d)
        for i in range(len(om)):
            _, rc = oracle.lu_solve(*Po.assemble_harela(mat, om[i]), rcond=True)
            assert rel(x[i], xp[i]) < max(1e-8, 1e-14 / rc), (d.name, i, rel(x[i], xp[i]), 1.0 / rc)
        assert st["max_backward_error"] <= 1e-12
    P = oracle.Problem(decks[1])
    Ao, bo = P.assemble_harela(mat, oms[1][0])
    assert rel(X[1][0], oracle.lu_solve(Ao, bo)) < 1e-8
    for r in regions:
        r.close()


@pytest.mark.parametrize("pivot", ["none", "partial"])
@pytest.mark.parametrize("name,mk", [("cube4", lambda: M.cube_clamped_top_traction(4)), ("slab4", lambda: M.slab(4, 1)),
                                     ("patch8", lambda: M.surface_patch(10.0, 8, 1.0))],
                         ids=["cube4", "slab4", "patch8"])
def test_mixed_sweep_pivoting_modes(oracle, monkeypatch, pivot, name, mk):
    """The mixed path's FP32 factors without row interchanges (the default
    first attempt: no pivot search across CTAs in the panel) and with partial
    pivoting both reach the FP64 oracle solution to 1e-8 after refinement."""
    monkeypatch.setenv("MFBEM_PIVOT", pivot)
    d = mk()
    mat = M.viscoelastic(1.0, 0.3, 1.0, 0.05)
    om = M.omega_from_a0([0.3, 1.2], mat)
    R = BemRegion(d)
    P = oracle.Problem(d)
    X = R.sweep_harela(mat, om, precision="mixed")
    for i, w in enumerate(om):
        Ao, bo = P.assemble_harela(mat, w)
        xo = oracle.lu_solve(Ao, bo)
        assert rel(X[i], xo) < 1e-8, (pivot, name, i, rel(X[i], xo))
    assert R.last_stats["max_backward_error"] <= 1e-12
    R.close()
