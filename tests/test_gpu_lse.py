"""mfbem_solve_{r,c} with the reference's lse_scaling, lse_condition and
lse_refine (src/solve_lse_r.f90:25-232, src/solve_lse_c.f90:25-219) against
the oracle of oracle/lse.py, itself pinned to LAPACK's ?gesvx.

Tolerances:
  equed, r, c, Ao (the equilibrated matrix), ipiv   identical
  LU factors          <= 1e-12 (max-norm relative)
  x                   <= 20 eps cond(A) (both sides' rounding, amplified)
  rcond               <= 1e-8 relative (the same estimator on factors that
                      differ in the last bits)
  ferr                within a factor of 4 (an estimated bound; rounding of
                      the last residual can steer ?lacn2 differently)
  berr                <= 4 eps
"""
import numpy as np
import pytest

import lse
from multifebe_gb300 import LseState, MfbemError, meshgen as M, BemRegion, solve_lse, _abi

pytestmark = pytest.mark.gpu
KINDS = ["none", "rows", "cols", "both"]


def _case(rng, n, cplx, kind, nrhs=2):
    A = rng.normal(size=(n, n)) + (1j * rng.normal(size=(n, n)) if cplx else 0)
    if kind in ("rows", "both"):
        A *= (10.0 ** rng.uniform(-4, 4, n))[:, None]
    if kind in ("cols", "both"):
        A *= (10.0 ** rng.uniform(-4, 4, n))[None, :]
    b = rng.normal(size=(n, nrhs)) + (1j * rng.normal(size=(n, nrhs)) if cplx else 0)
    return np.asfortranarray(A), np.asfortranarray(b)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("n", [65, 300])
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("cplx", [False, True])
def test_all_options_match_oracle(cplx, kind, n):
    rng = np.random.default_rng(100 + n + 7 * cplx + KINDS.index(kind))
    A, b = _case(rng, n, cplx, kind)
    ost = {}
    Ao_ = A.copy(order="F")
    xo = lse.solve_lse(Ao_, b, scaling=True, condition=True, refine=True, state=ost)
    st = LseState()
    A1, b1 = A.copy(order="F"), b.copy(order="F")
    _, ipiv = solve_lse(A1, b1, scaling=True, condition=True, refine=True, state=st)
    assert st.equed == ost["equed"]
    assert np.array_equal(st.r, ost["r"]) and np.array_equal(st.c, ost["c"])
    assert np.array_equal(st.Ao, ost["Ao"])
    assert np.array_equal(ipiv - 1, ost["piv"])  # scipy returns 0-based pivots
    assert _rel(A1, Ao_) < 1e-12
    assert np.abs(b1 - xo).max() <= 20 * lse.EPS / ost["rcond"] * np.abs(xo).max()
    assert abs(st.rcond / ost["rcond"] - 1) < 1e-8
    assert np.all(np.abs(np.log(st.ferr / ost["ferr"])) < np.log(4.0)), (st.ferr, ost["ferr"])
    assert np.all(st.berr <= 4 * lse.EPS)


@pytest.mark.parametrize("cplx", [False, True])
def test_refactor_free_call_reuses_state(cplx):
    """A second call with factorize = 0 reuses ipiv, equed, r, c and Ao, as
    the sensitivity solves of src/multifebe.f90:94,119 do."""
    rng = np.random.default_rng(5 + cplx)
    A, b = _case(rng, 200, cplx, "both")
    _, b2 = _case(rng, 200, cplx, "none", nrhs=3)
    ost = {}
    Ao_ = A.copy(order="F")
    lse.solve_lse(Ao_, b, scaling=True, refine=True, state=ost)
    xo = lse.solve_lse(Ao_, b2, factorize=False, scaling=True, refine=True, state=ost)
    st = LseState()
    A1 = A.copy(order="F")
    _, ipiv = solve_lse(A1, b.copy(order="F"), scaling=True, refine=True, state=st)
    assert np.isnan(st.rcond)
    x2 = b2.copy(order="F")
    solve_lse(A1, x2, ipiv=ipiv, factorize=False, scaling=True, refine=True, state=st)
    cond = 1.0 / lse.gecon_1(Ao_, np.cumsum(np.abs(ost["Ao"]), axis=0)[-1].max())
    assert np.abs(x2 - xo).max() <= 20 * lse.EPS * cond * np.abs(xo).max()
    assert st.ferr.shape == (3,) and np.all(st.berr <= 4 * lse.EPS)


@pytest.mark.parametrize("n", [1, 2, 64])
def test_condition_and_refine_small(n):
    rng = np.random.default_rng(n)
    A, b = _case(rng, n, True, "none", nrhs=1)
    ost = {}
    xo = lse.solve_lse(A.copy(order="F"), b, condition=True, refine=True, state=ost)
    st = LseState()
    b1 = b.copy(order="F")
    solve_lse(A.copy(order="F"), b1, condition=True, refine=True, state=st)
    assert abs(st.rcond / ost["rcond"] - 1) < 1e-8
    assert np.abs(b1 - xo).max() <= 20 * lse.EPS / ost["rcond"] * np.abs(xo).max()
    assert np.all(np.abs(np.log(st.ferr / ost["ferr"])) < np.log(4.0))


def test_option_errors():
    L = _abi.load()
    n = 8
    A = np.asfortranarray(np.eye(n))
    b = np.ones(n)
    ip = np.zeros(n, dtype=np.int32)
    dp, ipp = _abi._dp, _abi._ip
    # condition / refine need aodim == n (src/solve_lse_r.f90:70-78)
    rc = L.mfbem_solve_r(n, A.ctypes.data_as(dp), ip.ctypes.data_as(ipp), 1, None, None, None, None, 1,
                         b.ctypes.data_as(dp), 1, 0, 1, 0)
    assert rc == _abi.MFBEM_EARG
    # a reused factorisation needs a valid equed
    import ctypes
    r, c = np.ones(n), np.ones(n)
    eq = ctypes.create_string_buffer(b"X", 2)
    rc = L.mfbem_solve_r(n, A.ctypes.data_as(dp), ip.ctypes.data_as(ipp), 1, None, eq, r.ctypes.data_as(dp),
                         c.ctypes.data_as(dp), 1, b.ctypes.data_as(dp), 0, 1, 0, 0)
    assert rc == _abi.MFBEM_EARG
    # ?geequ: a zero row i returns i, a zero column j returns n + j
    A = np.asfortranarray(np.eye(n))
    A[4, :] = 0.0
    with pytest.raises(MfbemError) as e:
        solve_lse(A, np.ones((n, 1), order="F"), scaling=True, state=LseState())
    assert e.value.code == 5
    A = np.asfortranarray(np.eye(n))
    A[:, 6] = 0.0
    A[6, 0] = 1.0  # row 6 keeps a nonzero
    with pytest.raises(MfbemError) as e:
        solve_lse(A, np.ones((n, 1), order="F"), scaling=True, state=LseState())
    assert e.value.code == n + 7


def test_bem_system_with_all_options():
    """The cube's harmonic system: equilibrated, refined solve = plain solve."""
    d = M.cube_clamped_top_traction(4)
    R = BemRegion(d)
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    A, bb = R.build_lse_harela(mat, float(M.omega_from_a0([1.0], mat)[0]))
    R.close()
    A = np.asfortranarray(A)
    b = np.asfortranarray(bb.reshape(-1, 1))
    x0 = b.copy(order="F")
    solve_lse(A.copy(order="F"), x0)
    st = LseState()
    x1 = b.copy(order="F")
    solve_lse(A.copy(order="F"), x1, scaling=True, condition=True, refine=True, state=st)
    assert _rel(x1, x0) < 1e-12
    assert 0 < st.rcond < 1 and st.berr[0] <= 4 * lse.EPS and st.ferr[0] < 1e-10
