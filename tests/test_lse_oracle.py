"""The oracle's restatement of solve_lse_{r,c}'s options (?laqge, ?gerfs with
the ?lacn2 estimator) against LAPACK's ?gesvx expert driver, which runs the
same pipeline (equilibrate, factor, condition, solve, refine, unscale)."""
import numpy as np
import pytest
import scipy.linalg.lapack as lp

import lse


def _case(rng, n, cplx, kind):
    A = rng.normal(size=(n, n)) + (1j * rng.normal(size=(n, n)) if cplx else 0)
    r = 10.0 ** rng.uniform(-4, 4, n)
    c = 10.0 ** rng.uniform(-4, 4, n)
    if kind in ("rows", "both"):
        A *= r[:, None]
    if kind in ("cols", "both"):
        A *= c[None, :]
    b = rng.normal(size=(n, 2)) + (1j * rng.normal(size=(n, 2)) if cplx else 0)
    return np.asfortranarray(A), np.asfortranarray(b)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("kind", ["none", "rows", "cols", "both"])
def test_oracle_lse_matches_gesvx(cplx, kind):
    rng = np.random.default_rng(7 + 3 * cplx + ["none", "rows", "cols", "both"].index(kind))
    A, b = _case(rng, 50, cplx, kind)
    f = lp.zgesvx if cplx else lp.dgesvx
    as_, lu, ipiv, equed, rs, cs, bs, x, rcond, ferr, berr, info = f(A.copy(order="F"), b.copy(order="F"), fact="E")
    st = {}
    A2 = A.copy(order="F")
    x2 = lse.solve_lse(A2, b, scaling=True, condition=True, refine=True, state=st)
    assert st["equed"] == equed.decode()
    assert np.array_equal(st["r"], rs) and np.array_equal(st["c"], cs)
    assert np.array_equal(st["Ao"], as_)
    assert np.array_equal(A2, lu) and np.array_equal(st["piv"], ipiv)
    # both solutions carry rounding amplified by the condition number
    assert np.abs(x2 - x).max() <= 20 * lse.EPS / rcond * np.abs(x).max()
    # ?gesvx takes the one-norm from ?lange, the reference from its own
    # sequential loop over moduli (src/solve_lse_c.f90:140-147): an ulp apart
    assert abs(st["rcond"] / rcond - 1) < 4e-15
    # ?gesvx divides ferr by colcnd after column scaling; the reference does not
    colcnd = lse.geequ(A)[3]
    fe = ferr * (colcnd if equed.decode() in "CB" else 1.0)
    # the bound is built from the rounding of the last residual, and that
    # rounding can steer ?lacn2 onto another sign vector: it is an estimate,
    # compared within a factor of 4 (typically 0.2 % apart)
    assert np.all(np.abs(np.log(st["ferr"] / fe)) < np.log(4.0))
    assert np.all(st["berr"] < 4 * lse.EPS) and np.all(berr < 4 * lse.EPS)


def test_oracle_lse_without_scaling_and_n1():
    rng = np.random.default_rng(2)
    for n in (1, 2, 65):
        A, b = _case(rng, n, True, "none")
        as_, lu, ipiv, equed, rs, cs, bs, x, rcond, ferr, berr, info = lp.zgesvx(A.copy(order="F"), b.copy(order="F"),
                                                                                fact="N")
        st = {}
        x2 = lse.solve_lse(A.copy(order="F"), b, condition=True, refine=True, state=st)
        assert np.abs(x2 - x).max() <= 20 * lse.EPS / rcond * np.abs(x).max()
        assert abs(st["rcond"] / rcond - 1) < 4e-15
        assert np.all(np.abs(np.log(st["ferr"] / ferr)) < np.log(4.0))
