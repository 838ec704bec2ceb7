"""Oracle of solve_lse_r / solve_lse_c with every option (test infrastructure only).

src/solve_lse_r.f90:25-232 and src/solve_lse_c.f90:25-219 run, in order:
?geequ + ?laqge (lse_scaling), ?getrf, ?gecon (lse_condition), ?getrs,
?gerfs (lse_refine) and the unscaling of x. ?geequ, ?getrf, ?getrs and ?gecon
are LAPACK's own, called through scipy. ?laqge and ?gerfs (with the ?lacn2
one-norm estimator, Higham's refinement of Hager's method) are not exported by
scipy; they are restated here from LAPACK's published algorithms and pinned
against scipy's ?gesvx expert driver, which runs the same pipeline
(tests/test_lse_oracle.py).

Only tests/ import this module.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sl
import scipy.linalg.lapack as lp

SAFMIN = lp.dlamch("S")          # DLAMCH('Safe minimum')
PREC = lp.dlamch("P")            # DLAMCH('Precision') = eps * base
EPS = lp.dlamch("E")             # DLAMCH('Epsilon')
THRESH = 0.1                     # ?laqge


def _abs1(a):
    """|re| + |im| for complex (LAPACK's CABS1), |a| for real."""
    return np.abs(a.real) + np.abs(a.imag) if np.iscomplexobj(a) else np.abs(a)


def geequ(A):
    """?geequ: (r, c, rowcnd, colcnd, amax, info), LAPACK's own."""
    f = lp.zgeequ if np.iscomplexobj(A) else lp.dgeequ
    r, c, rowcnd, colcnd, amax, info = f(A)
    return r, c, rowcnd, colcnd, amax, info


def laqge(A, r, c, rowcnd, colcnd, amax):
    """?laqge: equilibrate A in place with r and/or c; returns equed."""
    small = SAFMIN / PREC
    large = 1.0 / small
    if rowcnd >= THRESH and small <= amax <= large:
        if colcnd >= THRESH:
            return "N"
        A *= c[None, :]
        return "C"
    if colcnd >= THRESH:
        A *= r[:, None]
        return "R"
    A *= c[None, :] * r[:, None]   # (c_j * r_i) * a_ij, the order of ?laqge
    return "B"


def lacn2(n, apply, cplx):
    """?lacn2 with the reverse communication unrolled: apply(kase, x) returns
    A x (kase 1) or A^H x (kase 2). Returns the estimate of ||A||_1."""
    dt = np.complex128 if cplx else np.float64
    absv = np.abs
    x = apply(1, np.full(n, 1.0 / n, dtype=dt))
    if n == 1:
        return float(absv(x[0]))
    est = float(absv(x).sum())
    if cplx:
        ax = absv(x)
        x = np.where(ax > SAFMIN, x / np.where(ax > SAFMIN, ax, 1.0), 1.0 + 0j)
    else:
        x = np.where(x >= 0, 1.0, -1.0)
        isgn = x.copy()
    x = apply(2, x)
    j = int(np.argmax(absv(x)))
    it = 2
    while True:
        e = np.zeros(n, dtype=dt)
        e[j] = 1.0
        x = apply(1, e)
        estold, est = est, float(absv(x).sum())
        if not cplx:
            s = np.where(x >= 0, 1.0, -1.0)
            if np.array_equal(s, isgn):
                break
        if est <= estold:
            break
        if cplx:
            ax = absv(x)
            x = np.where(ax > SAFMIN, x / np.where(ax > SAFMIN, ax, 1.0), 1.0 + 0j)
        else:
            x = s
            isgn = s.copy()
        x = apply(2, x)
        jlast, j = j, int(np.argmax(absv(x)))
        xl = absv(x[jlast]) if cplx else x[jlast]
        if xl != absv(x[j]) and it < 5:
            it += 1
            continue
        break
    alt = np.array([(1.0 if i % 2 == 0 else -1.0) * (1.0 + i / (n - 1)) for i in range(n)], dtype=dt)
    x = apply(1, alt)
    temp = 2.0 * (float(absv(x).sum()) / (3 * n))
    return max(est, temp) if temp > est else est


def _getrs(lu, piv, b, conj):
    return sl.lu_solve((lu, piv), b, trans=(2 if np.iscomplexobj(lu) else 1) if conj else 0, check_finite=False)


def gerfs(A, lu, piv, B, X):
    """?gerfs (no transpose): refined X, ferr, berr per right-hand side."""
    n, nrhs = B.shape
    cplx = np.iscomplexobj(A)
    nz = n + 1
    safe1 = nz * SAFMIN
    safe2 = safe1 / EPS
    X = X.copy()
    ferr = np.zeros(nrhs)
    berr = np.zeros(nrhs)
    aA = _abs1(A)
    for j in range(nrhs):
        count, lstres = 1, 3.0
        while True:
            R = B[:, j] - A @ X[:, j]
            W = _abs1(B[:, j]) + aA @ _abs1(X[:, j])
            aR = _abs1(R)
            s = np.where(W > safe2, aR / np.where(W > safe2, W, 1.0), (aR + safe1) / (W + safe1)).max()
            berr[j] = s
            if s > EPS and 2.0 * s <= lstres and count <= 5:
                X[:, j] = X[:, j] + _getrs(lu, piv, R, False)
                lstres = s
                count += 1
                continue
            break
        W = np.where(W > safe2, aR + nz * EPS * W, aR + nz * EPS * W + safe1)

        def apply(kase, x):
            if kase == 1:
                return W * _getrs(lu, piv, x, True)
            return _getrs(lu, piv, W * x, False)

        f = lacn2(n, apply, cplx)
        m = _abs1(X[:, j]).max()
        ferr[j] = f / m if m != 0 else f
    return X, ferr, berr


def gecon_1(lu, anorm):
    """?gecon (one-norm), LAPACK's own."""
    f = lp.zgecon if np.iscomplexobj(lu) else lp.dgecon
    rcond, info = f(lu, anorm, norm="1")
    return rcond


def solve_lse(A, b, factorize=True, scaling=False, condition=False, refine=False, state=None):
    """solve_lse_{r,c}: A (n x n) receives the (scaled) LU factors, returns x.
    state holds the caller-owned arrays of the reference (ipiv, Ao, equed, r,
    c) between calls, and the diagnostics (rcond, ferr, berr)."""
    st = state if state is not None else {}
    b = np.array(b, dtype=A.dtype, copy=True)
    if b.ndim == 1:
        b = b[:, None]
    if factorize:
        if scaling:
            r, c, rowcnd, colcnd, amax, info = geequ(A)
            if info != 0:
                raise ValueError(f"geequ info {info}")
            st["equed"] = laqge(A, r, c, rowcnd, colcnd, amax)
            st["r"], st["c"] = r, c
        if condition or refine:
            st["Ao"] = A.copy()
        lu, piv, info = (lp.zgetrf if np.iscomplexobj(A) else lp.dgetrf)(A)
        if info > 0:
            raise ValueError(f"getrf info {info}")
        A[...] = lu
        st["piv"] = piv
    piv = st["piv"]
    if scaling and st["equed"] in ("R", "B"):
        b *= st["r"][:, None]
    if condition and factorize:
        # column sums of moduli in row order (src/solve_lse_c.f90:140-147)
        anorm = np.cumsum(np.abs(st["Ao"]), axis=0)[-1].max()
        st["rcond"] = gecon_1(A, anorm)
    x = _getrs(A, piv, b, False)
    if refine:
        x, st["ferr"], st["berr"] = gerfs(st["Ao"], A, piv, b, x)
    if scaling and st["equed"] in ("C", "B"):
        x *= st["c"][:, None]
    return x
