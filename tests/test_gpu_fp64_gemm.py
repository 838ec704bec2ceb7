"""The plain FP64 LU's trailing-update kernels against an exact product.

C -= A B, complex and real, through the test hook mfbem_internal_f64_gemm:
mode 0 the Ozaki-scheme kernels (seven bf16 slices per operand on the tensor
cores, exact integer levels, binary64 recombination), mode 1 the binary64
SIMT kernel. The reference is the same update in extended precision
(numpy longdouble). Bound for the Ozaki kernels: the error of every entry is
at most 2^-50 (|C| + |A||B|), a few units of binary64 rounding of the sum of
magnitudes (measured about 3e-16, against about 1e-16 for a binary64 GEMM;
the classical binary64 bound is k u |A||B|).
"""
import ctypes

import numpy as np
import pytest

from multifebe_gb300 import _abi

pytestmark = pytest.mark.gpu

BOUND = 2.0 ** -50


def _lib():
    L = _abi.load()
    L.mfbem_internal_f64_gemm.argtypes = [ctypes.c_int32] * 4 + [ctypes.c_void_p] * 3 + [ctypes.c_int32]
    return L


def _run(A, B, C, mode):
    L = _lib()
    m, k = A.shape
    n = B.shape[1]
    C = C.copy(order="F")
    rc = L.mfbem_internal_f64_gemm(int(np.iscomplexobj(A)), m, n, k, A.ctypes.data, B.ctypes.data, C.ctypes.data,
                                   mode)
    assert rc == 0, L.mfbem_last_error()
    return C


def _exact(A, B, C):
    ld = np.longdouble
    if np.iscomplexobj(A):
        ar, ai, br, bi = (x.astype(ld) for x in (A.real, A.imag, B.real, B.imag))
        return C.real.astype(ld) - (ar @ br - ai @ bi), C.imag.astype(ld) - (ar @ bi + ai @ br)
    return (C.astype(ld) - A.astype(ld) @ B.astype(ld),)


def _err(Cg, A, B, C):
    ex = _exact(A, B, C)
    got = (Cg.real, Cg.imag) if np.iscomplexobj(Cg) else (Cg,)
    mag = np.abs(C) + np.abs(A) @ np.abs(B)
    return max(float((np.abs(g.astype(np.longdouble) - e) / mag).max()) for g, e in zip(got, ex))


def _mat(rng, m, n, cplx, spread, rows=True, cols=True):
    M = rng.standard_normal((m, n)) + (1j * rng.standard_normal((m, n)) if cplx else 0)
    if rows:
        M = M * 10.0 ** rng.uniform(-spread, spread, (m, 1))
    if cols:
        M = M * 10.0 ** rng.uniform(-spread, spread, (1, n))
    return M


@pytest.mark.parametrize("mode", [0, 1], ids=["ozaki", "dfma"])
@pytest.mark.parametrize("cplx", [True, False], ids=["complex", "real"])
@pytest.mark.parametrize("m,n,k", [(300, 200, 128), (129, 97, 32), (64, 500, 256), (257, 130, 300)])
def test_update_matches_extended_precision(mode, cplx, m, n, k):
    """Rows of A and columns of B with magnitudes spread over 1e-2..1e2 (the
    scales the splitting takes per row and per column)."""
    rng = np.random.default_rng(m * 7 + n + k)
    A = np.asfortranarray(_mat(rng, m, k, cplx, 2, cols=False))
    B = np.asfortranarray(_mat(rng, k, n, cplx, 2, rows=False))
    C = np.asfortranarray(_mat(rng, m, n, cplx, 1))
    e = _err(_run(A, B, C, mode), A, B, C)
    print("mode", mode, "cplx", cplx, (m, n, k), "max err / (|C| + |A||B|)", e)
    # the binary64 SIMT kernel: the classical bound k u of a sequential sum
    assert e <= (BOUND if mode == 0 else k * 2.0 ** -53)


def test_integer_operands_are_exact():
    """Integer operands below 2^15 (K = 256): every partial product lies in the
    exactly accumulated levels, so the update must equal the integer product
    bit for bit. Checks that the tensor cores' FP32 accumulation of the levels
    is exact."""
    rng = np.random.default_rng(9)
    for cplx in (False, True):
        m, n, k = 200, 170, 256 if not cplx else 128
        A = rng.integers(-2 ** 15, 2 ** 15, (m, k)).astype(np.float64)
        B = rng.integers(-2 ** 15, 2 ** 15, (k, n)).astype(np.float64)
        C = rng.integers(-2 ** 20, 2 ** 20, (m, n)).astype(np.float64)
        if cplx:
            A = A + 1j * rng.integers(-2 ** 15, 2 ** 15, (m, k))
            B = B + 1j * rng.integers(-2 ** 15, 2 ** 15, (k, n))
            C = C + 1j * rng.integers(-2 ** 20, 2 ** 20, (m, n))
        A, B, C = (np.asfortranarray(x) for x in (A, B, C))
        exact = C - A @ B  # integers below 2^53: exact in binary64
        got = _run(A, B, C, 0)
        assert np.array_equal(got, exact), (cplx, np.abs(got - exact).max())


def test_zero_rows_columns_and_wide_exponent_range():
    """Entries of a row (column) spread over twelve decades: the splitting
    keeps 2^-55 of each row's (column's) scale, so the bound is normwise over
    the row and column scales: |err| <= 2^-50 (|C| + k max_row|A| max_col|B|)."""
    rng = np.random.default_rng(3)
    m, n, k = 200, 150, 128
    A = np.asfortranarray(_mat(rng, m, k, True, 6))
    B = np.asfortranarray(_mat(rng, k, n, True, 6))
    A[5, :] = 0.0
    A[:, 7] = 0.0
    B[:, 11] = 0.0
    A[17, 3] = 1e-300  # rounded away against its row's scale
    C = np.asfortranarray(_mat(rng, m, n, True, 1))
    Cg = _run(A, B, C, 0)
    assert np.array_equal(Cg[5, :], C[5, :]) and np.array_equal(Cg[:, 11], C[:, 11])
    ex = _exact(A, B, C)
    ra = np.maximum(np.abs(A.real), np.abs(A.imag)).max(axis=1)
    cb = np.maximum(np.abs(B.real), np.abs(B.imag)).max(axis=0)
    bound = 2.0 ** -50 * (np.abs(C) + 2 * k * np.outer(ra, cb))
    for g, e in zip((Cg.real, Cg.imag), ex):
        assert np.all(np.abs(g.astype(np.longdouble) - e) <= bound)
