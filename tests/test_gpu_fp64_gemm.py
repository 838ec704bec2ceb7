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


def _mat(rng, m, n, cplx, spread):
    M = rng.standard_normal((m, n)) + (1j * rng.standard_normal((m, n)) if cplx else 0)
    return M * 10.0 ** rng.uniform(-spread, spread, (m, 1)) * 10.0 ** rng.uniform(-spread, spread, (1, n))


@pytest.mark.parametrize("mode", [0, 1], ids=["ozaki", "dfma"])
@pytest.mark.parametrize("cplx", [True, False], ids=["complex", "real"])
@pytest.mark.parametrize("m,n,k", [(300, 200, 128), (129, 97, 32), (64, 500, 256), (257, 130, 300)])
def test_update_matches_extended_precision(mode, cplx, m, n, k):
    rng = np.random.default_rng(m * 7 + n + k)
    A = np.asfortranarray(_mat(rng, m, k, cplx, 2))
    B = np.asfortranarray(_mat(rng, k, n, cplx, 2))
    C = np.asfortranarray(_mat(rng, m, n, cplx, 1))
    e = _err(_run(A, B, C, mode), A, B, C)
    print("mode", mode, "cplx", cplx, (m, n, k), "max err / (|C| + |A||B|)", e)
    # the binary64 SIMT kernel: the classical bound k u of a sequential sum
    assert e <= (BOUND if mode == 0 else k * 2.0 ** -53)


def test_zero_rows_columns_and_wide_exponent_range():
    rng = np.random.default_rng(3)
    m, n, k = 200, 150, 128
    A = np.asfortranarray(_mat(rng, m, k, True, 6))
    B = np.asfortranarray(_mat(rng, k, n, True, 6))
    A[5, :] = 0.0
    A[:, 7] = 0.0
    B[:, 11] = 0.0
    A[17, 3] = 1e-300  # denormal-range products are rounded away against the row scale
    C = np.asfortranarray(_mat(rng, m, n, True, 1))
    Cg = _run(A, B, C, 0)
    assert np.array_equal(Cg[5, :], C[5, :]) and np.array_equal(Cg[:, 11], C[:, 11])
    assert _err(Cg, A, B, C) <= BOUND
