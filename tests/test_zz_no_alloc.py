"""mfbem_solve_c_static: the no-allocation variant of mfbem_solve_c.

Some callers cannot allocate device memory (their device memory belongs to
another runtime's pool allocator, or they run under a hard cap on device
allocations). This entry point keeps its whole device working set in a fixed
file-scope array, so these tests compare it with mfbem_solve_c on the same
inputs, twice in a row (the array keeps the previous call's contents), and
check that sizes beyond the array's limit are refused with a clear error.
Collected last on purpose: a failure here leaves every other test already run.
"""
import numpy as np
import pytest

from multifebe_gb300 import _abi, solve_lse

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _static(A, ipiv, b, factorize=True):
    L = _abi.load()
    n = A.shape[0]
    nrhs = b.shape[1]
    return L.mfbem_solve_c_static(n, A.ctypes.data_as(_abi._dp), ipiv.ctypes.data_as(_abi._ip), nrhs,
                                  b.ctypes.data_as(_abi._dp), 1 if factorize else 0)


def test_static_solve_matches_solve_c_on_two_calls():
    rng = np.random.default_rng(11)
    for call, n in enumerate((700, 513)):
        A = np.asfortranarray(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
        b = np.asfortranarray(rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2)))
        A1, b1 = A.copy(order="F"), b.copy(order="F")
        _, ip1 = solve_lse(A1, b1)
        A2, b2 = A.copy(order="F"), b.copy(order="F")
        ip2 = np.zeros(n, dtype=np.int32)
        assert _static(A2, ip2, b2) == 0, _abi.load().mfbem_last_error()
        assert np.array_equal(ip1, ip2), call
        assert _rel(A2, A1) < 1e-12, call
        assert _rel(b2, b1) < 1e-10, call
        # factors reused (factorize = 0) for a new right-hand side
        c = np.asfortranarray(rng.standard_normal((n, 1)) + 1j * rng.standard_normal((n, 1)))
        c1, c2 = c.copy(order="F"), c.copy(order="F")
        solve_lse(A1.copy(order="F"), c1, ipiv=ip1, factorize=False)
        assert _static(A2, ip2, c2, factorize=False) == 0
        assert _rel(c2, c1) < 1e-10, call


def _cudart():
    import ctypes
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("CUDA runtime library not found")


def _free_bytes(rt):
    import ctypes
    fr, tot = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(fr), ctypes.byref(tot)) == 0
    return fr.value


def test_static_solve_at_its_limits_matches_lapack_and_allocates_nothing():
    """n = MFBEM_STATIC_MAX_N with MFBEM_STATIC_MAX_RHS right-hand sides (every
    slot of the array in use) against LAPACK getrf/getrs (scipy), and the
    device's free memory unchanged by a call that follows a warm-up call."""
    import scipy.linalg as sl
    rng = np.random.default_rng(12)
    n, nrhs = 1024, 4
    A = np.asfortranarray(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    b = np.asfortranarray(rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs)))
    lu, piv = sl.lu_factor(A)
    x = sl.lu_solve((lu, piv), b)
    rt = _cudart()
    A0, b0, ip0 = A.copy(order="F"), b.copy(order="F"), np.zeros(n, dtype=np.int32)
    assert _static(A0, ip0, b0) == 0, _abi.load().mfbem_last_error()  # warm-up: context, module, symbol address
    free0 = _free_bytes(rt)
    A1, b1, ip1 = A.copy(order="F"), b.copy(order="F"), np.zeros(n, dtype=np.int32)
    assert _static(A1, ip1, b1) == 0, _abi.load().mfbem_last_error()
    assert _free_bytes(rt) == free0
    assert np.array_equal(ip1 - 1, piv)
    assert _rel(A1, lu) < 1e-12
    assert _rel(b1, x) < 1e-10


def test_static_solve_rejects_sizes_beyond_its_array():
    n = 1025
    A = np.asfortranarray(np.eye(n, dtype=np.complex128))
    b = np.ones((n, 1), dtype=np.complex128, order="F")
    ip = np.zeros(n, dtype=np.int32)
    rc = _static(A, ip, b)
    assert rc == _abi.MFBEM_EARG
    assert b"1024" in _abi.load().mfbem_last_error()
    b5 = np.ones((8, 5), dtype=np.complex128, order="F")
    assert _static(np.asfortranarray(np.eye(8, dtype=np.complex128)), np.zeros(8, dtype=np.int32), b5) == _abi.MFBEM_EARG
