"""Failure detection of the bounded device waits, without a GPU fault.

Every spin-wait of the library's kernels (the tcgen05 pipeline's mbarrier
waits, the cooperative LU panel's inter-CTA barrier) has an iteration limit,
after which the kernel sets an error flag, drains its own copies and MMAs
(with the full limit), frees its TMEM and returns; the host turns the flag
into MFBEM_ETIMEOUT. The test hook mfbem_internal_set_spin_limit lowers the
limit to a few iterations, so the waits give up while the work they wait for
is still running (it completes normally). Each test checks the status, then
restores the limit and checks that the next call on the same context is
correct, i.e. no TMEM or other state was left behind.
"""
import ctypes

import numpy as np
import pytest
import scipy.linalg as sl

from multifebe_gb300 import _abi, meshgen as M, BemRegion, solve_lse, MfbemError

pytestmark = pytest.mark.gpu


def _lib():
    L = _abi.load()
    L.mfbem_internal_set_spin_limit.argtypes = [ctypes.c_int64]
    L.mfbem_internal_tc_cgemm.argtypes = [ctypes.c_int32] * 3 + [ctypes.c_void_p] * 3 + [ctypes.c_int32]
    return L


@pytest.fixture
def short_waits():
    L = _lib()
    yield L
    L.mfbem_internal_set_spin_limit(0)


def _tc(L, A, B, C, staged):
    m, k = A.shape
    n = B.shape[1]
    return L.mfbem_internal_tc_cgemm(m, n, k, A.ctypes.data, B.ctypes.data, C.ctypes.data, staged)


@pytest.mark.parametrize("staged", [0, 1])
def test_tensor_core_wait_gives_up_then_next_call_is_correct(short_waits, staged):
    L = short_waits
    rng = np.random.default_rng(5)
    m, n, k = 512, 384, 96
    A = np.asfortranarray((rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))).astype(np.complex64))
    B = np.asfortranarray((rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))).astype(np.complex64))
    C0 = np.asfortranarray((rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))).astype(np.complex64))
    L.mfbem_internal_set_spin_limit(1)
    C = C0.copy(order="F")
    assert _tc(L, A, B, C, staged) == _abi.MFBEM_ETIMEOUT
    assert b"timed out" in L.mfbem_last_error()
    L.mfbem_internal_set_spin_limit(0)
    for _ in range(2):
        C = C0.copy(order="F")
        assert _tc(L, A, B, C, staged) == 0, L.mfbem_last_error()
        ref = C0.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
        assert np.abs(C - ref).max() / np.abs(ref).max() < 2e-6


def test_fp64_tensor_core_wait_gives_up_then_next_call_is_correct(short_waits):
    """The Ozaki-scheme kernels of the plain LU's trailing update."""
    L = short_waits
    L.mfbem_internal_f64_gemm.argtypes = [ctypes.c_int32] * 4 + [ctypes.c_void_p] * 3 + [ctypes.c_int32]
    rng = np.random.default_rng(6)
    m, n, k = 300, 200, 128
    A = np.asfortranarray(rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k)))
    B = np.asfortranarray(rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n)))
    C0 = np.asfortranarray(rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n)))
    L.mfbem_internal_set_spin_limit(1)
    C = C0.copy(order="F")
    assert L.mfbem_internal_f64_gemm(1, m, n, k, A.ctypes.data, B.ctypes.data, C.ctypes.data, 0) == _abi.MFBEM_ETIMEOUT
    L.mfbem_internal_set_spin_limit(0)
    for _ in range(2):
        C = C0.copy(order="F")
        assert L.mfbem_internal_f64_gemm(1, m, n, k, A.ctypes.data, B.ctypes.data, C.ctypes.data, 0) == 0
        ref = C0 - A @ B
        assert np.abs(C - ref).max() / np.abs(ref).max() < 1e-14


def test_cooperative_panel_barrier_gives_up_then_next_solve_is_correct(short_waits):
    """n = 3300 complex: the FP64 LU's panel runs as a cooperative grid of
    several CTAs per matrix (its rows exceed the cluster panel's shared memory)."""
    L = short_waits
    rng = np.random.default_rng(8)
    n = 3300
    A = np.asfortranarray(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    b = np.asfortranarray(rng.standard_normal((n, 1)) + 1j * rng.standard_normal((n, 1)))
    L.mfbem_internal_set_spin_limit(1)
    with pytest.raises(MfbemError) as e:
        solve_lse(A.copy(order="F"), b.copy(order="F"))
    assert e.value.code == _abi.MFBEM_ETIMEOUT
    L.mfbem_internal_set_spin_limit(0)
    lu, piv = sl.lu_factor(A)
    x = sl.lu_solve((lu, piv), b)
    A1, b1 = A.copy(order="F"), b.copy(order="F")
    _, ipiv = solve_lse(A1, b1)
    assert np.array_equal(ipiv - 1, piv)
    assert np.abs(b1 - x).max() / np.abs(x).max() < 1e-10


def test_mixed_sweep_reports_the_timeout_then_recovers(short_waits, oracle):
    L = short_waits
    d = M.cube_clamped_top_traction(4)
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    om = M.omega_from_a0([0.5, 1.5], mat)
    R = BemRegion(d)
    R.sweep_harela(mat, om, precision="mixed")  # autotuner and kernels loaded at the normal limit
    L.mfbem_internal_set_spin_limit(1)
    with pytest.raises(MfbemError) as e:
        R.sweep_harela(mat, om, precision="mixed")
    assert e.value.code == _abi.MFBEM_ETIMEOUT
    L.mfbem_internal_set_spin_limit(0)
    X = R.sweep_harela(mat, om, precision="mixed")
    P = oracle.Problem(d)
    for i, w in enumerate(om):
        Ao, bo = P.assemble_harela(mat, float(w))
        xo = oracle.lu_solve(Ao, bo)
        assert np.abs(X[i] - xo).max() / np.abs(xo).max() < 1e-8
    R.close()
