"""The tcgen05 3xTF32 complex GEMM update (C -= A B) of the mixed LU against a
float64 reference computed from the same float32 inputs."""
import ctypes

import numpy as np
import pytest

from multifebe_gb300 import _abi

pytestmark = pytest.mark.gpu


def _tc(C, A, B, staged=0):
    L = _abi.load()
    L.mfbem_internal_tc_cgemm.argtypes = [ctypes.c_int32] * 3 + [ctypes.c_void_p] * 3 + [ctypes.c_int32]
    m, k = A.shape
    n = B.shape[1]
    Af = np.asfortranarray(A, dtype=np.complex64)
    Bf = np.asfortranarray(B, dtype=np.complex64)
    Cf = np.asfortranarray(C, dtype=np.complex64).copy(order="F")
    _abi.check(L.mfbem_internal_tc_cgemm(m, n, k, Af.ctypes.data, Bf.ctypes.data, Cf.ctypes.data, staged))
    return Cf


@pytest.mark.parametrize("staged", [0, 1], ids=["bulk", "staged"])
@pytest.mark.parametrize("m,n,k", [(64, 128, 16), (100, 70, 40), (300, 260, 128), (513, 129, 33), (64, 16, 1),
                                   (257, 600, 70)])
def test_tc_cgemm_matches_fp64_reference(m, n, k, staged):
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    A = (rng.normal(size=(m, k)) + 1j * rng.normal(size=(m, k))).astype(np.complex64)
    B = (rng.normal(size=(k, n)) + 1j * rng.normal(size=(k, n))).astype(np.complex64)
    C = (rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))).astype(np.complex64)
    got = _tc(C, A, B, staged).astype(np.complex128)
    ref = C.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    scale = (np.abs(A.astype(np.complex128)) @ np.abs(B.astype(np.complex128))).max() + np.abs(C).max()
    err = np.abs(got - ref).max() / scale
    # 3xTF32: about FP32 accuracy (a single TF32 pass would give ~1e-3)
    assert err < 2e-6, err
