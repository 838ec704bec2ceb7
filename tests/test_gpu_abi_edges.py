"""Edge cases of the C-ABI: the builders add into A and b as the reference's
do (src/build_lse_mechanics_static.f90:52-53 zeroes them once per system,
each region adds), MFBEM_OVERWRITE, a leading dimension larger than n,
device pointers, one-frequency sweeps, invalid arguments and meshes the
path does not cover."""
import ctypes

import numpy as np
import pytest

from multifebe_gb300 import BemRegion, MfbemError, meshgen as M, _abi

pytestmark = pytest.mark.gpu


def _harela_args(mat):
    lam = np.array([complex(mat["lambda"]).real, complex(mat["lambda"]).imag])
    mu = np.array([complex(mat["mu"]).real, complex(mat["mu"]).imag])
    nu = np.array([complex(mat["nu"]).real, complex(mat["nu"]).imag])
    return lam, mu, nu


def test_builders_accumulate_overwrite_and_lda():
    d = M.cube_clamped_top_traction(3)
    R = BemRegion(d)
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    om = 0.9
    A0, b0 = R.build_lse_harela(mat, om)
    A1, b1 = R.build_lse_harela(mat, om, A=A0.copy(order="F"), b=b0.copy())
    # each contribution is added to the entry in place: A0 + sum c rounds
    # differently from 2 sum c, so the added part equals A0 to rounding
    assert np.abs(A1 - 2 * A0).max() <= 1e-14 * np.abs(A0).max()
    assert np.abs(b1 - 2 * b0).max() <= 1e-14 * np.abs(b0).max()
    L = _abi.load()
    lam, mu, nu = _harela_args(mat)
    p = _abi._dp
    rc = L.mfbem_assemble_harela(R._h, lam.ctypes.data_as(p), mu.ctypes.data_as(p), float(mat["rho"]),
                                 nu.ctypes.data_as(p), om, A1.ctypes.data_as(p), R.n, b1.ctypes.data_as(p),
                                 _abi.MFBEM_OVERWRITE)
    assert rc == 0 and np.array_equal(A1, A0) and np.array_equal(b1, b0)
    # lda > n: the padding rows stay untouched
    n, lda = R.n, R.n + 5
    Ap = np.full((lda, n), 7.0 + 1j, dtype=np.complex128, order="F")
    Ap[:n, :] = 0.0
    bp = np.zeros(n, dtype=np.complex128)
    rc = L.mfbem_assemble_harela(R._h, lam.ctypes.data_as(p), mu.ctypes.data_as(p), float(mat["rho"]),
                                 nu.ctypes.data_as(p), om, Ap.ctypes.data_as(p), lda, bp.ctypes.data_as(p), 0)
    assert rc == 0 and np.array_equal(Ap[:n], A0) and np.all(Ap[n:] == 7.0 + 1j)
    # lda < n is refused
    rc = L.mfbem_assemble_harela(R._h, lam.ctypes.data_as(p), mu.ctypes.data_as(p), float(mat["rho"]),
                                 nu.ctypes.data_as(p), om, Ap.ctypes.data_as(p), n - 1, bp.ctypes.data_as(p), 0)
    assert rc == _abi.MFBEM_EARG
    # static builder, same semantics
    S0, c0 = R.build_lse_staela(0.4, 0.25)
    S1, c1 = R.build_lse_staela(0.4, 0.25, A=S0.copy(order="F"), b=c0.copy())
    assert np.abs(S1 - 2 * S0).max() <= 1e-14 * np.abs(S0).max()
    assert np.abs(c1 - 2 * c0).max() <= 1e-14 * np.abs(c0).max()
    R.close()


def test_device_pointers():
    torch = pytest.importorskip("torch")
    d = M.cube_clamped_top_traction(3)
    R = BemRegion(d)
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    A0, b0 = R.build_lse_harela(mat, 1.3)
    n = R.n
    At = torch.full((n * n,), 3.0 + 0j, dtype=torch.complex128, device="cuda")
    bt = torch.zeros(n, dtype=torch.complex128, device="cuda")
    lam, mu, nu = _harela_args(mat)
    p = _abi._dp
    L = _abi.load()
    rc = L.mfbem_assemble_harela(R._h, lam.ctypes.data_as(p), mu.ctypes.data_as(p), float(mat["rho"]),
                                 nu.ctypes.data_as(p), 1.3, ctypes.cast(At.data_ptr(), p), n,
                                 ctypes.cast(bt.data_ptr(), p), _abi.MFBEM_DEVICE_PTRS | _abi.MFBEM_OVERWRITE)
    assert rc == 0
    torch.cuda.synchronize()
    Ad = At.cpu().numpy().reshape(n, n).T  # column-major
    assert np.array_equal(Ad, A0) and np.array_equal(bt.cpu().numpy(), b0)
    R.close()


def test_one_frequency_sweep_matches_the_multi_frequency_sweep():
    d = M.cube_clamped_top_traction(4)
    R = BemRegion(d)
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    om = M.omega_from_a0(np.linspace(0.1, 2.0, 6), mat)
    # plain: the same FP64 factorisation either way; mixed: each run's FP32
    # factors (blocked per batch size) differ, and the refinement stops once
    # the estimated forward error is below 1e-10
    for prec, tol in (("plain", 1e-11), ("mixed", 1e-9)):
        X = R.sweep_harela(mat, om, precision=prec)
        x3 = R.sweep_harela(mat, om[3:4], precision=prec)
        assert np.abs(x3[0] - X[3]).max() / np.abs(X[3]).max() < tol
    R.close()


def test_sweep_argument_errors():
    d = M.cube_clamped_top_traction(2)
    R = BemRegion(d)
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    L = _abi.load()
    lam, mu, nu = _harela_args(mat)
    p = _abi._dp
    om = np.array([0.5])
    X = np.zeros((1, R.n), dtype=np.complex128)
    st = _abi.Stats()
    args = lambda nf, prec: (R._h, lam.ctypes.data_as(p), mu.ctypes.data_as(p), float(mat["rho"]),
                             nu.ctypes.data_as(p), nf, om.ctypes.data_as(p), prec, 1e-12, X.ctypes.data_as(p), 0,
                             ctypes.byref(st))
    assert L.mfbem_sweep_harela(*args(0, 1)) == _abi.MFBEM_EARG
    assert L.mfbem_sweep_harela(*args(1, 3)) == _abi.MFBEM_EARG
    assert L.mfbem_sweep_harela(*args(1, 1)) == 0
    R.close()


def test_upload_rejects_meshes_outside_the_path():
    d = M.cube_clamped_top_traction(2)
    d.ctype[0, 0] = 2  # neither u nor t prescribed: not an ordinary BE boundary condition
    with pytest.raises(MfbemError) as e:
        BemRegion(d)
    assert e.value.code in (_abi.MFBEM_EUNSUPPORTED, _abi.MFBEM_EARG)


def test_released_device_memory_is_reused_safely():
    """Upload, sweep and release, mesh after mesh of different sizes: the
    buffers, streams and cuBLAS handles cached from released meshes give the
    solutions of the first, freshly allocated, handle (a reused buffer with
    stale contents would show as a large error); trimming the cache
    returns 0 and a later upload still works."""
    L = _abi.load()
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    first = {}
    for rep in range(2):
        for n in (3, 4, 3):
            d = M.cube_clamped_top_traction(n)
            R = BemRegion(d)
            om = M.omega_from_a0(np.linspace(0.2, 1.6, 4), mat)
            X = R.sweep_harela(mat, om, precision="mixed")
            R.close()
            if n not in first:
                first[n] = X
            else:
                assert np.abs(X - first[n]).max() <= 1e-12 * np.abs(first[n]).max()
    assert L.mfbem_trim_device_cache() == 0
    R = BemRegion(M.cube_clamped_top_traction(3))
    X = R.sweep_harela(mat, M.omega_from_a0(np.linspace(0.2, 1.6, 4), mat), precision="mixed")
    R.close()
    assert np.abs(X - first[3]).max() <= 1e-12 * np.abs(first[3]).max()
