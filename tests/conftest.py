import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# sources of the reference (MultiFEBE) for the tests that read its tutorial
# files; those tests are skipped when the variable is unset
REFERENCE = os.environ.get("MULTIFEBE_REFERENCE_DIR", "")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


_GPU = None


def have_gpu():
    """CUDA device present (checked through the CUDA runtime, no torch import)."""
    global _GPU
    if _GPU is None:
        import ctypes
        _GPU = False
        for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
            try:
                rt = ctypes.CDLL(name)
                n = ctypes.c_int(0)
                _GPU = rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
                break
            except OSError:
                continue
    return _GPU


def pytest_collection_modifyitems(config, items):
    if have_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def reference_dir():
    if not REFERENCE or not os.path.isdir(REFERENCE):
        pytest.skip("reference sources not present (set MULTIFEBE_REFERENCE_DIR)")
    return REFERENCE
