import ctypes
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _gpu_count() -> int:
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            continue
    else:
        return 0
    n = ctypes.c_int(0)
    return n.value if rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 else 0


HAVE_GPU = _gpu_count() > 0


@pytest.fixture(scope="session")
def native():
    from arbo_gpu_fit_gb300 import _native
    return _native.load()


@pytest.fixture(scope="session")
def gpu():
    if not HAVE_GPU:
        pytest.skip("no CUDA device")
    from arbo_gpu_fit_gb300 import _native
    return _native.load()
