import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the product library and the oracle once per session."""
    from yune_gb300 import build as ybuild
    ybuild.build()
    from oracle import build_oracle
    build_oracle.build_oracle()
    yield


def have_gpu():
    try:
        import ctypes
        cudart = ctypes.CDLL("libcudart.so")
        n = ctypes.c_int()
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False
