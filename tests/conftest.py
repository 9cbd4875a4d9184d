import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the CPU oracle and the engine library once per session (both
    are quick and skip when up to date)."""
    from oracle_lib import build_oracle
    build_oracle()
    from sphfluidsimulation_gb300 import build
    build.build()
    yield


def gpu_available() -> bool:
    try:
        import ctypes
        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return False
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False
