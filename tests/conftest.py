import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: longer statistical test")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """The oracle and the native library are built once per session (the
    native build cross-compiles without a GPU)."""
    subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle"), "-s"])
    from iss_gb300 import build
    build.build()
    yield


def gpu_available() -> bool:
    try:
        from iss_gb300 import native
        import ctypes
        n = ctypes.c_int(0)
        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return os.path.exists("/dev/nvidia0")
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0 and native is not None
    except Exception:
        return False
