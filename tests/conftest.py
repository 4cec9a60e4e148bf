import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Make sure the in-tree library and the oracle are built and current."""
    from svl_gb300 import _build
    _build.build_all()
    yield


def gpu_available():
    try:
        from svl_gb300 import _capi as capi
        import ctypes as C
        n = C.c_int()
        return capi.lib().svl_device_info(C.byref(n), None, None, None) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not gpu_available():
        pytest.fail("GPU test requested but no CUDA device / library is usable")
    return True
