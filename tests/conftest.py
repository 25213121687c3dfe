import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN


@pytest.fixture(scope="session")
def native_lib():
    """The native library for host-only calls (no device needed); built if stale."""
    from ctwin_gb300 import build as _build
    _build.build()
    from ctwin_gb300._native import lib
    return lib()


@pytest.fixture(scope="session")
def native():
    """The native library; GPU tests require it to be built and a device present."""
    from ctwin_gb300 import build as _build  # noqa: F401
    from ctwin_gb300._native import lib
    L = lib()
    if L.ctw_device_count() == 0:
        pytest.fail("no CUDA device visible to libctwin_gb300 (GPU test run without a GPU)")
    return L
