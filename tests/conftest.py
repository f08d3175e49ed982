import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the CUDA library and the CPU oracle once per session (in-tree)."""
    from finitevolume_gb300 import build
    build.build_library()
    build.build_oracle()
    yield


@pytest.fixture(scope="session")
def gpu():
    from finitevolume_gb300 import capi
    if capi.lib().fv_device_count() == 0:
        pytest.skip("no CUDA device visible")
    return True
