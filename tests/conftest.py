import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def native_lib():
    """The in-tree native library; built on demand (no GPU needed to build)."""
    from uhm_gb300 import build
    build.build()
    from uhm_gb300 import api
    return api.lib()
