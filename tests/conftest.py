import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the native library and the CPU oracle once per session."""
    from rank_structured_cholesky_gb300 import _build
    _build.build_library()
    _build.build_oracle()
    yield
