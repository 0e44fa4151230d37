import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GPU host)")


@pytest.fixture(scope="session", autouse=True)
def native_builds():
    """Build the oracle and the package's native libraries once per session (incremental)."""
    import oracle
    from sarsolver_gb300 import build

    oracle.build()
    build.build()
    yield
