import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if stale) and loads the CUDA library; GPU tests fail loudly when it cannot load."""
    from solidboolean_gb300 import build as b
    import solidboolean_gb300 as sbg
    b.build()
    return sbg.lib()


@pytest.fixture(scope="session")
def port():
    from oracle import oracle
    return oracle.port()
