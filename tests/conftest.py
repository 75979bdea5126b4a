import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    """Build (if stale) and load the CUDA library."""
    from pdos_gb300 import build, _lib
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O
    O.build_port()
    return O
