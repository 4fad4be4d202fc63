import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build(ref=False)
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The product library, built in-tree; fails (never skips) if it cannot load."""
    from qdeqcycle_fdm_gb300 import build, _lib
    build.build()
    return _lib.load()
