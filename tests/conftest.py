import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) and runs the CUDA library")


@pytest.fixture(scope="session")
def tn():
    """The package, with libtennet_cuda.so built in-tree."""
    import __graft_entry__ as g
    g.build()
    return g.load_package()


@pytest.fixture(scope="session")
def ctx(tn):
    return tn.Context(0)
