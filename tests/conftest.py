import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


def golden(name):
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, name)))


@pytest.fixture(scope="session")
def lib_built():
    """Build libsapporo.so / libg6drive.so and the oracle port once."""
    from amuse_gb300 import build
    build.build()
    import oracle
    oracle.build_port()
    return True


@pytest.fixture(scope="session")
def g6(lib_built):
    """One opened library context for the whole GPU session."""
    import amuse_gb300 as ag
    ctx = ag.G6X(0)
    yield ctx
