import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    """The CPU restatement of the reference algorithm (the oracle)."""
    from oracle.oracle import Oracle
    o = Oracle("port")
    o.set_globals(1e-18, True, 8)
    return o


@pytest.fixture(scope="session")
def ref():
    """The reference headers compiled in place; only where the reference tree exists."""
    from oracle import oracle as orc
    if not os.path.isdir(os.path.join(orc.REFERENCE_TREE, "src")):
        pytest.skip("reference tree not present")
    o = orc.Oracle("ref")
    o.set_globals(1e-18, True, 8)
    return o
