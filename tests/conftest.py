import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build as ob
    from oracle import pyoracle

    ob.build()
    return pyoracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library; GPU tests fail (not skip) when it is missing."""
    from asend3d_gb300 import _lib
    from asend3d_gb300 import build as lb

    lb.build()
    return _lib.load()
