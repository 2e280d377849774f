import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def built():
    """Build the CUDA library and the oracle once per session."""
    from pathfinder_gb300 import build as pbuild
    import oracle
    pbuild.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def renderer(built):
    import pathfinder_gb300 as pf
    r = pf.Renderer(0)
    yield r
    r.close()
