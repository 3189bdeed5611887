import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib_built():
    """Builds libmprgp_gb300.so (nvcc cross-compiles; no GPU needed)."""
    import mprgp_gb300
    return mprgp_gb300.build()


@pytest.fixture(scope="session")
def ctx(lib_built):
    import mprgp_gb300 as M
    c = M.Context(0)
    yield c
    c.close()
