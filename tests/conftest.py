import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    """The oracle (test infrastructure) is a small C library; build it if absent."""
    lib = os.path.join(ROOT, "oracle", "_build", "libpsf_oracle.so")
    src = os.path.join(ROOT, "oracle", "psf_oracle.c")
    if not os.path.exists(lib) or os.path.getmtime(lib) < os.path.getmtime(src):
        from oracle import build as ob
        ob.build()
    yield
