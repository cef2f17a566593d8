import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the pfast_gb300 kernels")


@pytest.fixture(scope="session")
def ctx():
    """One pfast_gb300 device context for the GPU tests."""
    import pfast_gb300 as pg
    c = pg.Context(0)
    yield c
    c.close()
