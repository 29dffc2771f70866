import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def built():
    """Build the CUDA library (sm_103a) and the CPU oracle once per session."""
    from parmoon2022_gb300 import build as b
    b.build()
    import pyoracle
    pyoracle.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import parmoon2022_gb300 as pg
    c = pg.Context(0)
    yield c
    c.close()
