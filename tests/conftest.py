import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    from oracle import build as ob
    ob.build()
    return O


@pytest.fixture(scope="session")
def world():
    import tiledarray_gb300 as ta
    from tiledarray_gb300 import build as tb
    tb.build()
    w = ta.World(0)
    yield w
    w.close()
