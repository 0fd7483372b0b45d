import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libdto.so")


@pytest.fixture(scope="session")
def engine():
    from dual_threshold_optimization_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()


@pytest.fixture
def fresh_engine():
    """A context of its own: no ladders of earlier pairs' shapes, so a new
    pair's first long run measures its ladder from a first batch."""
    from dual_threshold_optimization_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()
