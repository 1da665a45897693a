import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle
