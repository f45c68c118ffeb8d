import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def orc():
    """The oracle (CPU restatement of the reference + FP64 kernel twins)."""
    from oracle import loader
    return loader.load()


@pytest.fixture(scope="session")
def pcf_lib():
    """libpcf.so, built in-tree."""
    from parcompfin_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def ctx(pcf_lib):
    from parcompfin_gb300 import Context
    c = Context(0)
    yield c
    c.close()
