import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import _sse_loader  # noqa: E402

_sse_loader.load()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")
    config.addinivalue_line("markers", "slow: long statistical run")


@pytest.fixture(scope="session")
def S():
    return _sse_loader.load()


@pytest.fixture(scope="session")
def O():
    from oracle import oracle

    oracle.lib()
    return oracle
