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


@pytest.fixture(scope="session")
def fake():
    """The engine library built against the fake CUDA runtime of tests/fake_cuda (no GPU needed),
    with its test hooks declared."""
    import ctypes as C
    import shutil

    if shutil.which("nvcc") is None:
        pytest.skip("nvcc unavailable")
    sys.path.insert(0, os.path.join(ROOT, "tests", "fake_cuda"))
    try:
        import build as fake_build
    finally:
        sys.path.pop(0)
    from sse_gb300.engine import load_library

    L = load_library(fake_build.build())
    for name in ("fake_cuda_live_allocs", "fake_cuda_allocs", "fake_cuda_bad_frees", "fake_cuda_launches"):
        getattr(L, name).restype = C.c_long
    L.fake_cuda_fail_alloc_in.argtypes = [C.c_long]
    return L
