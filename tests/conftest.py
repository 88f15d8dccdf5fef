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


def _build_script(subdir):
    """tests/<subdir>/build.py, loaded under its own module name (several test libraries have one)."""
    import importlib.util

    path = os.path.join(ROOT, "tests", subdir, "build.py")
    spec = importlib.util.spec_from_file_location(f"_test_build_{subdir}", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def fake():
    """The engine library built against the fake CUDA runtime of tests/fake_cuda (no GPU needed):
    device memory is host memory and kernel launches do nothing.  Its test hooks are declared."""
    import ctypes as C
    import shutil

    if shutil.which("nvcc") is None:
        pytest.skip("nvcc unavailable")
    from sse_gb300.engine import load_library

    L = load_library(_build_script("fake_cuda").build())
    for name in ("fake_cuda_live_allocs", "fake_cuda_allocs", "fake_cuda_bad_frees", "fake_cuda_launches"):
        getattr(L, name).restype = C.c_long
    L.fake_cuda_fail_alloc_in.argtypes = [C.c_long]
    return L


@pytest.fixture(scope="session")
def emu():
    """The engine library whose kernel launches run the engine's own kernels on emulated warps
    (tests/warp_emu), over the fake CUDA runtime (no GPU needed)."""
    import shutil

    if shutil.which("nvcc") is None or shutil.which(os.environ.get("CXX", "g++")) is None:
        pytest.skip("nvcc or g++ unavailable")
    from sse_gb300.engine import load_library

    return load_library(_build_script("warp_emu").build())
