"""Builds the engine library against the fake CUDA runtime in fake_cudart.cpp (test use only).

The engine source is compiled with the package's nvcc flags, except that the device code is kept
as PTX (nothing runs it here) and the CUDA runtime is not linked (-cudart none): every runtime call
binds to fake_cudart.cpp in the same shared object.
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(HERE, "_build", "libssegpu_fake.so")
SOURCES = [os.path.join(ROOT, "stochasticseriesexpansion.jl_gb300", "csrc", "sse_engine.cu"),
           os.path.join(HERE, "fake_cudart.cpp")]
DEPS = SOURCES + [os.path.join(ROOT, "stochasticseriesexpansion.jl_gb300", "csrc", "sse_device.cuh"),
                  os.path.join(ROOT, "include", "sse_gpu.h")]


def _up_to_date() -> bool:
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in DEPS)


def build() -> str:
    if _up_to_date():
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    import fcntl

    # pytest-xdist workers build at the same time: one builds, the others wait and reuse its library
    with open(LIB + ".lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if not _up_to_date():
            _build_locked()
    return LIB


def _build_locked() -> None:
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "_sse_pkg_build", os.path.join(ROOT, "stochasticseriesexpansion.jl_gb300", "build.py"))
    pkg_build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pkg_build)
    flags = [f.replace("code=sm_103a", "code=compute_103a") for f in pkg_build.NVCC_FLAGS if f != "-lineinfo"]
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")
    cmd = [nvcc, *flags, "-cudart", "none", "-I", os.path.join(ROOT, "include"), "-o", LIB + ".tmp", *SOURCES]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
