"""Builds ``libssegpu.so`` in-tree with nvcc for sm_103a.

The library is the product: there is no CPU fallback, and loading fails
loudly when it has not been built.
"""

from __future__ import annotations

import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libssegpu.so")
SOURCES = ["sse_engine.cu"]
HEADERS = ["sse_device.cuh"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo",
    "-O3",
    "-std=c++17",
    # accept/reject and controller arithmetic must not be contracted into FMAs.  The flag governs
    # floating-point contraction only (integer and address arithmetic still use fused multiply-adds);
    # a -fmad=true build gave bit-identical chains at the same speed, so it stays as a guard for
    # FP64 code written without the explicit *_rn intrinsics
    "-fmad=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off",
    "-shared",
]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(ROOT, "include", "sse_gpu.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")
    cmd = [nvcc, *NVCC_FLAGS, "-I", os.path.join(ROOT, "include"), "-o", LIB + ".tmp"]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    cmd += [os.path.join(CSRC, s) for s in SOURCES]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
