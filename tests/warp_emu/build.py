"""Builds libssegpu_emu.so (test use only): the engine library with the fake CUDA runtime of
tests/fake_cuda and a host build of the engine's own kernels running on emulated warps.

The kernels are not copied or rewritten by hand.  They are taken from the engine's sources at build
time: sse_device.cuh whole, and the blocks of sse_engine.cu between its "kernels: begin" /
"kernels: end" and "noalloc kernels: begin" / "noalloc kernels: end" markers.  Exactly two textual substitutions are applied, each checked to occur:
 - the PTX read of %lanemask_lt becomes the emulated lane mask;
 - the extern dynamic shared array becomes the emulated block's buffer.
The generated file is compiled with g++ against cuda_emu.h and emu_runtime.cpp.
"""

import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "stochasticseriesexpansion.jl_gb300", "csrc")
FAKE = os.path.join(ROOT, "tests", "fake_cuda")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libssegpu_emu.so")
DEPS = [os.path.join(CSRC, "sse_device.cuh"), os.path.join(CSRC, "sse_engine.cu"), os.path.join(ROOT, "include", "sse_gpu.h"),
        os.path.join(FAKE, "fake_cudart.cpp"), os.path.join(HERE, "cuda_emu.h"), os.path.join(HERE, "emu_runtime.cpp"),
        os.path.abspath(__file__)]

# kernel -> needle in its mangled device name (identifiers are length-prefixed there)
KERNELS = {
    "k_walk<1>": "6k_walkILi1E", "k_walk<0>": "6k_walkILi0E", "k_set_targets": "13k_set_targets",
    "k_apply_growth": "14k_apply_growth", "k_link_debug": "12k_link_debug", "k_gather_status": "15k_gather_status",
    "k_gather_obs": "12k_gather_obs", "k_check": "7k_check", "k_tempering": "11k_tempering",
    "k_noalloc_prep": "14k_noalloc_prep", "k_noalloc_finish": "16k_noalloc_finish",
}


def substitute_once(text, old, new, what):
    n = text.count(old)
    if n != 1:
        raise RuntimeError(f"warp emulator build: expected one {what} in the engine source, found {n}")
    return text.replace(old, new)


def generate() -> str:
    dev = open(os.path.join(CSRC, "sse_device.cuh")).read()
    dev = substitute_once(dev, 'asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));', "r = emu_lanemask_lt();",
                          "%lanemask_lt read")
    dev = dev.replace("#pragma once", "")
    if "asm" in re.sub(r"//.*", "", dev).split():
        raise RuntimeError("warp emulator build: sse_device.cuh has inline PTX the emulator does not handle")
    eng = open(os.path.join(CSRC, "sse_engine.cu")).read()
    begin = eng.index("// ==== kernels: begin")
    end = eng.index("// ==== kernels: end ====")
    block = eng[eng.index("\n", begin) + 1:end]
    nb = eng.index("// ==== noalloc kernels: begin")
    ne = eng.index("// ==== noalloc kernels: end ====")
    block += "\nnamespace {\n" + eng[eng.index("\n", nb) + 1:ne] + "\n}  // namespace\n"
    block, n = re.subn(r"extern __shared__ __align__\(\d+\) uint8_t (\w+)\[\];",
                       r"uint8_t *\1 = static_cast<uint8_t *>(emu_dynamic_smem());", block)
    if n == 0 or "extern __shared__" in block:
        raise RuntimeError("warp emulator build: unexpected dynamic shared memory declarations")
    found = set(re.findall(r"__global__ void (?:__launch_bounds__\([^)]*\) )?(\w+)", block))
    expected = {k.split("<")[0] for k in KERNELS}
    if found != expected:
        raise RuntimeError(f"warp emulator build: kernels {sorted(found)} but dispatch covers {sorted(expected)}")
    entries = " \\\n".join(f'  X("{needle}", {name})' for name, needle in KERNELS.items())
    return (
        "// Generated by tests/warp_emu/build.py from the engine's device sources.  Do not edit.\n"
        "#include <cstring>\n#include <tuple>\n#include <type_traits>\n#include <utility>\n\n"
        '#include "cuda_emu.h"\n#define sse sse_emu\n' + dev + '\n#include "sse_gpu.h"\nusing namespace sse;\n'
        + block + "\n#define EMU_KERNELS(X) \\\n" + entries + "\n"
        '#include "emu_dispatch.inc"\n'
    )


def _up_to_date() -> bool:
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in DEPS + [
        os.path.join(HERE, "emu_dispatch.inc")])


def build() -> str:
    if _up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    import fcntl

    # pytest-xdist workers build at the same time: one builds, the others wait and reuse its library
    with open(os.path.join(BUILD, ".lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if not _up_to_date():
            _build_locked()
    return LIB


def _build_locked() -> None:
    src = os.path.join(BUILD, "emu_kernels.cpp")
    with open(src, "w") as f:
        f.write(generate())
    gxx = os.environ.get("CXX", "g++")
    # IEEE double arithmetic, no contraction into fused multiply-adds: the *_rn intrinsics' rounding
    cflags = ["-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w",
              "-I", HERE, "-I", os.path.join(ROOT, "include")]
    objs = []
    for name, path in (("emu_kernels.o", src), ("emu_runtime.o", os.path.join(HERE, "emu_runtime.cpp"))):
        obj = os.path.join(BUILD, name)
        subprocess.run([gxx, *cflags, "-c", path, "-o", obj], check=True)
        objs.append(obj)
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "_sse_pkg_build", os.path.join(ROOT, "stochasticseriesexpansion.jl_gb300", "build.py"))
    pkg_build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pkg_build)
    flags = [f.replace("code=sm_103a", "code=compute_103a") for f in pkg_build.NVCC_FLAGS if f != "-lineinfo"]
    nvcc = os.environ.get("NVCC", "nvcc")
    subprocess.run([nvcc, *flags, "-cudart", "none", "-I", os.path.join(ROOT, "include"), "-o", LIB + ".tmp",
                    os.path.join(CSRC, "sse_engine.cu"), os.path.join(FAKE, "fake_cudart.cpp"), *objs], check=True)
    os.replace(LIB + ".tmp", LIB)


if __name__ == "__main__":
    print(build())
