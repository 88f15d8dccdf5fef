"""Development aid: dry-runs the -m gpu tests on the CPU with Engine() bound to the emulated-warp
build (tests/warp_emu), one test per process under a time limit.

The results are NOT GPU results.  They say that each test's logic holds for the engine's kernels
run on emulated warps: the checks a test makes, the host code it drives, and the kernels'
arithmetic against the oracle.  Whether the compiled sm_103a code does the same is what the real
-m gpu run on a GB300 decides.  Not runnable here, and skipped by default:
 - tests whose buffers come from torch.cuda;
 - the full-size 4096-walker test and the statistical comparisons with exact diagonalisation
   (hours of emulated sweeps).

    python tests/warp_emu/run_gpu_tests.py [pytest node ids ...] [--limit SECONDS]
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SKIP = ("test_gpu_fullsize", "test_zz_no_alloc", "_vs_ed", "matches_ed")

CHILD = r"""
import os, sys
sys.path.insert(0, {root!r}); sys.path.insert(0, os.path.join({root!r}, "tests"))
import importlib.util
import _sse_loader
_sse_loader.load()
spec = importlib.util.spec_from_file_location("_emu_build", os.path.join({here!r}, "build.py"))
build = importlib.util.module_from_spec(spec); spec.loader.exec_module(build)
import sse_gb300.engine as E
lib = E.load_library(build.build())
real = E.Engine.__init__
E.Engine.__init__ = lambda self, device=0, library=None: real(self, device, library if library is not None else lib)
import pytest
os.chdir({root!r})
sys.exit(pytest.main(["-q", "-p", "no:cacheprovider", "-m", "gpu", {node!r}]))
"""


def collect():
    out = subprocess.run([sys.executable, "-m", "pytest", "-m", "gpu", "--collect-only", "-q", "tests"], cwd=ROOT,
                         capture_output=True, text=True).stdout
    return [ln.strip() for ln in out.splitlines() if "::" in ln and not any(s in ln for s in SKIP)]


def main(argv):
    limit = 180
    if "--limit" in argv:
        i = argv.index("--limit")
        limit = int(argv[i + 1])
        argv = argv[:i] + argv[i + 2:]
    nodes = argv or collect()
    bad = []
    for node in nodes:
        code = CHILD.format(root=ROOT, here=HERE, node=node)
        try:
            r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=limit)
            status = "passed" if r.returncode == 0 else "FAILED"
        except subprocess.TimeoutExpired:
            status = f"over {limit} s"
        print(f"{status:10s} {node}", flush=True)
        if status != "passed":
            bad.append(node)
    print(f"{len(nodes) - len(bad)} of {len(nodes)} passed on the emulated engine")
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
