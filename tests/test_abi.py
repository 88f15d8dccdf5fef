"""The C-ABI library loads and exports every entry point include/sse_gpu.h declares
(no GPU needed: nothing is called)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^\s*(?:int|const char \*)\s*(sse_\w+)\s*\(", src, flags=re.M)
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "sse_sweep" in names and "sse_engine_create" in names
    assert len(names) == len(set(names))


def test_library_exports_every_declared_symbol():
    from sse_gb300 import build as B

    try:
        path = B.build()
    except (FileNotFoundError, OSError) as e:  # no nvcc on this machine
        pytest.skip(f"nvcc unavailable: {e}")
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from sse_gb300.engine import exported_symbols

    assert set(exported_symbols()) >= set(declared_symbols())
