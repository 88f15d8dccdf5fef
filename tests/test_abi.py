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


def test_abi_version_matches_header_and_bindings():
    """The structs of engine.py mirror the header's; the library reports the same version (a plain
    C function: nothing touches the GPU)."""
    from sse_gb300 import build as B
    from sse_gb300.engine import ABI_VERSION

    src = open(os.path.join(ROOT, "include", "sse_gpu.h")).read()
    (hv,) = re.findall(r"#define SSE_GPU_ABI_VERSION (\d+)", src)
    assert int(hv) == ABI_VERSION
    try:
        path = B.build()
    except (FileNotFoundError, OSError) as e:  # no nvcc on this machine
        pytest.skip(f"nvcc unavailable: {e}")
    lib = ctypes.CDLL(path)
    lib.sse_abi_version.restype = ctypes.c_int
    assert lib.sse_abi_version() == ABI_VERSION


def test_ctypes_structs_match_header_layout(tmp_path):
    """Every field offset and the size of the four ABI structs, as the C compiler lays them out
    from include/sse_gpu.h, equal those of the ctypes mirrors in engine.py."""
    import shutil
    import subprocess

    from sse_gb300.engine import ModelDesc, NoAllocWalker, WalkerInfo, WalkerParams

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"sse_model_desc": ModelDesc, "sse_walker_params": WalkerParams, "sse_walker_info": WalkerInfo,
               "sse_noalloc_walker": NoAllocWalker}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "sse_gpu.h"', "int main(void) {"]
    for cname, cls in mirrors.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {(a, b): int(c) for a, b, c in (ln.split() for ln in out if ln)}
    for cname, cls in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert got[(cname, field)] == getattr(cls, field).offset, (cname, field)



def test_model_tables_follow_desc_order_and_types():
    """register_model fills sse_model_desc's pointers from MODEL_TABLES in order, with the element
    type each pointer field declares."""
    from sse_gb300.engine import _CTYPE, MODEL_TABLES, ModelDesc

    ptr_fields = [(f, t) for f, t in ModelDesc._fields_ if issubclass(t, ctypes._Pointer)]
    assert [f for f, _ in ptr_fields] == [n for n, _ in MODEL_TABLES]
    for (f, t), (_, dt) in zip(ptr_fields, MODEL_TABLES):
        assert t._type_ is _CTYPE[dt], f


def test_model_table_conversion():
    import numpy as np

    from sse_gb300.engine import model_table

    # a wider integer type and a strided view are converted to contiguous int32
    a = {"bond_sites": np.arange(12, dtype=np.int64)[::2]}
    t = model_table(a, "bond_sites", np.int32)
    assert t.dtype == np.int32 and t.flags.c_contiguous and t.tolist() == list(range(0, 12, 2))
    # a conversion that changes values is refused
    with pytest.raises(ValueError):
        model_table({"bond_type": np.array([1 << 40])}, "bond_type", np.int32)
    with pytest.raises(ValueError):
        model_table({"leg_state": np.array([0.5])}, "leg_state", np.uint8)
    with pytest.raises(ValueError):
        model_table({"leg_state": np.array([-1])}, "leg_state", np.uint8)


def test_flattened_tables_need_no_conversion(S):
    """The host builder already emits every table of every model family in its C type, so
    registration passes the builder's own arrays."""
    import numpy as np

    from sse_gb300.engine import MODEL_TABLES, model_table
    from test_tables import families

    for family, make in families(S).items():
        flat = S.flatten_model(make(S))
        for name, dt in MODEL_TABLES:
            arr = flat.arrays[name]
            assert arr.dtype == dt and arr.flags.c_contiguous, (family, name)
            assert arr.size == 0 or np.shares_memory(model_table(flat.arrays, name, dt), arr), (family, name)
