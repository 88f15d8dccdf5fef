"""Import helper: the package directory name contains a dot, so it is loaded
by path and registered as ``sse_gb300``."""

import importlib.util
import os
import sys

PKG_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "stochasticseriesexpansion.jl_gb300")


def load():
    mod = sys.modules.get("sse_gb300")
    if mod is not None:
        return mod
    spec = importlib.util.spec_from_file_location(
        "sse_gb300", os.path.join(PKG_DIR, "__init__.py"), submodule_search_locations=[PKG_DIR]
    )
    mod = importlib.util.module_from_spec(spec)
    sys.modules["sse_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod
