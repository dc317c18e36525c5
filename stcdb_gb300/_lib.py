"""Locates and loads the in-tree shared libraries built by stcdb_gb300.build."""
from __future__ import annotations

import ctypes
import os

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib")

_cache: dict[str, ctypes.CDLL] = {}


def library_path(name: str) -> str:
    return os.path.join(LIB_DIR, name + ".so")


def load_library(name: str) -> ctypes.CDLL:
    """Loads lib/<name>.so; fails loudly when it has not been built."""
    lib = _cache.get(name)
    if lib is not None:
        return lib
    path = library_path(name)
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the native libraries first "
            f"(python -c 'import stcdb_gb300.build as b; b.build_all()')")
    lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    _cache[name] = lib
    return lib
