"""Loading of the package's native libraries.

``build.py`` compiles them in-tree into ``_lib/``. Loading fails loudly when a library is
missing: there is no pure-Python or CPU fallback for any traversal entry point.
"""
from __future__ import annotations

import ctypes
import os

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")
_cache: dict[str, ctypes.CDLL] = {}


def _load(name: str) -> ctypes.CDLL:
    if name in _cache:
        return _cache[name]
    path = os.path.join(LIB_DIR, name)
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the native libraries first "
                           "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(path)
    _cache[name] = lib
    return lib


def workloads() -> ctypes.CDLL:
    lib = _load("libgrt_workloads.so")
    lib.wl_log_uniform.restype = ctypes.c_uint64
    return lib


def grt() -> ctypes.CDLL:
    """The C-ABI traversal library (include/grt.h)."""
    from . import api  # noqa: F401  (declares the prototypes)
    return api.lib()
