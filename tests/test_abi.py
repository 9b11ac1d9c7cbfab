"""The C-ABI library loads, exports every function include/grt.h declares, and answers
argument errors with status codes (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    names = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"\b(grt_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(api):
    lib = ctypes.CDLL(os.path.join(ROOT, "illum-rt_gb300", "_lib", "libgrt.so"))
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_defaults(api):
    L = api.lib()
    assert L.grt_version() == 1002
    o = api.BvhOpts()
    L.grt_bvh_opts_default(ctypes.byref(o))
    assert (o.split, o.max_tris_per_node, o.number_of_planes, o.esc) == (2, 4, 16, 1)


def test_null_arguments_are_rejected(api):
    L = api.lib()
    assert L.grt_create(None, None) == 1
    assert L.grt_destroy(None) == 1
    assert L.grt_trace(None, None, None, 0, 0, None) == 1
    assert L.grt_check(None, None, 0) == 1
    assert L.grt_select_tracer(None, b"while-while") == 1
    assert L.grt_last_error(None) == b"null context"


def test_create_without_device_reports_no_device(api):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    h = ctypes.c_void_p()
    assert api.lib().grt_create(None, ctypes.byref(h)) == 9  # GRT_ERR_NO_DEVICE
    assert not h.value
