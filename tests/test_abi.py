"""The C-ABI library loads and exports every entry point of include/*.h;
argument validation happens before any device call."""
import ctypes
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    inc = os.path.join(ROOT, "include")
    names = set()
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            text = re.sub(r"/\*.*?\*/", "", open(os.path.join(inc, f)).read(), flags=re.S)
            names.update(re.findall(r"\b(stc_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_exports(built_cuda):
    from stcdb_gb300._lib import load_library
    lib = load_library("libstc")
    names = declared_functions()
    assert "stc_step" in names and "stc_create" in names and "stc_trace_dev_next" in names
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/ but not exported by libstc"


def test_defaults_and_validation(built_cuda):
    from stcdb_gb300.pipeline import _Config, _lib
    lib = _lib()
    c = _Config()
    lib.stc_config_default(ctypes.byref(c), 1000)
    assert c.num_objects == 1000 and c.grid_capacity == 50 and c.num_meeting_buckets == 2000
    assert abs(c.reach_distance - 2.0) < 1e-12 and c.min_meet_time == 5 and c.refine_size == 4
    h = ctypes.c_void_p()
    mbr = np.array([0.0, 0.0, 1.0, 1.0])
    xy = np.zeros((1000, 2))
    c.grid_capacity = 0  # invalid: rejected before touching a device
    st = lib.stc_create(ctypes.byref(c), mbr.ctypes.data, xy.ctypes.data, 1000, ctypes.byref(h))
    assert st == 1 and not h.value
    assert b"invalid" in lib.stc_last_error(None)


def test_random_access_probe_validates_arguments(built_cuda):
    from stcdb_gb300._lib import load_library
    lib = load_library("libstc")
    f = lib.stc_measure_random_access
    f.argtypes = [ctypes.c_uint32, ctypes.c_ulonglong, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]
    f.restype = ctypes.c_int
    ms = ctypes.c_float(-1.0)
    assert f(9, 1000, 0, ctypes.byref(ms)) == 1       # table below 2^10 slots
    assert f(33, 1000, 0, ctypes.byref(ms)) == 1      # table above 2^32 slots
    assert f(20, 0, 0, ctypes.byref(ms)) == 1         # no accesses
    assert f(20, 1000, 0, None) == 1                  # no result pointer
    assert b"invalid" in lib.stc_last_error(None)


def test_refine_chunk_validated_before_any_device_call(built_cuda):
    from stcdb_gb300.pipeline import _Config, _lib
    lib = _lib()
    mbr = np.array([0.0, 0.0, 1.0, 1.0])
    xy = np.zeros((1000, 2))
    for bad in (100, 4128):  # not a multiple of 32; above 4096
        c = _Config()
        lib.stc_config_default(ctypes.byref(c), 1000)
        c.refine_chunk = bad
        h = ctypes.c_void_p()
        assert lib.stc_create(ctypes.byref(c), mbr.ctypes.data, xy.ctypes.data, 1000, ctypes.byref(h)) == 1
        assert not h.value and b"refine_chunk" in lib.stc_last_error(None)
