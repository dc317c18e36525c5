"""CPU oracle for the co-occurrence path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker or the timed CPU baseline. The product
library (stcdb_gb300) never imports it.

  Oracle       ctypes wrapper of the C restatement in stc_oracle.c
  build()      compiles liboracle.so (and, where the read-only reference
               checkout exists, the reference harness oracle/_ref/ref_driver)
  run_reference_driver()  runs oracle/_ref/ref_driver on a trace (pinning)
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "liboracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

MEETING_DTYPE = np.dtype([("pid_lo", "<u4"), ("pid_hi", "<u4"), ("start", "<u4"), ("end", "<u4"),
                          ("mbr", "<f4", (4,))])


def build(reference: bool = True) -> None:
    src = os.path.join(HERE, "stc_oracle.c")
    deps = [src, os.path.join(HERE, "stc_oracle.h"), os.path.join(ROOT, "include", "stc.h")]
    if not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall",
                        "-I" + os.path.join(ROOT, "include"), "-o", LIB, src, "-lm"], check=True)
    if reference:
        subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True)


def _lib():
    if not os.path.exists(LIB):
        build(reference=False)
    lib = ctypes.CDLL(LIB)
    lib.oracle_create.restype = ctypes.c_void_p
    lib.oracle_create.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                  ctypes.c_int]
    lib.oracle_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
    lib.oracle_emitted.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
    lib.oracle_emitted.restype = ctypes.c_size_t
    lib.oracle_error.argtypes = [ctypes.c_void_p]
    lib.oracle_error.restype = ctypes.c_char_p
    lib.oracle_destroy.argtypes = [ctypes.c_void_p]
    lib.oracle_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.oracle_dpml.argtypes = [ctypes.c_double]
    lib.oracle_dpml.restype = ctypes.c_double
    lib.oracle_schema_size.argtypes = [ctypes.c_void_p]
    lib.oracle_schema_size.restype = ctypes.c_uint32
    lib.oracle_schema_stack_index.argtypes = [ctypes.c_void_p]
    lib.oracle_schema_stack_index.restype = ctypes.c_uint32
    lib.oracle_grids_stack_index.argtypes = [ctypes.c_void_p]
    lib.oracle_grids_stack_index.restype = ctypes.c_uint32
    lib.oracle_schema_dump.argtypes = [ctypes.c_void_p] * 5
    return lib


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = _lib()
    return _LIB


class Oracle:
    """Single-threaded (threads=1) is the deterministic golden order."""

    def __init__(self, cfg, mbr, xy0: np.ndarray, threads: int = 1):
        from stcdb_gb300.pipeline import config_struct
        self._cfg = config_struct(cfg)
        self._mbr = np.ascontiguousarray(mbr, dtype=np.float64)
        xy0 = np.ascontiguousarray(xy0, dtype=np.float64)
        self._lib = lib()
        self._h = self._lib.oracle_create(ctypes.byref(self._cfg), self._mbr.ctypes.data, xy0.ctypes.data,
                                          xy0.shape[0], threads)
        if not self._h:
            raise MemoryError("oracle_create failed")
        err = self._lib.oracle_error(self._h)
        if err:
            raise RuntimeError(err.decode())

    def step(self, xy: np.ndarray, t: int) -> np.ndarray:
        xy = np.ascontiguousarray(xy, dtype=np.float64)
        if self._lib.oracle_step(self._h, xy.ctypes.data, t) != 0:
            raise RuntimeError(self._lib.oracle_error(self._h).decode())
        p = ctypes.c_void_p()
        n = self._lib.oracle_emitted(self._h, ctypes.byref(p))
        if n == 0:
            return np.zeros(0, dtype=MEETING_DTYPE)
        buf = (ctypes.c_char * (n * MEETING_DTYPE.itemsize)).from_address(p.value)
        return np.frombuffer(bytes(buf), dtype=MEETING_DTYPE).copy()

    def stats(self):
        from stcdb_gb300.pipeline import StcStats
        s = StcStats()
        self._lib.oracle_stats(self._h, ctypes.byref(s))
        return s

    def schema(self):
        n = self._lib.oracle_schema_size(self._h)
        typ = np.zeros(n, np.int16)
        gid = np.zeros(n, np.uint32)
        ch = np.zeros((n, 4), np.uint32)
        bx = np.zeros((n, 4), np.float64)
        self._lib.oracle_schema_dump(self._h, typ.ctypes.data, gid.ctypes.data, ch.ctypes.data, bx.ctypes.data)
        return dict(type=typ, grid_id=gid, children=ch, boxes=bx,
                    schema_stack_index=self._lib.oracle_schema_stack_index(self._h),
                    grids_stack_index=self._lib.oracle_grids_stack_index(self._h))

    def close(self):
        if self._h:
            self._lib.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dpml(lat: float) -> float:
    return lib().oracle_dpml(lat)


# ---------------------------------------------------------------------------
# The reference's own CPU path (oracle/_ref/ref_driver), for pinning.

def write_trace(path: str, trace: np.ndarray, mbr) -> None:
    T, N, _ = trace.shape
    with open(path, "wb") as f:
        f.write(struct.pack("<II", N, T))
        f.write(np.asarray(mbr, np.float64).tobytes())
        f.write(np.ascontiguousarray(trace, dtype=np.float64).tobytes())


def read_reference_output(path: str):
    d = np.fromfile(path, dtype=np.uint32)
    i = 0
    steps = []
    while i < len(d):
        t, c, units, leaves = (int(v) for v in d[i:i + 4])
        i += 4
        recs = d[i:i + 4 * c].reshape(c, 4).copy()
        i += 4 * c
        steps.append(dict(t=t, units=units, leaves=leaves, meetings=recs))
    return steps


def reference_available() -> bool:
    return os.path.exists(REF_DRIVER)


def run_reference_driver(trace: np.ndarray, mbr, cfg, workdir: str):
    """Runs the reference's own single-threaded CPU path; returns per-step dicts
    with (pid_lo, pid_hi, start, end) rows in the reference's emission order."""
    os.makedirs(workdir, exist_ok=True)
    tp = os.path.join(workdir, "trace.bin")
    op = os.path.join(workdir, "ref_out.bin")
    write_trace(tp, trace, mbr)
    args = [REF_DRIVER, tp, op, repr(float(cfg.reach_distance)), str(cfg.min_meet_time),
            str(cfg.grid_capacity), repr(float(cfg.grid_amplify)), str(cfg.num_meeting_buckets),
            str(cfg.refine_size), "1", "1" if cfg.dynamic_schema else "0"]
    subprocess.run(args, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return read_reference_output(op)
