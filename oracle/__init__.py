"""CPU oracle for the co-occurrence path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker or the timed CPU baseline. The product
library (stcdb_gb300) never imports it.

  Oracle       ctypes wrapper of the C restatement in stc_oracle.c
  LsmOracle    memtable + flush restatement (stc_lsm.c) and its pinned
               single routines (ctf_bits, serialize_mbr, pack_key, o_bitmap)
  build()      compiles liboracle.so (and, where the read-only reference
               checkout exists, the reference harness oracle/_ref/ref_driver)
  run_reference_driver()  runs oracle/_ref/ref_driver on a trace (pinning)
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "liboracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")
REF_CTF = os.path.join(HERE, "_ref", "ref_ctf")
REF_COMPACT = os.path.join(HERE, "_ref", "ref_compact")

MEETING_DTYPE = np.dtype([("pid_lo", "<u4"), ("pid_hi", "<u4"), ("start", "<u4"), ("end", "<u4"),
                          ("mbr", "<f4", (4,))])


def build(reference: bool = True) -> None:
    srcs = [os.path.join(HERE, "stc_oracle.c"), os.path.join(HERE, "stc_lsm.c")]
    cpp = os.path.join(HERE, "stc_compact.cpp")
    deps = srcs + [cpp, os.path.join(HERE, "stc_oracle.h"), os.path.join(ROOT, "include", "stc.h")]
    if not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        inc = ["-I" + os.path.join(ROOT, "include"), "-I" + HERE]
        with tempfile.TemporaryDirectory() as tmp:
            obj = os.path.join(tmp, "stc_compact.o")
            subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-Wall", "-c", cpp, "-o", obj]
                           + inc, check=True)
            subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall"] + inc
                           + ["-o", LIB] + srcs + [obj, "-lstdc++", "-lm"], check=True)
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
    lib.cmp_compact.restype = ctypes.c_void_p
    lib.cmp_compact.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]
    lib.cmp_get.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.cmp_read.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 7
    lib.cmp_free.argtypes = [ctypes.c_void_p]
    lib.lsm_create.restype = ctypes.c_void_p
    lib.lsm_create.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double,
                               ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64]
    lib.lsm_destroy.argtypes = [ctypes.c_void_p]
    lib.lsm_error.argtypes = [ctypes.c_void_p]
    lib.lsm_error.restype = ctypes.c_char_p
    lib.lsm_append.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
    lib.lsm_kv_count.argtypes = [ctypes.c_void_p]
    lib.lsm_kv_count.restype = ctypes.c_uint64
    lib.lsm_flush.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
    lib.lsm_get_ctb.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.lsm_read_ctb.argtypes = [ctypes.c_void_p] * 8
    lib.lsm_ctf_bits.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_void_p]
    lib.lsm_serialize_mbr.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.lsm_serialize_mbr.restype = ctypes.c_uint64
    lib.lsm_pack_key.argtypes = [ctypes.c_uint64] * 5 + [ctypes.c_void_p, ctypes.c_void_p]
    lib.lsm_o_bitmap.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.lsm_o_bitmap_edge.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
    lib.lsm_set_bitmap_edge.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
    lib.lsm_decode_key.argtypes = [ctypes.c_void_p] * 8
    lib.lsm_query_object_block.argtypes = [ctypes.c_void_p] * 6 + [ctypes.c_uint32] * 3 + [
        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t]
    lib.lsm_query_object_block.restype = ctypes.c_size_t
    lib.lsm_query_box_block.argtypes = [ctypes.c_void_p] * 6 + [ctypes.c_uint32] * 2 + [
        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t]
    lib.lsm_query_box_block.restype = ctypes.c_size_t
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


class LsmOracle:
    """Memtable + flush restatement (stc_lsm.c). Feed each step's emitted
    meetings with append(); flush(t) builds a block readable with read()."""

    def __init__(self, num_objects: int, max_meet_time: int, ctf_count: int, area_restriction: float,
                 first_end_time_min: int, mbr, capacity: int, bitmap_edge: int = 0):
        self._lib = lib()
        self._n = num_objects
        self._map = np.ascontiguousarray(mbr, dtype=np.float64)
        self._h = self._lib.lsm_create(num_objects, max_meet_time, ctf_count, area_restriction,
                                       first_end_time_min, self._map.ctypes.data, capacity)
        if not self._h:
            raise MemoryError("lsm_create failed")
        if bitmap_edge and self._lib.lsm_set_bitmap_edge(self._h, bitmap_edge) != 0:
            self.close()
            raise ValueError(f"bitmap_edge {bitmap_edge}: a multiple of 32 up to 1024")

    def append(self, meetings: np.ndarray) -> None:
        m = np.ascontiguousarray(meetings, dtype=MEETING_DTYPE)
        if self._lib.lsm_append(self._h, m.ctypes.data, len(m)) != 0:
            raise RuntimeError(self._lib.lsm_error(self._h).decode())

    def kv_count(self) -> int:
        return int(self._lib.lsm_kv_count(self._h))

    def flush(self, t: int) -> None:
        if self._lib.lsm_flush(self._h, t) != 0:
            raise RuntimeError(self._lib.lsm_error(self._h).decode())

    def read(self):
        from stcdb_gb300.pipeline import StcCtbInfo, ctb_buffers, ctb_trim
        info = StcCtbInfo()
        if self._lib.lsm_get_ctb(self._h, ctypes.byref(info)) != 0:
            raise RuntimeError("no block flushed")
        b = ctb_buffers(info, self._n)
        self._lib.lsm_read_ctb(self._h, *[b[k].ctypes.data for k in (
            "ctfs", "bitmaps", "keys", "sids", "oversize_keys", "oversize_boxes", "oversize_bitmap")])
        return info, ctb_trim(info, b)

    def close(self):
        if self._h:
            self._lib.lsm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ctf_bits(mbr, map_box, num_objects: int, max_meet_time: int) -> np.ndarray:
    """lsm_ctf_bits for one CTF box: an stc_ctf record with the bit fields set."""
    from stcdb_gb300.pipeline import CTF_DTYPE
    c = np.zeros(1, CTF_DTYPE)
    c["mbr"][0] = np.asarray(mbr, np.float32)
    m = np.ascontiguousarray(map_box, np.float64)
    f = np.ascontiguousarray(np.asarray(mbr, np.float32))
    lib().lsm_ctf_bits(f.ctypes.data, m.ctypes.data, num_objects, max_meet_time, c.ctypes.data)
    return c


def serialize_mbr(box, ctf: np.ndarray) -> int:
    b = np.ascontiguousarray(np.asarray(box, np.float32))
    return int(lib().lsm_serialize_mbr(b.ctypes.data, ctf.ctypes.data))


def pack_key(pid_field: int, target: int, duration: int, end: int, value_mbr: int, ctf: np.ndarray) -> bytes:
    out = np.zeros(16, np.uint8)
    lib().lsm_pack_key(pid_field, target, duration, end, value_mbr, ctf.ctypes.data, out.ctypes.data)
    return bytes(out[: int(ctf["key_bit"][0]) // 8])


def o_bitmap(boxes: np.ndarray, map_box, edge: int = 256) -> np.ndarray:
    """The map bitmap (edge x edge bits) of a set of oversize key boxes."""
    bm = np.zeros(edge * edge // 8, np.uint8)
    m = np.ascontiguousarray(map_box, np.float64)
    for b in np.ascontiguousarray(boxes, np.float32).reshape(-1, 4):
        bb = np.ascontiguousarray(b)
        if edge == 256:
            lib().lsm_o_bitmap(bb.ctypes.data, m.ctypes.data, bm.ctypes.data)
        else:
            lib().lsm_o_bitmap_edge(bb.ctypes.data, m.ctypes.data, edge, bm.ctypes.data)
    return bm


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


def _block_args(info, bufs):
    return (ctypes.byref(info), bufs["ctfs"].ctypes.data, bufs["keys"].ctypes.data)


def query_blocks(blocks, queries) -> list:
    """The oracle's answers (lsm_query_*_block) over a list of (info, buffers)
    blocks as stc_read_ctb lays them out; one CONTACT_DTYPE array per query."""
    from stcdb_gb300.pipeline import CONTACT_DTYPE, QUERY_BOX
    out = []
    for q in queries:
        res = []
        for info, b in blocks:
            keys = b["keys"] if len(b["keys"]) else np.zeros(1, np.uint8)
            okeys = b["oversize_keys"] if len(b["oversize_keys"]) else np.zeros(2, np.uint64)
            oboxes = b["oversize_boxes"] if len(b["oversize_boxes"]) else np.zeros(4, np.float32)
            cap = 1 << 12
            while True:
                buf = np.zeros(cap, CONTACT_DTYPE)
                if int(q["kind"]) == QUERY_BOX:
                    qb = np.ascontiguousarray(q["box"], np.float64)
                    n = lib().lsm_query_box_block(ctypes.byref(info), b["ctfs"].ctypes.data, keys.ctypes.data,
                                                  okeys.ctypes.data, oboxes.ctypes.data, qb.ctypes.data,
                                                  int(q["t_start"]), int(q["t_end"]), buf.ctypes.data, cap, 0)
                else:
                    n = lib().lsm_query_object_block(ctypes.byref(info), b["ctfs"].ctypes.data, keys.ctypes.data,
                                                     b["sids"].ctypes.data, okeys.ctypes.data, oboxes.ctypes.data,
                                                     int(q["pid"]), int(q["t_start"]), int(q["t_end"]),
                                                     buf.ctypes.data, cap, 0)
                if n <= cap:
                    res.append(buf[:n])
                    break
                cap = n
        out.append(np.concatenate(res) if res else np.zeros(0, CONTACT_DTYPE))
    return out


def _cmp_block_type():
    """cmp_block (stc_oracle.h)."""
    from stcdb_gb300.pipeline import StcCtbInfo

    class CmpBlock(ctypes.Structure):
        _fields_ = [("info", StcCtbInfo), ("ctfs", ctypes.c_void_p), ("keys", ctypes.c_void_p),
                    ("sids", ctypes.c_void_p), ("okeys", ctypes.c_void_p), ("oboxes", ctypes.c_void_p),
                    ("obitmap", ctypes.c_void_p)]
    return CmpBlock


def compact(blocks, num_objects: int, split: int, max_meet_time: int, map_box, new_index: int,
            reference_mode: bool = False):
    """cmp_compact over a list of (info, buffers) blocks as stc_read_ctb lays
    them out; returns (info, buffers) of the merged block."""
    from stcdb_gb300.pipeline import StcCtbInfo, ctb_buffers, ctb_trim
    keep = []
    arr = (_cmp_block_type() * len(blocks))()
    for i, (info, b) in enumerate(blocks):
        bufs = {k: np.ascontiguousarray(b[k]) for k in ("ctfs", "keys", "sids", "oversize_keys", "oversize_boxes",
                                                        "oversize_bitmap")}
        for k, dt, n in (("keys", np.uint8, 16), ("oversize_keys", np.uint64, 2), ("oversize_boxes", np.float32, 4)):
            if len(bufs[k]) == 0:
                bufs[k] = np.zeros(n, dt)
        keep.append(bufs)
        arr[i].info = info
        arr[i].ctfs = bufs["ctfs"].ctypes.data
        arr[i].keys = bufs["keys"].ctypes.data
        arr[i].sids = bufs["sids"].ctypes.data
        arr[i].okeys = bufs["oversize_keys"].ctypes.data
        arr[i].oboxes = bufs["oversize_boxes"].ctypes.data
        arr[i].obitmap = bufs["oversize_bitmap"].ctypes.data
    m = np.ascontiguousarray(map_box, np.float64)
    err = ctypes.create_string_buffer(256)
    h = lib().cmp_compact(ctypes.byref(arr), len(blocks), num_objects, split, max_meet_time, m.ctypes.data,
                          new_index, int(bool(reference_mode)), err, 256)
    if not h:
        raise RuntimeError("cmp_compact: " + err.value.decode())
    try:
        info = StcCtbInfo()
        lib().cmp_get(h, ctypes.byref(info))
        out = ctb_buffers(info, num_objects)
        lib().cmp_read(h, *[out[k].ctypes.data for k in (
            "ctfs", "bitmaps", "keys", "sids", "oversize_keys", "oversize_boxes", "oversize_bitmap")])
    finally:
        lib().cmp_free(h)
    return info, ctb_trim(info, out)
