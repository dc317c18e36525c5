"""Python mirror of the C ABI in include/stc.h (ctypes over lib/libstc.so).

`Pipeline` follows the reference's driver loop (tracing/process.cpp:401-612):
it is created from the step-0 positions like partitioner::build_schema
(tracing/filter.cpp:27) and then processes one step per call like
process_with_gpu (cuda/geometry.cu:1573). Every call goes through the CUDA
library; there is no CPU fallback, and a missing library raises.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, fields, replace

import numpy as np

from ._lib import load_library

MEETING_DTYPE = np.dtype([("pid_lo", "<u4"), ("pid_hi", "<u4"), ("start", "<u4"), ("end", "<u4"),
                          ("mbr", "<f4", (4,))])

FLAG_SERIAL_SCHEMA = 1   # STC_FLAG_* of include/stc.h
FLAG_DIRECT_HITS = 2
FLAG_QUEUED_HITS = 4
FLAG_COPY_INPUT = 8

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "CUDA", 3: "CAPACITY", 4: "TIMEOUT", 5: "UNSUPPORTED", 6: "STATE"}


class StcError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class _Config(ctypes.Structure):
    _fields_ = [
        ("num_objects", ctypes.c_uint32),
        ("min_meet_time", ctypes.c_uint32),
        ("max_meet_time", ctypes.c_uint32),
        ("grid_capacity", ctypes.c_uint32),
        ("grid_amplify", ctypes.c_double),
        ("reach_distance", ctypes.c_double),
        ("num_meeting_buckets", ctypes.c_uint64),
        ("refine_size", ctypes.c_uint32),
        ("schema_update_delay", ctypes.c_uint32),
        ("dynamic_schema", ctypes.c_int32),
        ("mbr_filter", ctypes.c_int32),
        ("candidate_capacity", ctypes.c_uint64),
        ("emit_capacity", ctypes.c_uint64),
        ("hit_capacity", ctypes.c_uint64),
        ("device", ctypes.c_uint32),
        ("flags", ctypes.c_uint32),
        ("kv_restriction", ctypes.c_uint64),
        ("kv_capacity", ctypes.c_uint64),
        ("ctf_count", ctypes.c_uint32),
        ("start_time", ctypes.c_uint32),
        ("area_restriction", ctypes.c_double),
        ("ctb_retain", ctypes.c_uint32),
        ("step_slices", ctypes.c_uint32),
        ("job_chunk", ctypes.c_uint32),
        ("refine_blocks_per_sm", ctypes.c_uint32),
        ("hits_blocks_per_sm", ctypes.c_uint32),
        ("window_graphs", ctypes.c_uint32),
        ("bitmap_edge", ctypes.c_uint32),
        ("refine_chunk", ctypes.c_uint32),
    ]


class _TuneResult(ctypes.Structure):
    _fields_ = [("config", _Config), ("base_step_ms", ctypes.c_float), ("best_step_ms", ctypes.c_float),
                ("trials", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class StcStats(ctypes.Structure):
    _fields_ = [
        ("step", ctypes.c_uint32),
        ("leaves", ctypes.c_uint32),
        ("schema_nodes", ctypes.c_uint32),
        ("overflow_objects", ctypes.c_uint32),
        ("checking_units", ctypes.c_uint64),
        ("border_units", ctypes.c_uint64),
        ("pair_tests", ctypes.c_uint64),
        ("exact_tests", ctypes.c_uint64),
        ("hits", ctypes.c_uint64),
        ("new_candidates", ctypes.c_uint64),
        ("taken_buckets", ctypes.c_uint64),
        ("emitted", ctypes.c_uint64),
        ("pending", ctypes.c_uint64),
        ("splits", ctypes.c_uint32),
        ("merges", ctypes.c_uint32),
        ("kernel_launches", ctypes.c_uint32),
        ("schema_path", ctypes.c_uint32),
        ("ambiguous_tests", ctypes.c_uint32),
        ("step_ms", ctypes.c_float),
        ("phase_ms", ctypes.c_float * 8),
        ("memtable_keys", ctypes.c_uint64),
        ("flushes", ctypes.c_uint32),
        ("flush_ms", ctypes.c_float),
        ("window_device_ms", ctypes.c_float),
        ("window_wall_ms", ctypes.c_float),
        ("window_input_wait_ms", ctypes.c_float),
        ("window_copy_ms", ctypes.c_float),
        ("flush_stage_ms", ctypes.c_float * 5),
        ("compact_stage_ms", ctypes.c_float * 7),
    ]

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if name == "phase_ms" else v
        return d


class StcCtbInfo(ctypes.Structure):
    """stc_ctb_info: one flushed contact tracing block."""
    _fields_ = [
        ("index", ctypes.c_uint32),
        ("ctf_count", ctypes.c_uint32),
        ("flush_time", ctypes.c_uint32),
        ("end_time_min", ctypes.c_uint32),
        ("kv_count", ctypes.c_uint64),
        ("ctf_kv_count", ctypes.c_uint64),
        ("oversize_kv_count", ctypes.c_uint64),
        ("key_bytes", ctypes.c_uint64),
        ("sid_count", ctypes.c_uint32),
        ("oversize_oid_count", ctypes.c_uint32),
        ("o_start_time_min", ctypes.c_uint32),
        ("o_start_time_max", ctypes.c_uint32),
        ("o_end_time_min", ctypes.c_uint32),
        ("o_end_time_max", ctypes.c_uint32),
        ("bitmap_edge", ctypes.c_uint32),
        ("pad", ctypes.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


# stc_ctf (include/stc.h), 80 bytes
CTF_DTYPE = np.dtype([("mbr", "<f4", (4,)), ("kv_count", "<u4"), ("start_time_min", "<u4"),
                      ("start_time_max", "<u4"), ("end_time_min", "<u4"), ("end_time_max", "<u4"),
                      ("bitmap_bytes", "<u4"), ("key_bit", "<u2"), ("id_bit", "<u2"), ("duration_bit", "<u2"),
                      ("end_bit", "<u2"), ("low_x_bit", "<u2"), ("low_y_bit", "<u2"), ("edge_bit", "<u2"),
                      ("mbr_bit", "<u2"), ("x_grid", "<u2"), ("y_grid", "<u2"), ("pad", "<u4"),
                      ("first_key", "<u8"), ("key_offset", "<u8")])
assert CTF_DTYPE.itemsize == 80
BITMAP_BYTES = 8192  # STC_BITMAP_BYTES: one CTF bitmap slot


def map_bitmap_bytes(edge: int) -> int:
    """STC_MAP_BITMAP_BYTES: bytes of a block's map bitmap of edge x edge bits."""
    edge = int(edge) or 256
    return edge * edge // 8

# stc_contact and stc_query (include/stc.h)
CONTACT_DTYPE = np.dtype([("pid", "<u4"), ("target", "<u4"), ("start", "<u4"), ("end", "<u4"),
                          ("mbr", "<f8", (4,)), ("block", "<u4"), ("ctf", "<u4")])
assert CONTACT_DTYPE.itemsize == 56
QUERY_DTYPE = np.dtype([("kind", "<u4"), ("pid", "<u4"), ("t_start", "<u4"), ("t_end", "<u4"),
                        ("box", "<f8", (4,))])
assert QUERY_DTYPE.itemsize == 48
QUERY_OBJECT, QUERY_BOX, QUERY_COUNT_ONLY = 0, 1, 0x100
ANSWER_DTYPE = np.dtype([("ticket", "<u8"), ("count", "<u8"), ("contact_offset", "<u8"), ("stored", "<u4"),
                         ("status", "<u4"), ("latency_ms", "<f8"), ("batch", "<u4"), ("batch_size", "<u4")])
assert ANSWER_DTYPE.itemsize == 48


class _ServerConfig(ctypes.Structure):
    _fields_ = [("max_batch", ctypes.c_uint32), ("result_cap", ctypes.c_uint32), ("hbm_budget", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("answered", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("max_batch_queries", ctypes.c_uint64), ("max_batch_bytes", ctypes.c_uint64),
                ("budget_cuts", ctypes.c_uint64), ("overlapped_batches", ctypes.c_uint64),
                ("slowest_batch_wall_us", ctypes.c_uint64), ("slowest_batch_gpu_us", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


def sort_contacts(c: np.ndarray) -> np.ndarray:
    """Canonical order for comparing contact sets."""
    c = np.ascontiguousarray(c, dtype=CONTACT_DTYPE)
    order = np.lexsort((c["ctf"], c["block"], c["end"], c["start"], c["target"], c["pid"]))
    return c[order]


def ctb_buffers(info: StcCtbInfo, num_objects: int) -> dict:
    """Host arrays sized for one block, in the layout of stc_read_ctb."""
    return dict(ctfs=np.zeros(info.ctf_count, CTF_DTYPE),
                bitmaps=np.zeros(info.ctf_count * BITMAP_BYTES, np.uint8),
                keys=np.zeros(max(int(info.key_bytes), 1), np.uint8),
                sids=np.zeros(num_objects, np.uint16),
                oversize_keys=np.zeros(2 * max(int(info.oversize_kv_count), 1), np.uint64),
                oversize_boxes=np.zeros(4 * max(int(info.oversize_kv_count), 1), np.float32),
                oversize_bitmap=np.zeros(map_bitmap_bytes(info.bitmap_edge), np.uint8))


def ctb_trim(info: StcCtbInfo, bufs: dict) -> dict:
    """Cuts the padded buffers of ctb_buffers to the block's sizes."""
    out = dict(bufs)
    out["keys"] = bufs["keys"][: int(info.key_bytes)]
    out["oversize_keys"] = bufs["oversize_keys"][: 2 * int(info.oversize_kv_count)]
    out["oversize_boxes"] = bufs["oversize_boxes"][: 4 * int(info.oversize_kv_count)]
    return out


@dataclass(frozen=True)
class StcConfig:
    """Pipeline parameters (meanings of util/config.h:15-114)."""
    num_objects: int
    reach_distance: float = 2.0
    min_meet_time: int = 5
    max_meet_time: int = 4096
    grid_capacity: int = 50
    grid_amplify: float = 2.0
    num_meeting_buckets: int = 0      # 0 = reference default 2N
    refine_size: int = 4
    schema_update_delay: int = 1
    dynamic_schema: bool = True
    mbr_filter: bool = True
    candidate_capacity: int = 0
    emit_capacity: int = 0
    hit_capacity: int = 0
    device: int = 0
    flags: int = 0            # STC_FLAG_* bits of include/stc.h
    kv_restriction: int = 0   # memtable flush threshold in directed keys; 0 = no memtable
    kv_capacity: int = 0      # 0 = kv_restriction + 1,000,000
    ctf_count: int = 0        # 0 = 100
    start_time: int = 0
    area_restriction: float = 0.0  # 0 = 100 (no cut)
    ctb_retain: int = 0       # flushed blocks kept for queries; 0 = 8
    step_slices: int = 0      # launches per long step kernel (query latency under ingest); 0 = 1
    job_chunk: int = 0        # refinement launch shape (results do not depend on it); 0 = 8
    refine_blocks_per_sm: int = 0  # 0 = 8
    hits_blocks_per_sm: int = 0    # 0 = 16
    window_graphs: int = 0    # step_window replays captured graphs: 0 = for short steps (automatic), 1 = always, 2 = never
    bitmap_edge: int = 0      # edge of a block's map bitmap (oversize buffer); 0 = 256
    refine_chunk: int = 0     # refinement tile length, candidate positions per job (launch shape); 0 = by density

    def resolved(self) -> "StcConfig":
        if self.num_meeting_buckets == 0:
            return replace(self, num_meeting_buckets=2 * self.num_objects)
        return self


def config_struct(cfg: StcConfig) -> _Config:
    cfg = cfg.resolved()
    c = _Config()
    for f in fields(cfg):
        setattr(c, f.name, int(getattr(cfg, f.name)) if not isinstance(getattr(cfg, f.name), float)
                else getattr(cfg, f.name))
    return c


def autotune(cfg: StcConfig, mbr, xy_steps: np.ndarray, capacities=None) -> tuple:
    """stc_autotune: (the configuration with the chosen leaf capacity and
    refinement launch shape, {"base_step_ms", "best_step_ms", "trials"}).
    xy_steps: (steps >= 3, num_objects, 2) float64 positions in host memory."""
    lib = _lib()
    c = config_struct(cfg)
    mbr = np.ascontiguousarray(mbr, dtype=np.float64)
    xy = np.ascontiguousarray(xy_steps, dtype=np.float64)
    assert xy.ndim == 3 and xy.shape[1:] == (cfg.num_objects, 2)
    caps = np.ascontiguousarray(capacities if capacities is not None else [], dtype=np.uint32)
    r = _TuneResult()
    st = lib.stc_autotune(ctypes.byref(c), mbr.ctypes.data, xy.ctypes.data, cfg.num_objects, xy.shape[0],
                          caps.ctypes.data if len(caps) else None, len(caps), ctypes.byref(r))
    if st != 0:
        raise StcError(st, lib.stc_last_error(None).decode())
    chosen = replace(cfg, grid_capacity=int(r.config.grid_capacity), job_chunk=int(r.config.job_chunk),
                     refine_chunk=int(r.config.refine_chunk), refine_blocks_per_sm=int(r.config.refine_blocks_per_sm),
                     hits_blocks_per_sm=int(r.config.hits_blocks_per_sm))
    return chosen, {"base_step_ms": float(r.base_step_ms), "best_step_ms": float(r.best_step_ms),
                    "trials": int(r.trials)}


def _lib():
    lib = load_library("libstc")
    if not getattr(lib, "_stc_typed", False):
        lib.stc_config_default.argtypes = [ctypes.POINTER(_Config), ctypes.c_uint32]
        lib.stc_create.argtypes = [ctypes.POINTER(_Config), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                   ctypes.POINTER(ctypes.c_void_p)]
        lib.stc_create.restype = ctypes.c_int
        lib.stc_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
        lib.stc_step.restype = ctypes.c_int
        lib.stc_step_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
        lib.stc_step_device.restype = ctypes.c_int
        lib.stc_step_window.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32,
                                        ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t,
                                        ctypes.POINTER(ctypes.c_size_t)]
        lib.stc_step_window.restype = ctypes.c_int
        lib.stc_autotune.argtypes = [ctypes.POINTER(_Config), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                     ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                                     ctypes.POINTER(_TuneResult)]
        lib.stc_autotune.restype = ctypes.c_int
        lib.stc_server_start.argtypes = [ctypes.c_void_p, ctypes.POINTER(_ServerConfig), ctypes.POINTER(ctypes.c_void_p)]
        lib.stc_server_start.restype = ctypes.c_int
        lib.stc_server_submit.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double,
                                          ctypes.POINTER(ctypes.c_uint64)]
        lib.stc_server_submit.restype = ctypes.c_int
        lib.stc_server_poll.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                        ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), ctypes.c_int]
        lib.stc_server_poll.restype = ctypes.c_int
        lib.stc_server_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ServerStats)]
        lib.stc_server_get_stats.restype = ctypes.c_int
        lib.stc_server_stop.argtypes = [ctypes.c_void_p]
        lib.stc_server_stop.restype = ctypes.c_int
        lib.stc_drain_meetings.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                           ctypes.POINTER(ctypes.c_size_t)]
        lib.stc_drain_meetings.restype = ctypes.c_int
        lib.stc_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(StcStats)]
        lib.stc_get_stats.restype = ctypes.c_int
        lib.stc_last_error.argtypes = [ctypes.c_void_p]
        lib.stc_last_error.restype = ctypes.c_char_p
        lib.stc_destroy.argtypes = [ctypes.c_void_p]
        lib.stc_flush.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        lib.stc_flush.restype = ctypes.c_int
        lib.stc_get_ctb.argtypes = [ctypes.c_void_p, ctypes.POINTER(StcCtbInfo)]
        lib.stc_get_ctb.restype = ctypes.c_int
        lib.stc_read_ctb.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 7
        lib.stc_read_ctb.restype = ctypes.c_int
        lib.stc_get_block.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(StcCtbInfo)]
        lib.stc_get_block.restype = ctypes.c_int
        lib.stc_read_block.argtypes = [ctypes.c_void_p, ctypes.c_uint32] + [ctypes.c_void_p] * 7
        lib.stc_read_block.restype = ctypes.c_int
        lib.stc_compact.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_float)]
        lib.stc_compact.restype = ctypes.c_int
        lib.stc_set_step_slices.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        lib.stc_set_step_slices.restype = ctypes.c_int
        lib.stc_query_batch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                        ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
        lib.stc_query_batch.restype = ctypes.c_int
        lib.stc_get_config.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Config)]
        lib.stc_get_config.restype = ctypes.c_int
        lib.stc_checkpoint.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        lib.stc_checkpoint.restype = ctypes.c_int
        lib.stc_restore.argtypes = [ctypes.c_char_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p)]
        lib.stc_restore.restype = ctypes.c_int
        for fn in ("stc_write_ctb", "stc_load_ctb"):
            getattr(lib, fn).argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_char_p]
            getattr(lib, fn).restype = ctypes.c_int
        lib.stc_query_object.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        lib.stc_query_object.restype = ctypes.c_int
        lib.stc_query_box.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        lib.stc_query_box.restype = ctypes.c_int
        lib._stc_typed = True
    return lib


class Pipeline:
    """One GPU-resident co-occurrence pipeline (an stc_ctx)."""

    def __init__(self, cfg: StcConfig, mbr, xy0: np.ndarray):
        self.cfg = cfg.resolved()
        self._lib = _lib()
        self._c = config_struct(self.cfg)
        self._mbr = np.ascontiguousarray(mbr, dtype=np.float64)
        xy0 = np.ascontiguousarray(xy0, dtype=np.float64)
        h = ctypes.c_void_p()
        st = self._lib.stc_create(ctypes.byref(self._c), self._mbr.ctypes.data, xy0.ctypes.data,
                                  xy0.shape[0], ctypes.byref(h))
        if st != 0:
            raise StcError(st, self._lib.stc_last_error(h).decode())
        self._h = h

    def _check(self, st: int):
        if st != 0:
            raise StcError(st, self._lib.stc_last_error(self._h).decode())

    def step(self, xy: np.ndarray, t: int) -> None:
        xy = np.ascontiguousarray(xy, dtype=np.float64)
        assert xy.shape == (self.cfg.num_objects, 2)
        self._check(self._lib.stc_step(self._h, xy.ctypes.data, t))

    def step_device(self, xy_device_ptr: int, t: int) -> None:
        self._check(self._lib.stc_step_device(self._h, ctypes.c_void_p(xy_device_ptr), t))

    def step_window(self, xy, t0: int, out: np.ndarray | None = None) -> np.ndarray | None:
        """Steps t0 .. t0 + len(xy) - 1 as one pipelined window
        (stc_step_window: step i + 1 queued before step i's state is read). xy: a (steps, num_objects, 2) float64 numpy array
        in host memory, or (device pointer, steps) of that layout in device
        memory. With `out` (a MEETING_DTYPE array) each step's meetings are
        drained into it and the filled part is returned."""
        n = ctypes.c_size_t(0)
        optr, cap = (out.ctypes.data, len(out)) if out is not None else (None, 0)
        if isinstance(xy, tuple):
            ptr, steps = xy
            st = self._lib.stc_step_window(self._h, ctypes.c_void_p(ptr), 1, steps, t0, optr, cap, ctypes.byref(n))
        else:
            xy = np.ascontiguousarray(xy, dtype=np.float64)
            assert xy.ndim == 3 and xy.shape[1:] == (self.cfg.num_objects, 2)
            st = self._lib.stc_step_window(self._h, xy.ctypes.data, 0, xy.shape[0], t0, optr, cap, ctypes.byref(n))
        self._check(st)
        return out[:n.value] if out is not None else None

    def stats(self) -> StcStats:
        s = StcStats()
        self._check(self._lib.stc_get_stats(self._h, ctypes.byref(s)))
        return s

    def drain_some(self, out: np.ndarray) -> np.ndarray:
        """Up to len(out) pending meetings (stc_drain_meetings) into `out`, a
        MEETING_DTYPE array; the rest stays pending. Returns the filled part."""
        assert out.dtype == MEETING_DTYPE and out.flags.c_contiguous
        n = ctypes.c_size_t()
        self._check(self._lib.stc_drain_meetings(self._h, out.ctypes.data, len(out), ctypes.byref(n)))
        return out[: n.value]

    def drain(self, out: np.ndarray | None = None) -> np.ndarray:
        """The meetings emitted since the last drain (stc_drain_meetings).
        One buffer sized to the pending count receives them; the copy runs
        in the library without the interpreter lock, so threads that query
        meanwhile are not held up. `out`, a MEETING_DTYPE array (best in
        page-locked memory, which the library fills by direct DMA), is
        reused when it can hold them all; the result is then a view of it."""
        if out is not None:
            assert out.dtype == MEETING_DTYPE and out.flags.c_contiguous
            if int(self.stats().pending) <= len(out):
                n = ctypes.c_size_t()
                self._check(self._lib.stc_drain_meetings(self._h, out.ctypes.data, len(out), ctypes.byref(n)))
                return out[: n.value]
        out = []
        while True:
            cap = max(int(self.stats().pending), 1)
            buf = np.empty(cap, dtype=MEETING_DTYPE)
            n = ctypes.c_size_t()
            self._check(self._lib.stc_drain_meetings(self._h, buf.ctypes.data, cap, ctypes.byref(n)))
            out.append(buf[: n.value])
            if n.value < cap or n.value == 0 or self.stats().pending == 0:
                break
        return out[0] if len(out) == 1 else np.concatenate(out)

    def flush(self) -> bool:
        """Flushes the memtable into a block now; False if it was empty."""
        f = ctypes.c_int()
        self._check(self._lib.stc_flush(self._h, ctypes.byref(f)))
        return bool(f.value)

    def ctb_info(self) -> StcCtbInfo:
        info = StcCtbInfo()
        self._check(self._lib.stc_get_ctb(self._h, ctypes.byref(info)))
        return info

    def read_ctb(self) -> tuple:
        """(info, dict of host arrays) of the last flushed block."""
        info = self.ctb_info()
        b = ctb_buffers(info, self.cfg.num_objects)
        self._check(self._lib.stc_read_ctb(self._h, *[b[k].ctypes.data for k in (
            "ctfs", "bitmaps", "keys", "sids", "oversize_keys", "oversize_boxes", "oversize_bitmap")]))
        return info, ctb_trim(info, b)

    def block_info(self, index: int) -> StcCtbInfo:
        """Description of retained block `index`."""
        info = StcCtbInfo()
        self._check(self._lib.stc_get_block(self._h, index, ctypes.byref(info)))
        return info

    def read_block(self, index: int) -> tuple:
        """(info, dict of host arrays) of retained block `index`."""
        info = self.block_info(index)
        b = ctb_buffers(info, self.cfg.num_objects)
        self._check(self._lib.stc_read_block(self._h, index, *[b[k].ctypes.data for k in (
            "ctfs", "bitmaps", "keys", "sids", "oversize_keys", "oversize_boxes", "oversize_bitmap")]))
        return info, ctb_trim(info, b)

    def set_step_slices(self, slices: int) -> None:
        """Launches per long step kernel from the next step on (stc_set_step_slices)."""
        self._check(self._lib.stc_set_step_slices(self._h, slices))

    def compact(self, first_index: int, count: int, split: int) -> tuple:
        """Merges retained block first_index and the count - 1 after it into
        one block of split * split CTFs; returns (its index, device ms)."""
        idx = ctypes.c_uint32()
        ms = ctypes.c_float()
        self._check(self._lib.stc_compact(self._h, first_index, count, split, ctypes.byref(idx), ctypes.byref(ms)))
        return int(idx.value), float(ms.value)

    def query_batch(self, queries: np.ndarray, with_counts: bool = False):
        """Runs a batch (QUERY_DTYPE array); returns a list of CONTACT_DTYPE
        arrays (and the per-query match counts when with_counts)."""
        q = np.ascontiguousarray(queries, dtype=QUERY_DTYPE)
        offs = np.zeros(len(q) + 1, np.uint64)
        counts = np.zeros(max(len(q), 1), np.uint64)
        cap = 1 << 16
        while True:
            out = np.zeros(cap, CONTACT_DTYPE)
            st = self._lib.stc_query_batch(self._h, q.ctypes.data, len(q), out.ctypes.data, cap, offs.ctypes.data,
                                           counts.ctypes.data)
            if st != 0:
                raise StcError(st, self._lib.stc_last_error(None).decode())
            if int(offs[-1]) <= cap:
                res = [out[int(offs[i]):int(offs[i + 1])] for i in range(len(q))]
                return (res, counts[:len(q)]) if with_counts else res
            cap = int(offs[-1])

    def query_counts(self, queries: np.ndarray) -> np.ndarray:
        """Match counts only (STC_QUERY_COUNT_ONLY on every query)."""
        q = np.array(queries, dtype=QUERY_DTYPE, copy=True)
        q["kind"] |= QUERY_COUNT_ONLY
        return self.query_batch(q, with_counts=True)[1]

    def server(self, max_batch: int = 0, result_cap: int = 0, hbm_budget: int = 0) -> "Server":
        """A request loop answering queries by continuous batching (stc_server_start)."""
        srv = Server(self, max_batch, result_cap, hbm_budget)
        if not hasattr(self, "_servers"):
            self._servers = []
        self._servers.append(srv)
        return srv

    def checkpoint(self, path: str) -> None:
        """Writes the context's step-to-step state to one file (stc_checkpoint)."""
        self._check(self._lib.stc_checkpoint(self._h, path.encode()))

    @classmethod
    def restore(cls, path: str, device: int = 0) -> "Pipeline":
        """A pipeline continuing from a checkpoint file (stc_restore)."""
        lib = _lib()
        h = ctypes.c_void_p()
        st = lib.stc_restore(path.encode(), device, ctypes.byref(h))
        if st != 0:
            raise StcError(st, lib.stc_last_error(None).decode())
        c = _Config()
        lib.stc_get_config(h, ctypes.byref(c))
        p = cls.__new__(cls)
        p._lib, p._h, p._c = lib, h, c
        p.cfg = StcConfig(**{f.name: getattr(c, f.name) for f in fields(StcConfig)})
        return p

    def write_ctb(self, index: int, directory: str, prefix: str) -> None:
        """Writes retained block `index` as the reference's block files."""
        self._check(self._lib.stc_write_ctb(self._h, index, directory.encode(), prefix.encode()))

    def load_ctb(self, index: int, directory: str, prefix: str) -> None:
        """Reads block files into a retained block (queried like a flushed one)."""
        self._check(self._lib.stc_load_ctb(self._h, index, directory.encode(), prefix.encode()))

    def query_object(self, pid: int, t_start: int = 0, t_end: int = 0xFFFFFFFF) -> np.ndarray:
        q = np.zeros(1, QUERY_DTYPE)
        q["kind"], q["pid"], q["t_start"], q["t_end"] = QUERY_OBJECT, pid, t_start, t_end
        return self.query_batch(q)[0]

    def query_box(self, box, t_start: int = 0, t_end: int = 0xFFFFFFFF) -> np.ndarray:
        q = np.zeros(1, QUERY_DTYPE)
        q["kind"], q["t_start"], q["t_end"] = QUERY_BOX, t_start, t_end
        q["box"][0] = box
        return self.query_batch(q)[0]

    def close(self):
        for srv in list(getattr(self, "_servers", [])):
            srv.stop()  # a server must not outlive its context
        if getattr(self, "_h", None):
            self._lib.stc_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sort_meetings(m: np.ndarray) -> np.ndarray:
    """Canonical order for comparing meeting sets."""
    order = np.lexsort((m["end"], m["start"], m["pid_hi"], m["pid_lo"]))
    return m[order]


def meetings_digest(m: np.ndarray) -> str:
    """SHA-256 of the sorted tuple set (pid_lo, pid_hi, start, end, mbr bits)."""
    import hashlib
    s = sort_meetings(np.ascontiguousarray(m, dtype=MEETING_DTYPE))
    return hashlib.sha256(s.tobytes()).hexdigest()


class Server:
    """stc_server_*: queries submitted from any thread are answered by the
    library's two worker threads in batches admitted by device footprint
    (two batches may be on the GPU at once, each on its own stream); answers
    carry the latency from each query's arrival (seconds on the monotonic
    clock, as time.perf_counter on Linux)."""

    def __init__(self, pipe: "Pipeline", max_batch: int = 0, result_cap: int = 0, hbm_budget: int = 0):
        self._lib = pipe._lib
        self._pipe = pipe
        cfg = _ServerConfig(max_batch, result_cap, hbm_budget)
        h = ctypes.c_void_p()
        st = self._lib.stc_server_start(pipe._h, ctypes.byref(cfg), ctypes.byref(h))
        if st != 0:
            raise StcError(st, self._lib.stc_last_error(None).decode())
        self._h = h

    def submit(self, queries: np.ndarray, arrival: float = 0.0) -> int:
        """Queues the queries (QUERY_DTYPE); returns the first ticket."""
        q = np.ascontiguousarray(queries, dtype=QUERY_DTYPE)
        first = ctypes.c_uint64()
        st = self._lib.stc_server_submit(self._h, q.ctypes.data, len(q), float(arrival), ctypes.byref(first))
        if st != 0:
            raise StcError(st, "stc_server_submit")
        return int(first.value)

    def poll(self, cap: int = 65536, contacts_cap: int = 0, wait_ms: int = 0) -> tuple:
        """(answers, contacts) completed since the last poll (copies; the
        receiving buffers are kept between polls)."""
        if getattr(self, "_ans", None) is None or len(self._ans) < cap:
            self._ans = np.empty(cap, ANSWER_DTYPE)
        if getattr(self, "_con", None) is None or len(self._con) < max(contacts_cap, 1):
            self._con = np.empty(max(contacts_cap, 1), CONTACT_DTYPE)
        n = ctypes.c_size_t(0)
        st = self._lib.stc_server_poll(self._h, self._ans.ctypes.data, cap, self._con.ctypes.data, contacts_cap,
                                       ctypes.byref(n), int(wait_ms))
        if st != 0:
            raise StcError(st, "stc_server_poll")
        a = self._ans[: n.value].copy()
        used = int((a["contact_offset"] + a["stored"]).max()) if len(a) else 0
        return a, self._con[:used].copy()

    def stats(self) -> ServerStats:
        s = ServerStats()
        self._lib.stc_server_get_stats(self._h, ctypes.byref(s))
        return s

    def stop(self) -> None:
        """Answers everything queued and stops the serving thread."""
        if self._h:
            self._lib.stc_server_stop(self._h)
            self._h = None
            servers = getattr(self._pipe, "_servers", [])
            if self in servers:
                servers.remove(self)

