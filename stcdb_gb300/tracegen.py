"""ctypes wrapper of the seeded grid-graph trace generator (csrc/tracegen.c).

The generator stands in for the reference's unseeded road-network trace
generator (tracing/generator.cpp:387-406); see csrc/tracegen.c for the model.
Presets follow the synthetic workloads the pipeline is measured on.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, replace

import numpy as np

from ._lib import load_library


class _Cfg(ctypes.Structure):
    _fields_ = [
        ("num_objects", ctypes.c_uint32),
        ("grid_n", ctypes.c_int32),
        ("box_m", ctypes.c_double),
        ("jitter_m", ctypes.c_double),
        ("speed_lo", ctypes.c_double),
        ("speed_hi", ctypes.c_double),
        ("n_hotspots", ctypes.c_int32),
        ("hot_frac", ctypes.c_double),
        ("sigma_m", ctypes.c_double),
        ("zipf_s", ctypes.c_double),
        ("seed", ctypes.c_uint64),
    ]


@dataclass(frozen=True)
class TraceConfig:
    num_objects: int
    grid_n: int = 200
    box_m: float = 40000.0
    jitter_m: float = 20.0
    speed_lo: float = 1.0
    speed_hi: float = 15.0
    n_hotspots: int = 0
    hot_frac: float = 0.0
    sigma_m: float = 300.0
    zipf_s: float = 1.1
    seed: int = 1

    def scaled(self, **kw) -> "TraceConfig":
        return replace(self, **kw)


def uniform_grid(num_objects: int = 100_000, seed: int = 1) -> TraceConfig:
    """100k objects on a 200x200 jittered grid graph over 40 km x 40 km."""
    return TraceConfig(num_objects=num_objects, seed=seed)


def hotspot_grid(num_objects: int = 10_000_000, n_hotspots: int = 1000, hot_frac: float = 0.7,
                 sigma_m: float = 300.0, seed: int = 1, grid_n: int = 200,
                 box_m: float = 40000.0) -> TraceConfig:
    """70% of objects from Zipf(1.1)-weighted Gaussian hotspots, 30% uniform."""
    return TraceConfig(num_objects=num_objects, n_hotspots=n_hotspots, hot_frac=hot_frac,
                       sigma_m=sigma_m, seed=seed, grid_n=grid_n, box_m=box_m)


def _lib():
    lib = load_library("libstctrace")
    if not getattr(lib, "_stc_typed", False):
        lib.stc_tracegen_create.restype = ctypes.c_void_p
        lib.stc_tracegen_create.argtypes = [ctypes.POINTER(_Cfg)]
        lib.stc_tracegen_destroy.argtypes = [ctypes.c_void_p]
        lib.stc_tracegen_next.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.stc_tracegen_next.restype = ctypes.c_int
        lib.stc_tracegen_map_box.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
        lib._stc_typed = True
    return lib


class TraceGenerator:
    """Yields (N, 2) float64 lon/lat arrays, one per second."""

    def __init__(self, cfg: TraceConfig):
        self.cfg = cfg
        c = _Cfg(cfg.num_objects, cfg.grid_n, cfg.box_m, cfg.jitter_m, cfg.speed_lo, cfg.speed_hi,
                 cfg.n_hotspots, cfg.hot_frac, cfg.sigma_m, cfg.zipf_s, cfg.seed)
        self._lib = _lib()
        self._h = self._lib.stc_tracegen_create(ctypes.byref(c))
        if not self._h:
            raise ValueError(f"invalid trace configuration {cfg}")

    def map_box(self, pad_m: float = 100.0) -> np.ndarray:
        out = np.zeros(4, dtype=np.float64)
        self._lib.stc_tracegen_map_box(self._h, pad_m, out.ctypes.data)
        return out

    def next(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.cfg.num_objects, 2), dtype=np.float64)
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == 2 * self.cfg.num_objects
        if self._lib.stc_tracegen_next(self._h, out.ctypes.data) != 0:
            raise RuntimeError("trace generator failed")
        return out

    def steps(self, count: int) -> np.ndarray:
        out = np.empty((count, self.cfg.num_objects, 2), dtype=np.float64)
        for t in range(count):
            self.next(out[t])
        return out

    def close(self):
        if self._h:
            self._lib.stc_tracegen_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _dev_lib():
    lib = load_library("libstc")
    if not getattr(lib, "_stc_trace_typed", False):
        lib.stc_trace_dev_create.restype = ctypes.c_int
        lib.stc_trace_dev_create.argtypes = [ctypes.POINTER(_Cfg), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        lib.stc_trace_dev_next.restype = ctypes.c_int
        lib.stc_trace_dev_next.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
        lib.stc_trace_dev_step.restype = ctypes.c_uint32
        lib.stc_trace_dev_step.argtypes = [ctypes.c_void_p]
        lib.stc_trace_dev_map_box.restype = ctypes.c_int
        lib.stc_trace_dev_map_box.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
        lib.stc_trace_dev_last_ms.restype = ctypes.c_float
        lib.stc_trace_dev_last_ms.argtypes = [ctypes.c_void_p]
        lib.stc_trace_dev_destroy.argtypes = [ctypes.c_void_p]
        lib._stc_trace_typed = True
    return lib


class DeviceTraceGenerator:
    """The same walker with its state in GPU memory (stc_trace_dev_* in
    libstc): writes steps straight into a device buffer, bit-identical to
    TraceGenerator's output for the same configuration."""

    def __init__(self, cfg: TraceConfig, device: int = 0):
        self.cfg = cfg
        c = _Cfg(cfg.num_objects, cfg.grid_n, cfg.box_m, cfg.jitter_m, cfg.speed_lo, cfg.speed_hi,
                 cfg.n_hotspots, cfg.hot_frac, cfg.sigma_m, cfg.zipf_s, cfg.seed)
        self._lib = _dev_lib()
        h = ctypes.c_void_p()
        st = self._lib.stc_trace_dev_create(ctypes.byref(c), device, ctypes.byref(h))
        if st != 0:
            raise ValueError(f"stc_trace_dev_create failed with status {st} for {cfg}")
        self._h = h.value

    def map_box(self, pad_m: float = 100.0) -> np.ndarray:
        out = np.zeros(4, dtype=np.float64)
        self._lib.stc_trace_dev_map_box(self._h, pad_m, out.ctypes.data)
        return out

    def next_into(self, xy_device_ptr: int, steps: int = 1) -> None:
        """Writes `steps` steps of (N, 2) f64 positions at the device address
        (16-byte aligned), step k at offset 16 * N * k bytes."""
        st = self._lib.stc_trace_dev_next(self._h, ctypes.c_void_p(xy_device_ptr), steps)
        if st != 0:
            raise RuntimeError(f"stc_trace_dev_next failed with status {st}")

    @property
    def step(self) -> int:
        return int(self._lib.stc_trace_dev_step(self._h))

    @property
    def last_ms(self) -> float:
        """Device time of the last next_into call."""
        return float(self._lib.stc_trace_dev_last_ms(self._h))

    def close(self):
        if self._h:
            self._lib.stc_trace_dev_destroy(self._h)
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
