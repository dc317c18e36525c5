"""Shared helpers for parity tests: run the CUDA pipeline and the oracle on
the same seeded trace and compare the emitted meeting sets step by step."""
from __future__ import annotations

import numpy as np

from stcdb_gb300.pipeline import MEETING_DTYPE, Pipeline, StcConfig, sort_meetings
from stcdb_gb300.tracegen import TraceGenerator


def trace_and_box(tcfg, steps, pad=100.0):
    g = TraceGenerator(tcfg)
    tr = g.steps(steps)
    return tr, g.map_box(pad)


def as_tuples(m: np.ndarray) -> np.ndarray:
    s = sort_meetings(np.ascontiguousarray(m, dtype=MEETING_DTYPE))
    return s


def describe_diff(a: np.ndarray, b: np.ndarray, limit=5) -> str:
    ka = {tuple(int(v) for v in (r["pid_lo"], r["pid_hi"], r["start"], r["end"])): r for r in a}
    kb = {tuple(int(v) for v in (r["pid_lo"], r["pid_hi"], r["start"], r["end"])): r for r in b}
    only_a = sorted(set(ka) - set(kb))[:limit]
    only_b = sorted(set(kb) - set(ka))[:limit]
    mbr_diff = [k for k in set(ka) & set(kb) if ka[k]["mbr"].tobytes() != kb[k]["mbr"].tobytes()][:limit]
    return f"only_gpu={only_a} only_oracle={only_b} mbr_diff={mbr_diff} (gpu {len(a)} vs oracle {len(b)})"


def run_pair(cfg: StcConfig, trace: np.ndarray, mbr, steps=None):
    """Yields (t, gpu_meetings, oracle_meetings, gpu_stats, oracle_stats) per step."""
    import oracle as orc
    T = trace.shape[0] if steps is None else steps
    pipe = Pipeline(cfg, mbr, trace[0])
    ref = orc.Oracle(cfg, mbr, trace[0])
    try:
        for t in range(T):
            pipe.step(trace[t], t)
            g = pipe.drain()
            o = ref.step(trace[t], t)
            yield t, as_tuples(g), as_tuples(o), pipe.stats(), ref.stats()
    finally:
        pipe.close()
        ref.close()
