"""Generates the golden fixtures from the reference's own CPU implementation.

Runs oracle/_ref/ref_driver -- the reference's unmodified CPU co-occurrence
path (tracing/filter.cpp, refinement.cpp, meeting.cpp, workbench.cpp,
step_merge.cpp) compiled by oracle/build_ref.sh, single-threaded -- on seeded
traces from stcdb_gb300.tracegen and stores per step the emitted meetings
(pid_lo, pid_hi, start, end) and the number of checking units. Only this
script needs the reference checkout; the fixtures it writes are committed.

    python tests/golden/make_golden.py

Fixtures (tests/golden/*.npz):
  c1_uniform_100k   the CPU-runnable configuration: 100,000 objects, 100
                    steps, 40 km street grid, reach 10 m, min meeting 5,
                    leaf capacity 200 -- every meeting tuple stored
  hotspot_30k       dense hotspots (30k objects, 3 km box, sigma 120 m),
                    leaf overflow (grid_amplify 1.2), loaded meeting table
                    (restarts across cleared slots), dynamic splits/merges:
                    per-step tuple count and SHA-256 of the sorted tuples
  uniform_20k_small 20k objects, 25 steps, every tuple stored
"""
from __future__ import annotations

import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = {
    "c1_uniform_100k": dict(trace=dict(kind="uniform", num_objects=100_000, seed=1), steps=100,
                            cfg=dict(reach_distance=10.0, min_meet_time=5, grid_capacity=200,
                                     num_meeting_buckets=800_000), full=True),
    "uniform_20k_small": dict(trace=dict(kind="uniform", num_objects=20_000, seed=3), steps=25,
                              cfg=dict(reach_distance=10.0, min_meet_time=5, grid_capacity=200,
                                       num_meeting_buckets=200_000), full=True),
    "hotspot_30k": dict(trace=dict(kind="hotspot", num_objects=30_000, n_hotspots=30, box_m=3000.0, grid_n=16,
                                   sigma_m=120.0, seed=11), steps=15,
                        cfg=dict(reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.2,
                                 num_meeting_buckets=1_500_000), full=False),
}


def trace_config(t):
    from stcdb_gb300.tracegen import hotspot_grid, uniform_grid
    t = dict(t)
    kind = t.pop("kind")
    return uniform_grid(**t) if kind == "uniform" else hotspot_grid(**t)


def make_trace(case):
    from stcdb_gb300.tracegen import TraceGenerator
    g = TraceGenerator(trace_config(case["trace"]))
    return g.steps(case["steps"]), g.map_box(100.0)


def stc_config(case):
    from stcdb_gb300.pipeline import StcConfig
    return StcConfig(num_objects=case["trace"]["num_objects"], **case["cfg"])


def tuples_digest(rows: np.ndarray) -> str:
    """SHA-256 of the (pid_lo, pid_hi, start, end) rows sorted lexicographically, as little-endian u32."""
    rows = np.asarray(rows, dtype=np.uint32).reshape(-1, 4)
    order = np.lexsort((rows[:, 3], rows[:, 2], rows[:, 1], rows[:, 0]))
    return hashlib.sha256(np.ascontiguousarray(rows[order]).astype("<u4").tobytes()).hexdigest()


def trace_digest(trace: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(trace, dtype="<f8").tobytes()).hexdigest()


def main():
    import oracle
    import stcdb_gb300.build as b
    b.build_tracegen()
    oracle.build(reference=True)
    if not oracle.reference_available():
        raise SystemExit("reference harness not built (no reference checkout here)")
    for name, case in CASES.items():
        trace, mbr = make_trace(case)
        cfg = stc_config(case)
        with tempfile.TemporaryDirectory() as d:
            steps = oracle.run_reference_driver(trace, mbr, cfg.resolved(), d)
        counts = np.array([len(s["meetings"]) for s in steps], dtype=np.int64)
        units = np.array([s["units"] for s in steps], dtype=np.int64)
        digests = np.array([tuples_digest(s["meetings"]) for s in steps])
        out = dict(counts=counts, units=units, digests=digests, trace_sha256=np.array(trace_digest(trace)),
                   mbr=np.asarray(mbr))
        if case["full"]:
            rows = np.concatenate([s["meetings"] for s in steps]) if counts.sum() else np.zeros((0, 4), np.uint32)
            out["rows"] = rows.astype(np.uint32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: {counts.sum()} meetings over {len(steps)} steps")


if __name__ == "__main__":
    main()
