"""Fixtures at the benchmark's own scale, from the reference's CPU implementation.

Runs oracle/_ref/ref_driver -- the reference's unmodified single-threaded CPU
co-occurrence path (tracing/filter.cpp, refinement.cpp, meeting.cpp,
workbench.cpp), built by oracle/build_ref.sh -- on the benchmark workloads and
stores, per step, the number of emitted meetings, the number of checking
units and the SHA-256 of the sorted (pid_lo, pid_hi, start, end) tuples
(tests/golden/make_golden.py: tuples_digest). Only digests are kept: the
tuples themselves run to millions per step.

    python tests/golden/make_golden_scale.py [case ...]

Cases (tests/golden/scale_<case>.npz):
  uniform_10m         the benchmark's uniform-10M workload (10M objects on the
                      40 km street grid, seed 1, reach 10 m, minimum meeting
                      5 steps, leaf capacity 200, amplify 2, 2^28 table
                      slots): its first 12 steps
  hotspot_1m          the hotspot model (70% of objects in 1000 Zipf(1.1)
                      Gaussian hotspots, sigma 300 m) at 1M objects, the
                      benchmark's hotspot-1M workload (seed 1, amplify 8):
                      first 10 steps
  hotspot_100k_scaled the same hotspot model scaled down with its densities
                      kept: 1/100 of the objects, of the hotspots and of the
                      area (100k objects, 10 hotspots, 4 km box, 20x20
                      street grid so blocks stay 200 m, sigma 300 m): 25 steps

Each case runs in its own reference process; cases given on the command line
run in parallel.
"""
from __future__ import annotations

import multiprocessing
import os
import sys
import tempfile
import time
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

SCALE_CASES = {
    "uniform_10m": dict(trace=dict(kind="uniform", num_objects=10_000_000, seed=1), steps=12,
                        cfg=dict(reach_distance=10.0, min_meet_time=5, grid_capacity=200, grid_amplify=2.0,
                                 num_meeting_buckets=1 << 28)),
    "hotspot_1m": dict(trace=dict(kind="hotspot", num_objects=1_000_000, n_hotspots=1000, seed=1), steps=10,
                       cfg=dict(reach_distance=10.0, min_meet_time=5, grid_capacity=200, grid_amplify=8.0,
                                num_meeting_buckets=1 << 28)),
    "hotspot_100k_scaled": dict(trace=dict(kind="hotspot", num_objects=100_000, n_hotspots=10, box_m=4000.0,
                                           grid_n=20, seed=2), steps=25,
                                cfg=dict(reach_distance=10.0, min_meet_time=5, grid_capacity=200, grid_amplify=8.0,
                                         num_meeting_buckets=1 << 24)),
}


def fixture_path(name: str) -> str:
    return os.path.join(HERE, f"scale_{name}.npz")


def run_case(name: str) -> str:
    import oracle
    from golden.make_golden import make_trace, stc_config, trace_digest, tuples_digest
    case = SCALE_CASES[name]
    t0 = time.time()
    trace, mbr = make_trace(case)
    cfg = stc_config(case)
    with tempfile.TemporaryDirectory() as d:
        steps = oracle.run_reference_driver(trace, mbr, cfg.resolved(), d)
    counts = np.array([len(s["meetings"]) for s in steps], dtype=np.int64)
    units = np.array([s["units"] for s in steps], dtype=np.int64)
    digests = np.array([tuples_digest(s["meetings"]) for s in steps])
    np.savez_compressed(fixture_path(name), counts=counts, units=units, digests=digests,
                        trace_sha256=np.array(trace_digest(trace)), mbr=np.asarray(mbr))
    return f"{name}: {counts.sum()} meetings over {len(steps)} steps ({time.time() - t0:.0f} s)"


def main():
    import oracle
    import stcdb_gb300.build as b
    b.build_tracegen()
    oracle.build(reference=True)
    if not oracle.reference_available():
        raise SystemExit("reference harness not built (no reference checkout here)")
    names = sys.argv[1:] or list(SCALE_CASES)
    for n in names:
        if n not in SCALE_CASES:
            raise SystemExit(f"unknown case {n}; choose from {sorted(SCALE_CASES)}")
    with ProcessPoolExecutor(max_workers=len(names), mp_context=multiprocessing.get_context("spawn")) as ex:
        for msg in ex.map(run_case, names):
            print(msg, flush=True)


if __name__ == "__main__":
    main()
