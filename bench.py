"""Benchmark of the GB300 co-occurrence pipeline (one JSON line on rank 0).

A step is one time step of the hot path over all objects: partition, border
lookup, refinement, meeting-table insert, expire/emit sweep and quadtree
update (the reference's filter + reachability + update_meetings +
update_schema, tracing/process.cpp:452-459, 608-612).

Workload (default "uniform-10M"): 10,000,000 objects walking a seeded
200x200 jittered street grid over 40 km x 40 km at U[1,15] m/s, uniform
starts, reach 10 m, minimum meeting 5 steps, leaf capacity 200, 2^28 table
slots (about 68M pairs are live per step, so the reference default of 2N
slots would overflow). This is the pure-uniform window of the batching
configuration (1M-20M objects, 0-90% hotspot) at the headline 10M objects.
The 10M-object hotspot configuration (70% in 1000 Zipf hotspots, sigma
300 m) is out of reach of one GPU and of any reference check: its live pairs
grow with N^2 (measured 24.1M, 97.0M and 212.6M per step at 1M, 2M and 3M
objects, so about 2.4e9 at 10M). "hotspot-1M" (2M, 3M, 5M) runs that model
at those counts; "uniform-3M" is the default workload at 3M objects (a few
GB on the device, the case the kernel profiles are captured on).

value: position updates per second with positions already resident in HBM
  (stc_step_device), summed device time of K steps (CUDA events on the
  library's stream). Inputs (160 MB per step) and the meeting table exceed
  the 129 MB L2, so no flush is inserted between steps.
Every step also appends its emitted meetings to the memtable (two directed
  keys each, as the reference's GPU step does); the JSON's "flush" times one
  flush of everything gathered over the run into 100 CTFs.
e2e: the same metric through the public C ABI with host input: pipelined
  windows of 10 steps (stc_step_window), every step's positions read from
  pinned host memory by the step's descent (copied in by a copy engine while
  a request loop is attached) and its emitted meetings drained back to the
  host beside the next step; wall clock. "host_link" gives the copy rates of
  one step's positions and "windows" how busy the windows kept the GPU.
queries_under_ingest: 2K more steps (host input, pipelined windows of 4
  steps) while the library's serving workers answer a Poisson query stream
  (default 20,000/s) over the flushed block by continuous batching: 60%
  object queries returning their contacts, 40% box queries returning match
  counts, as the reference's searches do; p50/p99 latency from arrival.
queries_under_ingest_hbm_input: the same for 2K further steps whose
  positions are already in HBM (as for `value`), over the two blocks flushed
  by then: the serving's own cost to ingest, without the host link's.
batched: 64 uneven ingest windows (100k-2M objects log-uniform, a tenth of
  the batching configuration's 1M-20M, which --batched-full runs; 10-50
  steps, reach 5/10/20 m, 0-90% hotspot, lowered where the table would not fit) run
  as plain steps and as pipelined windows (stc_step_window) from fresh
  contexts: both rates, the speed-up and whether the two emitted the same
  meetings (--no-batched skips it and autotune).
autotune: stc_autotune on the hotspot-1M model: the leaf capacity and launch
  shape it picks and the device time per step before and after.
sort: the library's radix sort on 100M random 32-bit pairs.
table_random_access: the rate at which HBM serves random 32-byte slot reads,
  each with a store to its slot, over a table of the workload's size
  (stc_measure_random_access), one access per hit of a step, and the refine
  phase's hits per second against it: the table update's ceiling.
--impl reference: the oracle's C restatement of the reference CPU path with
  all host threads (the reference's own sources are not on the GPU host).
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pos-updates/s at 10M objs (bit-exact meetings); query p50/p99 under ingest"
UNIT = "pos-updates/s"

WORKLOADS = {
    # launch shape chosen by stc_autotune on 8 steps of this workload (4
    # pair-test and 32 table-update blocks per SM: 15.12 -> 14.80 ms a step);
    # it does not change results
    "uniform-10M": dict(objects=10_000_000, hot=0, reach=10.0, min_meet=5, grid_capacity=200, amplify=2.0,
                        buckets=1 << 28, kv_restriction=1 << 27, refine_bps=4, hits_bps=32),
    "hotspot-1M": dict(objects=1_000_000, hot=1000, reach=10.0, min_meet=5, grid_capacity=200, amplify=8.0,
                       buckets=1 << 28, kv_restriction=1 << 27),
    # the hotspot model at larger object counts (live pairs grow with N^2)
    # (the warm-up window holds its steps' meetings: emit buffers of 16 N)
    "hotspot-2M": dict(objects=2_000_000, hot=1000, reach=10.0, min_meet=5, grid_capacity=200, amplify=8.0,
                       buckets=1 << 29, kv_restriction=1 << 27, emit_per_object=16),
    "hotspot-3M": dict(objects=3_000_000, hot=1000, reach=10.0, min_meet=5, grid_capacity=200, amplify=8.0,
                       buckets=1 << 30, kv_restriction=1 << 27, emit_per_object=16),
    "hotspot-5M": dict(objects=5_000_000, hot=1000, reach=10.0, min_meet=5, grid_capacity=200, amplify=8.0,
                       buckets=1 << 31, kv_restriction=1 << 27, emit_per_object=16),
    # the stress configuration's model (90% of objects in 200 hotspots,
    # sigma 150 m, reach 20 m, minimum meeting 3 steps) at the largest object
    # count whose live pairs fit a table in HBM: its Zipf-weighted first
    # hotspot alone holds ~17% of the hot objects, so live pairs grow as N^2
    # (about 3e8 at 1M objects); its blocks carry 512 x 512 map bitmaps
    "stress-1M": dict(objects=1_000_000, hot=200, hot_frac=0.9, sigma_m=150.0, reach=20.0, min_meet=3,
                      grid_capacity=200, amplify=32.0, buckets=1 << 30, kv_restriction=1 << 27,
                      emit_per_object=128, bitmap_edge=512),
    # the same with blocks of 2^28 keys, four of which (about 2^30 keys, the
    # stress configuration's largest runs) are compacted at the end
    "stress-1M-lsm": dict(objects=1_000_000, hot=200, hot_frac=0.9, sigma_m=150.0, reach=20.0, min_meet=3,
                          grid_capacity=200, amplify=32.0, buckets=1 << 30, kv_restriction=1 << 28,
                          emit_per_object=128, bitmap_edge=512, compact_blocks=4),
    # the hotspot model at the headline's 10M objects: about 2.2e9 live pairs
    # a step (2^32 table slots, 137 GB; hit buffer of 2.5e9 records, 80 GB);
    # the memtable stays off to leave room (no flush, no queries)
    "hotspot-10M": dict(objects=10_000_000, hot=1000, reach=10.0, min_meet=5, grid_capacity=200, amplify=8.0,
                        buckets=1 << 32, kv_restriction=0, emit_per_object=16, hit_capacity=2_500_000_000),
    "uniform-3M": dict(objects=3_000_000, hot=0, reach=10.0, min_meet=5, grid_capacity=200, amplify=2.0,
                       buckets=1 << 26, kv_restriction=1 << 25),
    "uniform-100k": dict(objects=100_000, hot=0, reach=10.0, min_meet=5, grid_capacity=200, amplify=2.0,
                         buckets_per_object=8, kv_restriction=1 << 22),
}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_trace_cfg(w, seed):
    from stcdb_gb300.tracegen import hotspot_grid, uniform_grid
    if w["hot"]:
        return hotspot_grid(w["objects"], n_hotspots=w["hot"], seed=seed, hot_frac=w.get("hot_frac", 0.7),
                            sigma_m=w.get("sigma_m", 300.0))
    return uniform_grid(w["objects"], seed=seed)


def make_cfg(w, device=0, step_slices=0):
    from stcdb_gb300.pipeline import StcConfig
    b = w.get("buckets") or w["buckets_per_object"] * w["objects"]
    return StcConfig(num_objects=w["objects"], reach_distance=w["reach"], min_meet_time=w["min_meet"],
                     grid_capacity=w["grid_capacity"], grid_amplify=w["amplify"], num_meeting_buckets=b,
                     device=device, kv_restriction=w["kv_restriction"], step_slices=step_slices,
                     emit_capacity=w.get("emit_per_object", 0) * w["objects"],
                     refine_blocks_per_sm=w.get("refine_bps", 0), hits_blocks_per_sm=w.get("hits_bps", 0),
                     refine_chunk=w.get("refine_chunk", 0), bitmap_edge=w.get("bitmap_edge", 0), hit_capacity=w.get("hit_capacity", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


E2E_WINDOW = 10  # steps per stc_step_window call of the end-to-end run
SERVE_WINDOW = 4  # steps per stc_step_window call while the server answers queries


class HostSteps:
    """Host position steps first..first+len-1, indexed by step number."""

    def __init__(self, arr, first):
        self.arr, self.first = arr, first

    def __getitem__(self, t):
        return self.arr[t - self.first]


def run_gpu(args, w, rank, local):
    import torch
    from stcdb_gb300.pipeline import Pipeline
    from stcdb_gb300.tracegen import DeviceTraceGenerator

    torch.cuda.set_device(local)
    N = w["objects"]
    K, W = args.steps, args.warmup
    # positions come from the device trace generator (bit-identical to the
    # host generator): steps 0..W+K-1 stay in HBM for the device-resident
    # run, steps W+K..W+3K-1 go to pinned host memory for the end-to-end and
    # serving runs
    gen = DeviceTraceGenerator(make_trace_cfg(w, seed=1 + rank), local)
    mbr = gen.map_box(100.0)
    dev = torch.empty((W + K, N, 2), dtype=torch.float64, device=f"cuda:{local}")
    gen.next_into(dev.data_ptr(), W + K)
    gen_ms = gen.last_ms
    S = args.serve_steps if args.serve_steps > 0 else 2 * K
    host = torch.empty((K + S, N, 2), dtype=torch.float64, pin_memory=True)
    stage = torch.empty((K, N, 2), dtype=torch.float64, device=f"cuda:{local}")
    for lo in range(0, K + S, K):
        n = min(K, K + S - lo)
        gen.next_into(stage.data_ptr(), n)
        host[lo:lo + n].copy_(stage[:n])
    # S more steps kept in HBM: the second serving run ingests them without
    # the host link
    dev_serve = None
    if args.query_rate > 0 and w["kv_restriction"]:
        dev_serve = torch.empty((S, N, 2), dtype=torch.float64, device=f"cuda:{local}")
        gen.next_into(dev_serve.data_ptr(), S)
    gen.close()
    # the host link's copy rates for one step's positions (page-locked host
    # memory, CUDA events, best of three): the end-to-end rate cannot beat
    # the step's input copy
    link = {}
    for name, src, dst in (("h2d", host[0], stage[0]), ("d2h", stage[0], host[0])):
        best = None
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        link[name + "_gbs"] = 16.0 * N / (best / 1e3) / 1e9
    link["bytes"] = 16 * N
    # each end-to-end step's own input copy once, in order (the rate can
    # differ across the page-locked allocation)
    rates = []
    for k in range(K):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        stage[0].copy_(host[k], non_blocking=True)
        e1.record()
        e1.synchronize()
        rates.append(16.0 * N / (e0.elapsed_time(e1) / 1e3) / 1e9)
    link["h2d_gbs_e2e_steps"] = {"min": min(rates), "median": float(np.median(rates)), "max": max(rates)}
    del stage
    hnp = HostSteps(host.numpy(), W + K)
    torch.cuda.synchronize()
    trace_gen = {"steps": W + K, "ms": gen_ms, "ms_per_step": gen_ms / (W + K),
                 "positions_per_s": N * (W + K) / (gen_ms / 1e3),
                 "written_gb_s": 16.0 * N * (W + K) / (gen_ms / 1e3) / 1e9}
    cfg = make_cfg(w, device=local, step_slices=args.step_slices)
    pipe = Pipeline(cfg, mbr, dev[0].cpu().numpy())
    # warm-up steps (device-resident input), as one window: it also captures
    # the step graphs of both input buffers that the end-to-end windows replay
    checked = []  # every meeting drained from the device-resident steps, for the bit-exact check
    if W >= 2:
        pipe.step_window((dev.data_ptr(), W), 0)
        checked.append(pipe.drain())
    else:
        for t in range(W):
            pipe.step_device(dev[t].data_ptr(), t)
            checked.append(pipe.drain())
    stats = []
    clk = ClockSampler(local).__enter__()  # sampling before the first timed step
    time.sleep(0.2)
    barrier(args)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for t in range(W, W + K):
        pipe.step_device(dev[t].data_ptr(), t)
        stats.append(pipe.stats())
        checked.append(pipe.drain())
    torch.cuda.synchronize()
    wall_dev = time.perf_counter() - t0
    clk.__exit__(None, None, None)
    checked = np.concatenate([meeting_rows(m) for m in checked])
    units = {W + i: int(s.checking_units) for i, s in enumerate(stats)}
    barrier(args)
    dev_ms = sum(s.step_ms for s in stats)
    # end to end: host positions in, meetings out, through the C ABI, in
    # windows of up to E2E_WINDOW steps (stc_step_window: each step's
    # positions read from page-locked host memory by its descent, its
    # meetings drained after it); the meetings land in a reused page-locked
    # buffer, as a server would keep one
    from stcdb_gb300.pipeline import MEETING_DTYPE
    per_step = max(max(s.emitted for s in stats), 1)
    win = min(K, E2E_WINDOW)
    cap = max(int(per_step * win * 1.5) + 4096, 8 * N // 10)
    mbuf = torch.empty(cap * MEETING_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    mnp = mbuf.numpy().view(MEETING_DTYPE)
    e2e_stats = []
    d2h = 0
    barrier(args)
    torch.cuda.synchronize()
    # the clock sampler starts and stops outside the timed region (starting
    # nvidia-smi takes tens of milliseconds)
    e2e_clk = ClockSampler(local).__enter__()
    time.sleep(0.2)
    t1 = time.perf_counter()
    for c0 in range(0, K, win):
        n = min(win, K - c0)
        m = pipe.step_window(hnp.arr[c0:c0 + n], W + K + c0, out=mnp)
        d2h += m.nbytes + 128 * n
        e2e_stats.append(pipe.stats())
    torch.cuda.synchronize()
    wall_e2e = time.perf_counter() - t1
    e2e_clk.__exit__(None, None, None)
    e2e_busy = {"window_device_ms": [round(float(s.window_device_ms), 3) for s in e2e_stats],
                "window_input_wait_ms": [round(float(s.window_input_wait_ms), 3) for s in e2e_stats],
                "window_copy_ms": [round(float(s.window_copy_ms), 3) for s in e2e_stats],
                "window_wall_ms": [round(float(s.window_wall_ms), 3) for s in e2e_stats],
                "clocks": e2e_clk.summary(),
                "gpu_busy_frac": float(sum(s.window_device_ms for s in e2e_stats) /
                                       max(sum(s.window_wall_ms for s in e2e_stats), 1e-9)),
                "host_load_avg": list(os.getloadavg()), "host_cpus": os.cpu_count()}
    # one flush of everything the memtable gathered (W + 2K steps)
    lsm = bool(w["kv_restriction"])  # a workload may run without the memtable (and its queries)
    flush = None
    if lsm:
        keys = pipe.stats().memtable_keys
        pipe.flush()
        fs = pipe.stats()
        info = pipe.ctb_info()
        flush = dict(keys=int(keys), ms=float(fs.flush_ms), ctf_keys=int(info.ctf_kv_count),
                     oversize_keys=int(info.oversize_kv_count), key_bytes=int(info.key_bytes),
                     ctfs=int(info.ctf_count), steps=W + 2 * K,
                     stages_ms=dict(zip(FLUSH_STAGES, (float(x) for x in fs.flush_stage_ms))))
    # queries under ingest: K more steps while a serving thread answers a
    # Poisson query stream over the flushed block
    queries = queries_hbm = None
    if args.query_rate > 0 and lsm:
        queries = serve_under_ingest(args, pipe, hnp, W + 2 * K, S, N, mbr, mnp)
        # the same with the ingest's positions already in HBM (the input
        # `value` is measured with), over the two blocks flushed by then
        pipe.flush()
        queries_hbm = serve_under_ingest(args, pipe, hnp, W + 2 * K + S, S, N, mbr, mnp, dev_serve)
        del dev_serve
    # compaction: the last `compact_blocks` (2) blocks flushed merge into one
    # block of split x split CTFs (100 CTFs, as a flush makes)
    compaction = None
    if lsm:
        pipe.flush()
    m = w.get("compact_blocks", 2)
    last = int(pipe.stats().flushes) - 1  # no block merged yet: block i is the i-th flush
    if lsm and last + 1 >= m:
        first = last - m + 1
        keys_in = sum(int(pipe.block_info(first + j).kv_count) for j in range(m))
        try:
            new, cms = pipe.compact(first, m, 10)
            out = pipe.block_info(new)
            compaction = dict(blocks=m, keys=keys_in, split=10, ms=cms, keys_per_s=keys_in / (cms / 1e3),
                              out_ctf_keys=int(out.ctf_kv_count), out_oversize_keys=int(out.oversize_kv_count),
                              stages_ms=dict(zip(COMPACT_STAGES,
                                                 (float(x) for x in pipe.stats().compact_stage_ms))))
        except Exception as e:  # noqa: BLE001 - e.g. no room for the merge; reported in the line
            compaction = dict(blocks=m, keys=keys_in, error=str(e))
    pipe.close()
    return dict(stats=stats, dev_ms=dev_ms, wall_dev=wall_dev, wall_e2e=wall_e2e, e2e_stats=e2e_stats, link=link,
                e2e_busy=e2e_busy,
                d2h=d2h, clocks=clk.summary(), flush=flush, queries=queries, queries_hbm=queries_hbm,
                trace_gen=trace_gen,
                compaction=compaction, bit_exact=bit_exact_check(args.workload, rank, checked, units, W + K))


def meeting_rows(m):
    """(pid_lo, pid_hi, start, end) rows of drained meetings."""
    if not len(m):
        return np.zeros((0, 4), np.uint32)
    return np.stack([m["pid_lo"], m["pid_hi"], m["start"], m["end"]], 1).astype(np.uint32)


# fixtures made by the reference's own single-threaded CPU path on the
# workloads' first steps (tests/golden/make_golden_scale.py)
SCALE_FIXTURES = {"uniform-10M": "scale_uniform_10m.npz", "hotspot-1M": "scale_hotspot_1m.npz"}


def bit_exact_check(workload, rank, rows, units, steps_run):
    """Compares the meetings the run emitted in its first steps with the
    reference's: per step the SHA-256 of the sorted tuples, their count and
    the checking units (known for the individually timed steps). A meeting
    is emitted at the first step after its end, so the drained rows split
    into steps by end + 1."""
    import hashlib
    name = SCALE_FIXTURES.get(workload)
    path = os.path.join(ROOT, "tests", "golden", name) if name else None
    if rank != 0 or not path or not os.path.exists(path):
        return None
    fx = np.load(path)
    n = min(len(fx["counts"]), steps_run)
    step_of = rows[:, 3].astype(np.int64) + 1
    mismatched = []
    for t in range(n):
        r = rows[step_of == t]
        r = r[np.lexsort((r[:, 3], r[:, 2], r[:, 1], r[:, 0]))] if len(r) else r
        ok = len(r) == int(fx["counts"][t]) and \
            hashlib.sha256(np.ascontiguousarray(r).astype("<u4").tobytes()).hexdigest() == str(fx["digests"][t])
        if t in units and units[t] != int(fx["units"][t]):
            ok = False
        if not ok:
            mismatched.append(t)
    return {"bit_exact": not mismatched, "steps_compared": n, "mismatched_steps": mismatched,
            "meetings_compared": int(np.asarray(fx["counts"][:n]).sum()), "units_compared": sorted(t for t in units if t < n),
            "fixture": "tests/golden/" + name,
            "reference": "the reference's own CPU path (tracing/filter.cpp, refinement.cpp, meeting.cpp), "
                         "single thread, same seeded positions"}


def make_queries(rng, n, N, mbr, t_now):
    """The query mix of the serving configuration: 60% object queries
    (uniform object, window log-uniform 10-10,000 steps), 40% box queries
    (side log-uniform 50 m-5 km at a uniform centre, window 10-3600 steps)."""
    import math
    from stcdb_gb300.pipeline import QUERY_BOX, QUERY_DTYPE, QUERY_OBJECT
    dpm_lat = 360.0 / 40076000.0  # degrees per metre of latitude
    lat = abs(float((mbr[1] + mbr[3]) / 2))
    dpm_lon = 360.0 / (math.sin((90 - lat) * math.pi / 180) * 40076000.0)
    q = np.zeros(n, QUERY_DTYPE)
    obj = rng.random(n) < 0.6
    q["kind"] = np.where(obj, QUERY_OBJECT, QUERY_BOX)
    q["pid"] = rng.integers(0, N, n)
    win = np.where(obj, 10 ** rng.uniform(1, 4, n), 10 ** rng.uniform(1, np.log10(3600), n)).astype(np.int64)
    q["t_end"] = t_now + 1
    q["t_start"] = np.maximum(t_now + 1 - win, 0)
    side_m = 10 ** rng.uniform(np.log10(50), np.log10(5000), n)
    cx = mbr[0] + rng.random(n) * (mbr[2] - mbr[0])
    cy = mbr[1] + rng.random(n) * (mbr[3] - mbr[1])
    hx, hy = side_m / 2 * dpm_lon, side_m / 2 * dpm_lat
    q["box"] = np.stack([cx - hx, cy - hy, cx + hx, cy + hy], 1)
    return q


def serve_under_ingest(args, pipe, hnp, t0, steps, N, mbr, mout=None, dev_steps=None):
    """Queries arrive as a Poisson stream and go to the library's request loop
    (stc_server_*), which answers them by continuous batching (whatever has
    arrived while a batch ran forms the next batch, admitted by device
    footprint). Latency = answer time - arrival time, both on the monotonic
    clock. The main thread keeps stepping meanwhile (host input). Object
    queries return their contacts (who met the object, up to result_cap
    each); box queries return match counts, as the reference's searches do."""
    from stcdb_gb300.pipeline import QUERY_BOX, QUERY_COUNT_ONLY
    rng = np.random.default_rng(12345)
    result_cap = 4096
    rate = float(args.query_rate)
    answers = []
    lags = []  # submit time - arrival time per query (the submitting thread's delay)
    arrived = {}  # ticket -> arrival time
    cur_t = [t0 - 1]
    done = threading.Event()
    errors = []
    srv = pipe.server(max_batch=4096, result_cap=result_cap, hbm_budget=64 << 20)
    stored = [0]  # contacts returned to the bench

    def take(cap, wait_ms):
        a, c = srv.poll(cap=cap, contacts_cap=1 << 20, wait_ms=wait_ms)
        if len(a):
            answers.append(a)
            stored[0] += int(a["stored"].sum())

    def server():
        next_arrival = time.perf_counter() + rng.exponential(1.0 / rate)
        while not done.is_set():
            now = time.perf_counter()
            arrivals = []
            while next_arrival <= now:
                arrivals.append(next_arrival)
                next_arrival += rng.exponential(1.0 / rate)
            if not arrivals:
                take(8192, 0)
                time.sleep(min(max(next_arrival - time.perf_counter(), 0.0), 0.0005))
                continue
            qs = make_queries(rng, len(arrivals), N, mbr, cur_t[0])
            qs["kind"] = np.where(qs["kind"] == QUERY_BOX, QUERY_BOX | QUERY_COUNT_ONLY, qs["kind"])
            try:
                for q, t_arr in zip(qs, arrivals):
                    arrived[srv.submit(q[None], arrival=t_arr)] = t_arr
                    lags.append(time.perf_counter() - t_arr)
            except Exception as e:  # noqa: BLE001 - reported in the JSON line
                errors.append(str(e))
                return

    th = threading.Thread(target=server, daemon=True)
    pipe.set_step_slices(args.serve_slices)  # query kernels get the GPU between slices
    gc.collect()
    gc.disable()  # no collector pause holds the interpreter lock while serving
    th.start()
    step_ms = []
    win_ms = []  # (device ms, input wait ms, steps) of each ingest window
    w0 = time.perf_counter()
    # ingest as pipelined windows (stc_step_window, host input, meetings
    # drained into the page-locked buffer), as the end-to-end run does
    for w0t in range(t0, t0 + steps, SERVE_WINDOW):
        n = min(SERVE_WINDOW, t0 + steps - w0t)
        if dev_steps is not None:  # positions already in HBM (no host link traffic)
            pipe.step_window((dev_steps[w0t - t0].data_ptr(), n), w0t, out=mout)
        else:
            pipe.step_window(hnp.arr[w0t - hnp.first:w0t - hnp.first + n], w0t, out=mout)
        ws = pipe.stats()
        step_ms.append(ws.step_ms)
        win_ms.append((ws.window_device_ms, ws.window_input_wait_ms, n, ws.window_copy_ms))
        cur_t[0] = w0t + n - 1
    wall = time.perf_counter() - w0
    done.set()
    th.join()
    # the rest of what was submitted, then the loop's statistics
    deadline = time.perf_counter() + 30.0
    while sum(len(a) for a in answers) < srv.stats().submitted and time.perf_counter() < deadline:
        take(65536, 100)
    sst = srv.stats()
    srv.stop()
    gc.enable()
    pipe.set_step_slices(args.step_slices)
    if errors:
        return {"error": errors[0]}
    ans = np.concatenate(answers) if answers else np.zeros(0)
    # an object query with more than result_cap contacts is answered with its
    # count and STC_ERR_CAPACITY; any other status is a failure
    over_cap = int((ans["status"] == 3).sum()) if len(ans) else 0
    if len(ans) and ((ans["status"] != 0) & (ans["status"] != 3)).any():
        return {"error": f"{int(((ans['status'] != 0) & (ans['status'] != 3)).sum())} queries failed"}
    lat_ms = ans["latency_ms"] if len(ans) else np.zeros(0)
    sizes = np.bincount(ans["batch"]) if len(ans) else np.zeros(0)
    # where the slowest answers come from: their batch (size, latency spread:
    # a small minimum means its queries waited before the batch started)
    # and the batch before it: its completion time (arrival + latency, one
    # clock) and its own latency spread; a batch runs at most its minimum
    # latency, so a long gap with a short run means the queries queued behind
    # the previous batch
    worst = {}
    if len(ans):
        wb = int(ans["batch"][int(np.argmax(lat_ms))])
        wl = lat_ms[ans["batch"] == wb]
        worst = {"batch_queries": int(len(wl)), "min_latency_ms": float(wl.min()),
                 "max_latency_ms": float(wl.max())}
        done_at = np.array([arrived.get(int(tk), np.nan) for tk in ans["ticket"]]) + lat_ms * 1e-3
        prev = ans["batch"] == (wb - 1 if wb > 0 else wb)
        if wb > 0 and prev.any():
            worst["since_previous_batch_ms"] = float((np.nanmax(done_at[ans["batch"] == wb]) -
                                                      np.nanmax(done_at[prev])) * 1e3)
            worst["previous_batch_queries"] = int(prev.sum())
            worst["previous_min_latency_ms"] = float(lat_ms[prev].min())
    lag_ms = np.asarray(lags) * 1e3
    return {"rate_target_per_s": rate, "answered": len(ans), "qps": len(ans) / wall,
            "p50_ms": float(np.percentile(lat_ms, 50)) if len(ans) else None,
            "p99_ms": float(np.percentile(lat_ms, 99)) if len(ans) else None,
            "p999_ms": float(np.percentile(lat_ms, 99.9)) if len(ans) else None,
            "max_ms": float(lat_ms.max()) if len(ans) else None,
            "mean_batch": float(sizes[sizes > 0].mean()) if len(ans) else 0.0, "batches": int(sst.batches),
            "slowest_batch": worst,
            "submit_lag_ms": {"p99": float(np.percentile(lag_ms, 99)) if len(lag_ms) else None,
                              "max": float(lag_ms.max()) if len(lag_ms) else None},
            "matches_per_query": float(ans["count"].mean()) if len(ans) else 0.0,
            "contacts_returned": stored[0], "object_queries_over_result_cap": over_cap,
            "server": {"loop": "stc_server (two library worker threads, continuous batching, two query "
                               "streams)", "max_batch": 4096, "result_cap": result_cap,
                       "hbm_budget_bytes": 64 << 20, "max_batch_queries": int(sst.max_batch_queries),
                       "max_batch_bytes": int(sst.max_batch_bytes), "budget_cuts": int(sst.budget_cuts),
                       "overlapped_batches": int(sst.overlapped_batches),
                       "slowest_batch_wall_ms": sst.slowest_batch_wall_us / 1e3,
                       "slowest_batch_gpu_ms": sst.slowest_batch_gpu_us / 1e3},
            "mix": "60% object queries returning contacts (meets-whom, window 10-10000 steps), 40% box "
                   "queries returning match counts (50 m-5 km, window 10-3600 steps)",
            "blocks": int(pipe.stats().flushes), "input": "HBM" if dev_steps is not None else "host (page-locked)",
            "step_slices": args.serve_slices, "ingest_window_steps": SERVE_WINDOW,
            "ingest_pos_updates_per_s": N * steps / wall,
            "ingest_device_ms_per_step": float(np.mean(step_ms)),
            "ingest_window_device_ms_per_step": sum(x[0] for x in win_ms) / max(sum(x[2] for x in win_ms), 1),
            "ingest_input_wait_ms_per_step": sum(x[1] for x in win_ms) / max(sum(x[2] for x in win_ms), 1),
            "ingest_input_copy_ms_per_step": sum(x[3] for x in win_ms) / max(sum(x[2] for x in win_ms), 1)}


def barrier(args):
    if args.world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(args, v):
    if args.world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# DRAM bytes (read + write) of the refinement phase (k_refine_a + k_hits)
# per hit, from one ncu capture of each kernel on the 3M-object workload
# (profiles/kernels_refine_hits_strips_uniform-3M.md): 388.5 MB (reads and
# writes of both kernels) for one of the step's four parts, about a quarter
# of its 6.086M hits. The traffic grows with the hits (32-byte records
# written and read, one table slot per hit), so the 10M line scales it by
# its own hit count.
REFINE_DRAM_BYTES_PER_HIT = (54.36e6 + 33.70e6 + 264.20e6 + 36.23e6) / (6.086e6 / 4)


def kernel_bytes(s, N, B, prev_live=None):
    """Algorithmic bytes per launch of the step's kernels.
    partition: 36 N (read positions, write leaf-ordered points, id map)
    refine:    16 N + 16 H + 8 Q plus the fused probe, 64 B per hit
    sweep:     32 B per table slot read, 32 B per slot it writes (each new
               meeting's claim finalised, each meeting not hit this step
               cleared) + 64 B per emitted meeting. A meeting stays live only
               when hit, so the cleared ones are the previous step's live
               meetings less this step's extensions (hits - new);
               `prev_live` defaults to this step's live count."""
    H, Q = s.border_units, s.hits
    new = s.new_candidates
    prev = s.taken_buckets if prev_live is None else prev_live
    cleared = max(prev - (Q - new), 0)
    return {"partition": 36.0 * N, "refine": 16.0 * N + 16.0 * H + 72.0 * Q,
            "sweep": 32.0 * B + 32.0 * (new + cleared) + 64.0 * s.emitted}


FLUSH_STAGES = ("object_order", "key_sort", "ctf_limits", "encode", "store_and_index")


def flush_line(f, peak):
    """One memtable flush: algorithmic bytes 64 per key (key + box read and
    written once) plus the packed keys and the bitmap slots written. Its
    stages (stc_stats.flush_stage_ms): the object order (oversize cut, STR
    sorts, slabs, sids), the key sort, the per-CTF limits and metadata, the
    key encoding (each CTF key's record and box read once, 32 B, and its
    packed bytes written: `encode_gbs`) and the block's store with its query
    index."""
    if not f or not f["keys"]:
        return dict(f) if f else None
    ab = 64.0 * f["keys"] + f["key_bytes"] + 8192.0 * (f["ctfs"] + 1)
    gbs = ab / (f["ms"] / 1e3) / 1e9
    out = dict(f, keys_per_s=f["keys"] / (f["ms"] / 1e3), algorithmic_bytes=ab, achieved_gbs=gbs,
               frac_of_peak=gbs / peak)
    st = f.get("stages_ms") or {}
    if st.get("encode", 0) > 0:
        eb = 32.0 * f["ctf_keys"] + f["key_bytes"]
        out["encode_gbs"] = eb / (st["encode"] / 1e3) / 1e9
        out["encode_frac_of_peak"] = out["encode_gbs"] / peak
    if st.get("key_sort", 0) > 0:
        out["key_sort_keys_per_s"] = f["keys"] / (st["key_sort"] / 1e3)
    return out


def sort_line(device, peak, n=100_000_000, reps=5):
    """The library's stable LSD radix sort (stc_sort_pairs_u32) on n random
    32-bit (key, value) pairs in HBM: 4 passes of 8 bits, each reading and
    writing every key and value once, 16 * 4 = 64 algorithmic bytes per pair.
    Device time of the passes only (the call's scratch allocation excluded)."""
    import ctypes
    import torch
    from stcdb_gb300._lib import load_library
    lib = load_library("libstc")
    lib.stc_sort_pairs_u32.restype = ctypes.c_int
    lib.stc_sort_pairs_u32.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32]
    lib.stc_last_sort_ms.restype = ctypes.c_float
    g = torch.Generator(device=f"cuda:{device}").manual_seed(3)
    k = torch.randint(0, 2 ** 31 - 1, (n,), dtype=torch.int32, device=f"cuda:{device}", generator=g)
    v = torch.arange(n, dtype=torch.int32, device=f"cuda:{device}")
    ko, vo = torch.empty_like(k), torch.empty_like(v)
    times = []
    for r in range(reps + 2):
        if lib.stc_sort_pairs_u32(k.data_ptr(), v.data_ptr(), ko.data_ptr(), vo.data_ptr(), n, 32, device) != 0:
            return {"error": "stc_sort_pairs_u32 failed"}
        if r >= 2:
            times.append(float(lib.stc_last_sort_ms()))
    ms = statistics.median(times)
    ok = bool(torch.all(ko[1:] >= ko[:-1]).item())
    b = 64.0 * n
    del k, v, ko, vo
    return {"pairs": n, "key_bits": 32, "ms": ms, "pairs_per_s": n / (ms / 1e3), "algorithmic_bytes": b,
            "achieved_gbs": b / (ms / 1e3) / 1e9, "frac_of_peak": b / (ms / 1e3) / 1e9 / peak, "sorted": ok}


def random_access_line(device, buckets, hits, refine_ms):
    """The meeting-table update's random-access ceiling: stc_measure_random_access
    on a table of the workload's size (2^round(log2 B) 32-byte slots, at most
    2^30) with as many accesses as the step has hits. Every hit reads its home
    slot, a random 32-byte sector of the table, and writes it (its end time
    or its claim); HBM serves such accesses at this rate, far below its copy
    bandwidth.
    `refine_frac` = the refine phase's hits per second (pair tests and table
    update together) / the ceiling: how close the phase is to one random slot
    access per hit at the measured rate."""
    import ctypes
    from stcdb_gb300._lib import load_library
    lib = load_library("libstc")
    f = lib.stc_measure_random_access
    f.argtypes = [ctypes.c_uint32, ctypes.c_ulonglong, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]
    f.restype = ctypes.c_int
    log2 = min(max(int(round(np.log2(max(buckets, 1024)))), 10), 30)
    n = max(int(hits), 1 << 20)
    ms = ctypes.c_float(0.0)
    if f(log2, n, device, ctypes.byref(ms)) != 0 or ms.value <= 0:
        return {"error": lib.stc_last_error(None).decode(errors="replace")}
    ceiling = n / (ms.value / 1e3)
    line = {"table_bytes": 32 << log2, "accesses": n, "ms": ms.value, "accesses_per_s": ceiling}
    if refine_ms > 0 and hits > 0:
        line["refine_hits_per_s"] = hits / (refine_ms / 1e3)
        line["refine_frac"] = line["refine_hits_per_s"] / ceiling
    return line


def _live_estimate(n, hot, reach):
    """Live meeting pairs per step of the grid-graph walker on the 40 km map:
    6.7 per object at 10M uniform objects and reach 10 m (measured), growing
    with the density (N) and the reach disc (reach^2); a hotspot share h
    multiplies it by 1 + 104 h^2 (3.5e7 live pairs measured at 1M objects
    with h = 0.7, against 6.7e5 uniform)."""
    return 6.7 * n * (n / 1e7) * (reach / 10.0) ** 2 * (1.0 + 104.0 * hot * hot)


def _meeting_checksum(buf, k, device):
    """(count, order-independent 64-bit checksum) of meetings buf[:k]:
    every 32-byte record hashed as four 64-bit words, the hashes summed with
    wrap-around, on the GPU."""
    import torch
    if k == 0:
        return 0, 0
    w = torch.from_numpy(np.ascontiguousarray(buf[:k]).view(np.int64).reshape(-1, 4)).to(f"cuda:{device}")
    c = torch.tensor([-7046029254386353131, -4658895280553007687, 7640891576956012809, -2398030916697513551],
                     dtype=torch.int64, device=w.device)
    h = w * c
    x = h[:, 0] ^ (h[:, 1] >> 17) ^ (h[:, 2] << 13) ^ (h[:, 3] >> 29)
    x = x * -7046029254386353131
    x = x ^ (x >> 31)
    return k, int(x.sum().item())


def _batched_run(mode, cfg, mbr, x0, xy, steps, n, buf, cap, device):
    """One window from a fresh context, as plain steps or as pipelined
    stc_step_window calls, its meetings drained into the page-locked `buf`
    (checksummed whenever half full). Returns ((count, checksum), rate, wall
    seconds over steps and drains, window calls, live meetings after the
    last step)."""
    import torch
    from stcdb_gb300.pipeline import Pipeline, StcError
    p = Pipeline(cfg, mbr, x0)
    cnt, chk, fill, elapsed, calls = 0, 0, 0, 0.0, 0

    def settle():
        nonlocal cnt, chk, fill
        a, b = _meeting_checksum(buf, fill, device)
        cnt, chk, fill = cnt + a, (chk + b) & 0xFFFFFFFFFFFFFFFF, 0

    try:
        torch.cuda.synchronize(device)
        if mode == "plain":
            for t in range(steps):
                t0 = time.perf_counter()
                p.step_device(xy[t].data_ptr(), t)
                while True:
                    fill += len(p.drain_some(buf[fill:]))
                    if not p.stats().pending:
                        break
                    elapsed += time.perf_counter() - t0
                    settle()
                    t0 = time.perf_counter()
                elapsed += time.perf_counter() - t0
                if fill > cap // 2:
                    settle()
        else:
            t = 0
            while t < steps:
                t0 = time.perf_counter()
                try:
                    fill += len(p.step_window((xy[t].data_ptr(), steps - t), t, buf[fill:]))
                    t = steps
                except StcError as e:
                    if e.status != 3:  # only a full output buffer is expected
                        raise
                    t = int(p.stats().step) + 1  # the steps that ran; their undrained meetings wait
                    fill = cap  # the call filled the buffer
                elapsed += time.perf_counter() - t0
                calls += 1
                if fill > cap // 2 or t < steps:
                    settle()
                    while p.stats().pending:
                        fill += len(p.drain_some(buf[fill:]))
                        settle()
        settle()
        live = int(p.stats().taken_buckets)
    finally:
        p.close()
    return (cnt, chk), n * steps / elapsed, elapsed, calls, live


def batched_line(device, windows=64, seed=7, live_cap=1.2e8, objects=(1e6, 2e7)):
    """Uneven ingest windows of the batching configuration: `windows` windows,
    each with a seeded object count log-uniform in `objects` (the
    configuration's 1M-20M; the default bench line runs them at a tenth,
    100k-2M, so that the line takes seconds), 10-50 steps, a
    reach from {5, 10, 20} m and a share of objects in the 1000-hotspot model
    uniform in 0-90%. Where a window's expected live pairs (_live_estimate)
    would exceed live_cap the hotspot share is lowered (and, for the largest
    windows, the reach), which the line reports per window: the full
    configuration at 20M objects, 90% in hotspots and 20 m holds ~10^11 live
    pairs, more than any table in HBM. Each window runs twice from fresh
    contexts with positions in HBM: as plain steps (stc_step_device and a
    drain per step; the host waits for every step) and as pipelined
    stc_step_window calls (step i + 1 queued before step i's state is read;
    steps of up to 2M objects replayed from captured graphs), both draining
    into one page-locked buffer. The two runs must emit the same meetings:
    their counts and order-independent checksums (_meeting_checksum) are
    compared. Times are wall-clock over the steps and drains, checksums
    excluded."""
    import torch
    from stcdb_gb300.pipeline import MEETING_DTYPE, StcConfig, StcError
    from stcdb_gb300.tracegen import DeviceTraceGenerator, hotspot_grid, uniform_grid
    rng = np.random.default_rng(seed)
    cap = 48_000_000
    pinned = torch.empty(cap * MEETING_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    buf = pinned.numpy().view(MEETING_DTYPE)
    per, same, pos, secs = [], True, 0, {"plain": 0.0, "window": 0.0}
    for w in range(windows):
        n = int(round(10 ** rng.uniform(np.log10(objects[0]), np.log10(objects[1]))))
        steps = int(rng.integers(10, 51))
        reach = float(rng.choice([5.0, 10.0, 20.0]))
        hot = float(rng.uniform(0.0, 0.9))
        want = (reach, hot)
        while _live_estimate(n, 0.0, reach) > live_cap and reach > 5.0:
            reach /= 2
        if _live_estimate(n, hot, reach) > live_cap:
            base = _live_estimate(n, 0.0, reach)
            hot = float(np.sqrt(max(live_cap / base - 1.0, 0.0) / 104.0))
        live = _live_estimate(n, hot, reach)
        # the estimate is rough (hotspot draws vary): 8 slots per expected
        # live pair keeps the load low even at several times the estimate
        B = 1 << max(24, int(np.ceil(np.log2(8.0 * live + 1))))
        tcfg = hotspot_grid(n, hot_frac=hot, seed=seed + w) if hot > 0.005 else uniform_grid(n, seed=seed + w)
        gen = DeviceTraceGenerator(tcfg, device)
        mbr = gen.map_box(100.0)
        xy = torch.empty((steps, n, 2), dtype=torch.float64, device=f"cuda:{device}")
        gen.next_into(xy.data_ptr(), steps)
        gen.close()
        cfg = StcConfig(num_objects=n, reach_distance=reach, min_meet_time=5, grid_capacity=200, grid_amplify=8.0,
                        num_meeting_buckets=B, emit_capacity=max(4 * n, int(0.25 * live) + (1 << 22)),
                        device=device)
        x0 = xy[0].cpu().numpy()
        sums, rate, dts, calls, live_seen = {}, {}, {}, 0, 0
        try:
            for mode in ("plain", "window"):
                sums[mode], rate[mode], dts[mode], c, live_seen = _batched_run(mode, cfg, mbr, x0, xy, steps, n,
                                                                               buf, cap, device)
                calls += c
        except StcError as e:
            # a window the library refuses (a table too small for its pairs)
            # is reported, not timed
            per.append({"objects": n, "steps": steps, "hot_frac": round(hot, 4), "reach_m": reach,
                        "table_slots": B, "error": str(e)})
            same = False
            del xy
            continue
        for mode in dts:
            secs[mode] += dts[mode]
        same &= sums["plain"] == sums["window"]
        pos += n * steps
        per.append({"objects": n, "steps": steps, "hot_frac": round(hot, 4), "reach_m": reach,
                    "drawn": {"reach_m": want[0], "hot_frac": round(want[1], 4)}, "table_slots": B,
                    "live_estimate": int(live), "live_meetings": live_seen,
                    "meetings": sums["plain"][0], "same": sums["plain"] == sums["window"],
                    "plain_pos_per_s": rate["plain"], "window_pos_per_s": rate["window"], "window_calls": calls})
        del xy
    if not pos:
        return {"windows": len(per), "error": "no window ran", "per_window": per}
    return {"windows": len(per), "objects_range": [int(objects[0]), int(objects[1])],
            "failed_windows": sum(1 for w in per if "error" in w),
            "plain_pos_per_s": pos / secs["plain"], "window_pos_per_s": pos / secs["window"],
            "speedup": secs["plain"] / secs["window"], "same_meetings": bool(same), "unit": "pos-updates/s",
            "per_window": per}


def tune_line(device, steps=8):
    """stc_autotune on the hotspot-1M model (1M objects, 70% in 1000 Zipf
    hotspots): leaf capacity among 64/128/256/512 (the workload's own 200 is
    the base) and the refinement launch shape, scored on device time per
    step."""
    import numpy as np
    from stcdb_gb300.pipeline import autotune
    from stcdb_gb300.tracegen import TraceGenerator
    w = WORKLOADS["hotspot-1M"]
    g = TraceGenerator(make_trace_cfg(w, seed=5))
    mbr = g.map_box(100.0)
    xy = np.stack([g.next() for _ in range(steps)])
    g.close()
    cfg = make_cfg(w, device=device)
    chosen, rep = autotune(cfg, mbr, xy, capacities=[64, 128, 256, 512])
    return {"workload": "hotspot-1M", "steps": steps, "base_grid_capacity": cfg.grid_capacity,
            "grid_capacity": chosen.grid_capacity, "job_chunk": chosen.job_chunk,
            "refine_chunk": chosen.refine_chunk, "refine_blocks_per_sm": chosen.refine_blocks_per_sm, "hits_blocks_per_sm": chosen.hits_blocks_per_sm,
            "base_step_ms": rep["base_step_ms"], "best_step_ms": rep["best_step_ms"],
            "speedup": rep["base_step_ms"] / rep["best_step_ms"], "trials": rep["trials"]}


COMPACT_STAGES = ("scratch_alloc", "decode", "object_order", "key_sort", "ctf_limits_and_alloc", "encode",
                  "index")


def compaction_line(c, peak):
    """Merge throughput; algorithmic bytes 2 x 32 per merged key (read and
    write each key and its box once). Its stages (stc_stats.compact_stage_ms):
    scratch allocation, the inputs' decode, the object order, the key sort,
    the CTF limits and metadata with the new block's allocation, the key
    encoding and the query index (host work between them included)."""
    if not c or "error" in c:
        return c
    b = 64.0 * c["keys"]
    c = dict(c)
    c.update(algorithmic_bytes=b, achieved_gbs=b / (c["ms"] / 1e3) / 1e9,
             frac_of_peak=b / (c["ms"] / 1e3) / 1e9 / peak)
    return c


def cpu_baseline(w, warmup, steps, threads, sample_note):
    """The oracle's C restatement of the reference CPU path on `threads` host
    threads: steps 0..warmup-1 untimed, then steps warmup..warmup+steps-1
    timed (the step indices the GPU arm times)."""
    import oracle
    from stcdb_gb300.tracegen import TraceGenerator
    gen = TraceGenerator(make_trace_cfg(w, seed=1))
    mbr = gen.map_box(100.0)
    x0 = gen.next().copy()
    cfg = make_cfg(w)
    o = oracle.Oracle(cfg, mbr, x0, threads=threads)
    o.step(x0, 0)
    for t in range(1, warmup):
        o.step(gen.next(), t)
    xs = [gen.next().copy() for _ in range(steps)]
    t0 = time.perf_counter()
    for k in range(steps):
        o.step(xs[k], warmup + k)
    dt = time.perf_counter() - t0
    o.close()
    gen.close()
    return {"value": w["objects"] * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": sample_note.format(steps=steps, first=warmup, last=warmup + steps - 1, seconds=round(dt, 2))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="uniform-10M", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-steps", type=int, default=2, help="steps timed for the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the plain-versus-window comparison")
    ap.add_argument("--batched-full", action="store_true",
                    help="batched line at the configuration's 1M-20M objects (tens of minutes) instead of 100k-2M")
    ap.add_argument("--query-rate", type=float, default=20000.0,
                    help="Poisson query arrivals per second during the serving phase (0: skip)")
    ap.add_argument("--step-slices", type=int, default=0,
                    help="launches per long step kernel (stc_config.step_slices; 0 = 1)")
    ap.add_argument("--serve-steps", type=int, default=0,
                    help="ingest steps of the serving phase (0 = twice --steps)")
    ap.add_argument("--serve-slices", type=int, default=1,
                    help="step slices while the serving phase answers queries (stc_set_step_slices)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_env()
    args.world = ws
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
    w = WORKLOADS[args.workload]
    N = w["objects"]
    threads = os.cpu_count() or 1
    workload_cfg = {"workload": args.workload, "objects": N, "steps_per_run": args.steps,
                    "street_grid": "200x200 over 40 km, jitter 20 m", "speed_mps": [1, 15],
                    "hotspots": w["hot"], "hot_frac": w.get("hot_frac", 0.7) if w["hot"] else 0.0,
                    "sigma_m": w.get("sigma_m", 300.0) if w["hot"] else None,
                    "reach_m": w["reach"], "min_meet_steps": w["min_meet"],
                    "leaf_capacity": w["grid_capacity"], "grid_amplify": w["amplify"],
                    "launch_shape": {"refine_blocks_per_sm": w.get("refine_bps", 8),
                                     "hits_blocks_per_sm": w.get("hits_bps", 16),
                                     "refine_chunk": w.get("refine_chunk") or "by density (64 or 256)"},
                    "meeting_buckets": make_cfg(w).resolved().num_meeting_buckets,
                    "memtable": (f"on, flush past {w['kv_restriction']} directed keys, 100 CTFs, "
                                 f"{w.get('bitmap_edge', 256)}x{w.get('bitmap_edge', 256)} map bitmaps"
                                 if w["kv_restriction"] else "off"),
                    "l2": "inputs and table larger than L2; no flush", "parallelism": f"replicas x{ws}"}

    if args.impl == "reference":
        if rank != 0:
            return
        steps = args.steps
        base = cpu_baseline(w, args.warmup, steps, threads,
                            "oracle C port of the reference CPU path, all host threads, steps {first}-{last} "
                            "({steps} full steps) after the warm-up steps ({seconds} s)")
        line = {"metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": ws, "steps": steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * N / base["value"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic (seeded grid-graph traces)", "impl": "reference",
                "config": workload_cfg, "cpu_baseline": base,
                "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    r = run_gpu(args, w, rank, local)
    K = args.steps
    dev_s = max_over_ranks(args, r["dev_ms"] / 1000.0)
    e2e_s = max_over_ranks(args, r["wall_e2e"])
    if rank != 0:
        return
    value = N * K * ws / dev_s
    e2e = N * K * ws / e2e_s
    s_last = r["stats"][-1]
    peak, peak_kind = measured_peaks()
    B = make_cfg(w).resolved().num_meeting_buckets
    phase_names = ["partition", "border", "refine", "insert", "sweep", "schema", "copy_in", "memtable"]
    phase_ms = {nm: sum(s.phase_ms[i] for s in r["stats"]) / K for i, nm in enumerate(phase_names)}
    st = r["stats"]
    kb = {k: sum(kernel_bytes(x, N, B, st[i - 1].taken_buckets if i else None)[k] for i, x in enumerate(st)) / K
          for k in ("partition", "refine", "sweep")}
    dom = max(("refine", "sweep", "partition"), key=lambda k: phase_ms[k])
    achieved = kb[dom] / (phase_ms[dom] / 1e3) / 1e9
    launches = sum(s.kernel_launches for s in r["stats"])
    base = None
    if not args.no_cpu_baseline:
        base = cpu_baseline(w, 1, args.cpu_steps, threads,
                            "oracle C port of the reference CPU path, all host threads, {steps} full steps "
                            "of the same workload after one warm-up step ({seconds} s)")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": args.warmup,
        "ms_per_step": r["dev_ms"] / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded grid-graph traces)", "config": workload_cfg,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 16 * N,
                "d2h_bytes_per_step": int(r["d2h"] / K), "host_link": r["link"], "windows": r["e2e_busy"]},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (REFINE_DRAM_BYTES_PER_HIT * sum(s.hits for s in r["stats"]) / K
                                 if dom == "refine" else None),
                     "traffic_source": "ncu capture of k_refine_a + k_hits at 3M objects, scaled by hits",
                     "algorithmic_bytes": kb[dom], "launch_ms": phase_ms[dom]},
        "phase_ms": phase_ms,
        "phase_gbs": {k: kb[k] / (phase_ms[k] / 1e3) / 1e9 for k in kb if phase_ms[k] > 0},
        "phase_frac_of_peak": {k: kb[k] / (phase_ms[k] / 1e3) / 1e9 / peak for k in kb if phase_ms[k] > 0},
        "flush": flush_line(r["flush"], peak),
        "queries_under_ingest": r["queries"],
        "queries_under_ingest_hbm_input": r["queries_hbm"],
        "trace_gen": r["trace_gen"],
        "compaction": compaction_line(r["compaction"], peak),
        "sort": sort_line(local, peak),
        "table_random_access": random_access_line(local, B, sum(s.hits for s in r["stats"]) / K,
                                                  phase_ms["refine"]),
        "batched": None if args.no_batched else batched_line(
            local, objects=(1e6, 2e7) if args.batched_full else (1e5, 2e6)),
        "autotune": None if args.no_batched else tune_line(local),
        "bit_exact": r["bit_exact"]["bit_exact"] if r["bit_exact"] else None,
        "bit_exact_check": r["bit_exact"],
        "per_step": {"pair_tests": s_last.pair_tests, "exact_tests": s_last.exact_tests, "hits": s_last.hits,
                     "new_candidates": s_last.new_candidates, "live_meetings": s_last.taken_buckets,
                     "emitted": s_last.emitted, "border_units": s_last.border_units, "leaves": s_last.leaves,
                     "overflow_objects": s_last.overflow_objects, "ambiguous_tests": s_last.ambiguous_tests,
                     "splits": s_last.splits, "merges": s_last.merges, "schema_path": s_last.schema_path},
        "wall_s": {"device_steps": r["wall_dev"], "e2e_steps": r["wall_e2e"]},
        "clocks": r["clocks"],
        "cpu_baseline": base,
    }
    # the figures a reader of the line's tail needs, repeated last
    q = r["queries"] or {}
    line["summary"] = {"value": value, "e2e": e2e, "bit_exact": line["bit_exact"],
                       "query_p50_ms": q.get("p50_ms"), "query_p99_ms": q.get("p99_ms"),
                       "query_max_ms": q.get("max_ms"), "queries_per_s": q.get("qps"),
                       "ingest_pos_updates_per_s_while_serving": q.get("ingest_pos_updates_per_s"),
                       "ingest_pos_updates_per_s_while_serving_hbm_input":
                           (r["queries_hbm"] or {}).get("ingest_pos_updates_per_s"),
                       "query_p99_ms_hbm_input": (r["queries_hbm"] or {}).get("p99_ms"),
                       "roofline_frac": line["roofline"]["frac"]}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
