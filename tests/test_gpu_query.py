"""GPU queries over the retained flushed blocks (stc_query.cu) against the
oracle's per-block queries (oracle/stc_lsm.c) on the same blocks: identical
contact sets (pid, target, start, end, decoded box bits, block, CTF)."""
import threading

import numpy as np
import pytest

from stcdb_gb300.pipeline import (QUERY_BOX, QUERY_DTYPE, QUERY_OBJECT, Pipeline, StcConfig, sort_contacts)
from stcdb_gb300.tracegen import hotspot_grid

from parity import trace_and_box

pytestmark = pytest.mark.gpu


def _ingest(cfg, tcfg, steps, retain):
    """Runs the pipeline and the oracle side by side; returns the pipeline and
    the oracle's copies of the retained blocks."""
    import oracle as orc
    tr, mbr = trace_and_box(tcfg, steps)
    pipe = Pipeline(cfg, mbr, tr[0])
    ref = orc.Oracle(cfg, mbr, tr[0])
    lsm = orc.LsmOracle(cfg.num_objects, cfg.max_meet_time, cfg.ctf_count or 100, cfg.area_restriction or 100.0,
                        cfg.start_time + cfg.min_meet_time, mbr, 1 << 21, bitmap_edge=cfg.bitmap_edge)
    blocks = []
    try:
        for t in range(steps):
            pipe.step(tr[t], t)
            pipe.drain()
            lsm.append(ref.step(tr[t], t))
            if lsm.kv_count() > cfg.kv_restriction:
                lsm.flush(t)
                blocks.append(lsm.read())
        blocks = blocks[-retain:]
    finally:
        ref.close()
        lsm.close()
    assert pipe.stats().flushes > retain, "the run should evict blocks"
    return pipe, blocks, mbr


def _queries(rng, blocks, mbr, n_obj, n_box):
    qs = np.zeros(n_obj + n_box, QUERY_DTYPE)
    sids = np.stack([b["sids"] for _, b in blocks])
    over = np.flatnonzero((sids == 1).any(0))
    ctf = np.flatnonzero((sids >= 2).any(0))
    none = np.flatnonzero((sids == 0).all(0))
    t_lo = max(min(int(i.end_time_min) for i, _ in blocks) - 10, 0)
    t_hi = max(int(i.flush_time) for i, _ in blocks) + 2
    for i in range(n_obj):
        pool = over if (i % 4 == 0 and len(over)) else none if (i % 10 == 1 and len(none)) else ctf
        qs[i]["kind"], qs[i]["pid"] = QUERY_OBJECT, int(rng.choice(pool))
        if i % 3 == 0:
            qs[i]["t_start"], qs[i]["t_end"] = 0, 0xFFFFFFFF
        else:
            a = int(rng.integers(t_lo, t_hi))
            qs[i]["t_start"], qs[i]["t_end"] = a, a + int(rng.integers(1, 8))
    W, H = mbr[2] - mbr[0], mbr[3] - mbr[1]
    for j in range(n_box):
        i = n_obj + j
        qs[i]["kind"] = QUERY_BOX
        if j == 0:
            qs[i]["box"] = mbr
        else:
            # about 5 m to 2.5 km; every fifth one 250 m to 5 km, so that some
            # counted queries cover whole cells of the index
            side = 10 ** (rng.uniform(-2.5, -1.3) if j % 5 == 4 else rng.uniform(-4.3, -1.6))
            x, y = mbr[0] + rng.random() * (W - side), mbr[1] + rng.random() * (H - side)
            qs[i]["box"] = (x, y, x + side, y + side * 0.8)
        if j % 2:
            a = int(rng.integers(t_lo, t_hi))
            qs[i]["t_start"], qs[i]["t_end"] = a, a + int(rng.integers(1, 6))
        else:
            qs[i]["t_start"], qs[i]["t_end"] = 0, 0xFFFFFFFF
    return qs


def _compare(pipe, blocks, qs):
    import oracle as orc
    got, counts = pipe.query_batch(qs, with_counts=True)
    want = orc.query_blocks(blocks, qs)
    only = pipe.query_counts(qs)  # count-only, with the contained-CTF shortcut
    total = 0
    for i in range(len(qs)):
        g, w = sort_contacts(got[i]), sort_contacts(want[i])
        assert len(g) == len(w) and g.tobytes() == w.tobytes(), \
            f"query {i} ({qs[i]}): GPU {len(g)} contacts, oracle {len(w)}"
        assert int(counts[i]) == len(w) and int(only[i]) == len(w), f"query {i}: counts {counts[i]}, {only[i]}"
        total += len(w)
    return total


@pytest.mark.parametrize("edge", [0, 512])
def test_queries_hotspot_with_oversize(built_cuda, edge):
    """Oversize keys in every block; box queries prune the oversize buffer by
    the block's map bitmap (256 x 256 by default, 512 x 512 as in the stress
    configuration)."""
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=11)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, max_meet_time=6, grid_capacity=50,
                    grid_amplify=1.2, num_meeting_buckets=1_500_000, kv_restriction=40_000, ctf_count=16,
                    ctb_retain=3, bitmap_edge=edge)
    pipe, blocks, mbr = _ingest(cfg, tc, 15, 3)
    try:
        rng = np.random.default_rng(1)
        qs = _queries(rng, blocks, mbr, 200, 60)
        assert _compare(pipe, blocks, qs) > 1000
        # the one-query calls give the batch's answers
        for i in (0, 1, 4, 200, 201):
            q = qs[i]
            one = (pipe.query_object(int(q["pid"]), int(q["t_start"]), int(q["t_end"])) if q["kind"] == QUERY_OBJECT
                   else pipe.query_box(q["box"], int(q["t_start"]), int(q["t_end"])))
            assert sort_contacts(one).tobytes() == sort_contacts(pipe.query_batch(qs[i:i + 1])[0]).tobytes()
    finally:
        pipe.close()


def test_queries_area_restriction_100_ctfs(built_cuda):
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=5)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.2,
                    num_meeting_buckets=1_500_000, kv_restriction=60_000, ctf_count=100,
                    area_restriction=7.24534e-06, ctb_retain=2)
    pipe, blocks, mbr = _ingest(cfg, tc, 12, 2)
    try:
        rng = np.random.default_rng(2)
        assert _compare(pipe, blocks, _queries(rng, blocks, mbr, 150, 40)) > 1000
    finally:
        pipe.close()


def test_queries_while_ingesting(built_cuda):
    """A second thread queries while the main thread steps and flushes: every
    answer equals the oracle's answer over the blocks that existed when the
    query ran (the blocks flushed before it started, or one or two more when
    a flush ran meanwhile)."""
    import oracle as orc
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=7)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.2,
                    num_meeting_buckets=1_500_000, kv_restriction=30_000, ctf_count=16, ctb_retain=32)
    steps = 14
    tr, mbr = trace_and_box(tc, steps)
    # the oracle's blocks, flush by flush
    ref = orc.Oracle(cfg, mbr, tr[0])
    lsm = orc.LsmOracle(cfg.num_objects, cfg.max_meet_time, cfg.ctf_count, cfg.area_restriction or 100.0,
                        cfg.start_time + cfg.min_meet_time, mbr, 1 << 21)
    blocks = []
    try:
        for t in range(steps):
            lsm.append(ref.step(tr[t], t))
            if lsm.kv_count() > cfg.kv_restriction:
                lsm.flush(t)
                blocks.append(lsm.read())
    finally:
        ref.close()
        lsm.close()
    assert 2 <= len(blocks) <= 32
    errors, records = [], []
    flushed = [0]  # blocks flushed by the steps that have returned
    stop = threading.Event()
    with Pipeline(cfg, mbr, tr[0]) as pipe:
        def worker():
            rng = np.random.default_rng(3)
            while not stop.is_set():
                try:
                    q = np.zeros(1, QUERY_DTYPE)
                    q["t_start"], q["t_end"] = 0, 0xFFFFFFFF
                    if rng.random() < 0.5:
                        q["kind"], q["pid"] = QUERY_OBJECT, int(rng.integers(0, 30000))
                    else:
                        x = mbr[0] + rng.random() * (mbr[2] - mbr[0] - 0.003)
                        y = mbr[1] + rng.random() * (mbr[3] - mbr[1] - 0.003)
                        q["kind"], q["box"] = QUERY_BOX, (x, y, x + 0.003, y + 0.002)
                    f0 = flushed[0]
                    got = pipe.query_batch(q)[0]
                    records.append((q[0].copy(), got.copy(), f0, flushed[0]))
                except Exception as e:  # noqa: BLE001 - reported below
                    errors.append(e)
                    return
        th = threading.Thread(target=worker)
        th.start()
        try:
            for t in range(steps):
                pipe.step(tr[t], t)
                pipe.drain()
                flushed[0] = pipe.stats().flushes
        finally:
            stop.set()
            th.join()
        assert pipe.stats().flushes == len(blocks)
    assert not errors, errors
    assert len(records) > 20
    answered_with_blocks = 0
    for q, got, f0, f1 in records:
        g = sort_contacts(got).tobytes()
        ok = False
        for f in range(f0, min(f1 + 1, len(blocks)) + 1):
            want = orc.query_blocks(blocks[:f], q[None])[0] if f else np.zeros(0, got.dtype)
            if sort_contacts(want).tobytes() == g:
                ok = True
                break
        assert ok, f"query {q} (flushes {f0}..{f1}): {len(got)} contacts match no block set of the oracle"
        answered_with_blocks += f0 > 0
    assert answered_with_blocks > 0
