"""The library's request loop (stc_server_*): answers equal direct query
batches, batches stay within their device-footprint budget, every query is
answered once, latencies are measured from the given arrival times."""
import time

import numpy as np
import pytest

from stcdb_gb300.pipeline import (QUERY_BOX, QUERY_COUNT_ONLY, QUERY_DTYPE, QUERY_OBJECT, Pipeline, StcConfig,
                                  sort_contacts)
from stcdb_gb300.tracegen import hotspot_grid

from parity import trace_and_box

pytestmark = pytest.mark.gpu


def _pipeline():
    tr, mbr = trace_and_box(hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=21), 14)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.5,
                    num_meeting_buckets=1_500_000, kv_restriction=40_000, ctf_count=16)
    p = Pipeline(cfg, mbr, tr[0])
    for t in range(len(tr)):
        p.step(tr[t], t)
        p.drain()
    assert p.stats().flushes >= 1
    return p, mbr


def _queries(rng, n, mbr, count_every):
    qs = np.zeros(n, QUERY_DTYPE)
    W, H = mbr[2] - mbr[0], mbr[3] - mbr[1]
    for i in range(n):
        if i % 2:
            qs[i]["kind"], qs[i]["pid"] = QUERY_OBJECT, int(rng.integers(0, 30000))
        else:
            x, y = mbr[0] + rng.random() * W, mbr[1] + rng.random() * H
            s = rng.random() * 0.05 * W
            qs[i]["kind"], qs[i]["box"] = QUERY_BOX, (x, y, x + s, y + s)
        qs[i]["t_start"], qs[i]["t_end"] = 0, 0xFFFFFFFF
        if i % count_every == 0:
            qs[i]["kind"] |= QUERY_COUNT_ONLY
    return qs


def test_server_answers_match_direct_batches(built_cuda):
    p, mbr = _pipeline()
    rng = np.random.default_rng(4)
    qs = _queries(rng, 300, mbr, 3)
    contacts, want_counts = p.query_batch(qs, with_counts=True)
    # a budget that fits a few contact-returning queries per batch
    srv = p.server(max_batch=64, result_cap=4096, hbm_budget=3 * (4096 * 64 + 72) + 40 * 72)
    try:
        first = None
        t_arr = time.perf_counter()
        for k in range(0, len(qs), 50):
            f = srv.submit(qs[k:k + 50], arrival=t_arr)
            first = f if first is None else first
        got, contacts_got = [], []
        deadline = time.time() + 60
        while sum(len(a) for a in got) < len(qs) and time.time() < deadline:
            a, c = srv.poll(cap=4096, contacts_cap=4_000_000, wait_ms=200)
            got.append(a)
            contacts_got.append((a, c))
        st = srv.stats()
    finally:
        srv.stop()
    ans = np.concatenate(got)
    assert len(ans) == len(qs) and sorted(ans["ticket"]) == list(range(first, first + len(qs)))
    assert st.answered == len(qs) and st.batches > 1 and st.budget_cuts > 0
    assert st.max_batch_bytes <= 3 * (4096 * 64 + 72) + 40 * 72
    assert (ans["latency_ms"] > 0).all()
    for a, c in contacts_got:
        for r in a:
            i = int(r["ticket"] - first)
            assert r["count"] == want_counts[i], f"query {i}: count {r['count']} vs {want_counts[i]}"
            if qs[i]["kind"] & QUERY_COUNT_ONLY:
                assert r["stored"] == 0
            elif r["status"] == 0:
                mine = c[int(r["contact_offset"]): int(r["contact_offset"] + r["stored"])]
                assert np.array_equal(sort_contacts(mine), sort_contacts(contacts[i]))
    p.close()


def test_server_stop_answers_everything_queued(built_cuda):
    p, mbr = _pipeline()
    qs = _queries(np.random.default_rng(5), 200, mbr, 1)  # all counting
    srv = p.server(max_batch=16)
    srv.submit(qs)
    srv.stop()  # returns once every queued query has been answered
    p.close()
