"""The library's request loop (stc_server_*): answers equal direct query
batches and each query's answer alone, also while another thread steps;
batches stay within their device-footprint budget; contacts are capped per
query; batches over many blocks run as several passes; every query is
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


def _collect(srv, n, contacts_cap=4_000_000, timeout=60):
    got = []
    deadline = time.time() + timeout
    while sum(len(a) for a, _ in got) < n and time.time() < deadline:
        a, c = srv.poll(cap=4096, contacts_cap=contacts_cap, wait_ms=100)
        if len(a):
            got.append((a, c))
    return got


def test_server_answers_alone_equal_answers_in_a_mix_under_ingest(built_cuda):
    """Each query answered alone (a batch of one, before the mix) equals its
    answer from the server while another thread keeps stepping. The retained
    blocks stay fixed during the mix (flushes are explicit, none runs then),
    so the answers must be identical, contacts and counts."""
    import threading
    tr, mbr = trace_and_box(hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=23), 16)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.5,
                    num_meeting_buckets=1_500_000, kv_restriction=4_000_000, ctf_count=16, ctb_retain=8)
    with Pipeline(cfg, mbr, tr[0]) as p:
        for t in range(10):
            p.step(tr[t], t)
            p.drain()
            if t in (5, 9):
                assert p.flush()
        qs = _queries(np.random.default_rng(8), 240, mbr, 4)
        alone = [p.query_batch(qs[i:i + 1], with_counts=True) for i in range(len(qs))]
        srv = p.server(max_batch=32, result_cap=1 << 20)
        errors = []

        def ingest():
            try:
                for t in range(10, 16):
                    p.step(tr[t], t)
                    p.drain()
            except Exception as e:  # noqa: BLE001 - reported below
                errors.append(e)

        th = threading.Thread(target=ingest)
        th.start()
        rng = np.random.default_rng(9)
        first = None
        for k in range(0, len(qs), 8):
            f = srv.submit(qs[k:k + 8])
            first = f if first is None else first
            time.sleep(float(rng.uniform(0, 0.002)))
        got = _collect(srv, len(qs))
        th.join()
        st = srv.stats()
        srv.stop()
        assert not errors, errors
        assert p.stats().flushes == 2  # the blocks did not change during the mix
    assert st.answered == len(qs) and st.batches > 1
    seen = 0
    for a, c in got:
        for r in a:
            i = int(r["ticket"] - first)
            contacts, counts = alone[i]
            assert r["status"] == 0 and r["count"] == counts[0], f"query {i}"
            if not qs[i]["kind"] & QUERY_COUNT_ONLY:
                mine = c[int(r["contact_offset"]): int(r["contact_offset"] + r["stored"])]
                assert np.array_equal(sort_contacts(mine), sort_contacts(contacts[0])), f"query {i}: contacts"
            seen += 1
    assert seen == len(qs)


def test_server_caps_contacts_per_query(built_cuda):
    """One query over its contact reservation among small ones: only that
    query is answered with STC_ERR_CAPACITY (and its count); the others get
    their contacts, whatever batch they share."""
    p, mbr = _pipeline()
    try:
        qs = _queries(np.random.default_rng(11), 400, mbr, 1)
        qs["kind"] &= np.uint32(0xFF)  # all return contacts (no STC_QUERY_COUNT_ONLY)
        counts = p.query_counts(qs)
        small = np.flatnonzero((counts >= 1) & (counts <= 8))[:20]
        big = np.flatnonzero(counts > 64)[:1]
        assert len(small) >= 5 and len(big) == 1
        pick = np.concatenate([small[:3], big, small[3:]])
        mix = qs[pick]
        want = p.query_batch(mix)
        srv = p.server(max_batch=64, result_cap=8, hbm_budget=1 << 30)
        try:
            first = srv.submit(mix)
            got = _collect(srv, len(mix))
        finally:
            srv.stop()
        n = 0
        for a, c in got:
            for r in a:
                i = int(r["ticket"] - first)
                assert r["count"] == len(want[i])
                if i == 3:
                    assert r["status"] == 3 and r["stored"] == 0  # STC_ERR_CAPACITY
                else:
                    assert r["status"] == 0
                    mine = c[int(r["contact_offset"]): int(r["contact_offset"] + r["stored"])]
                    assert np.array_equal(sort_contacts(mine), sort_contacts(want[i]))
                n += 1
        assert n == len(mix)
    finally:
        p.close()


def test_server_full_batch_over_many_blocks(built_cuda):
    """16 retained blocks and a 4096-query batch: more than the 65535
    queries x blocks of one device pass, so the batch runs as several
    passes; every answer equals the direct batch's count."""
    tr, mbr = trace_and_box(hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=24), 20)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.5,
                    num_meeting_buckets=1_500_000, kv_restriction=4_000_000, ctf_count=16, ctb_retain=16)
    with Pipeline(cfg, mbr, tr[0]) as p:
        for t in range(20):
            p.step(tr[t], t)
            p.drain()
            if t >= 3:
                p.flush()
        assert p.stats().flushes >= 16
        qs = _queries(np.random.default_rng(12), 4096, mbr, 1)  # counting
        want = p.query_counts(qs)
        srv = p.server(max_batch=4096)
        try:
            first = srv.submit(qs)
            got = _collect(srv, len(qs))
        finally:
            srv.stop()
        ans = np.concatenate([a for a, _ in got])
        assert len(ans) == len(qs) and (ans["status"] == 0).all()
        assert np.array_equal(ans["count"][np.argsort(ans["ticket"])], want)
        assert first >= 1
