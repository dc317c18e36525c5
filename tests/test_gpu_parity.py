"""GPU parity: the CUDA pipeline against the oracle (the reference's CPU
algorithm, single-threaded) on seeded workloads, step by step, bit-exact on
(pid_lo, pid_hi, start, end) and on the float MBR."""
import numpy as np
import pytest

from stcdb_gb300.pipeline import StcConfig
from stcdb_gb300.tracegen import hotspot_grid, uniform_grid

from parity import describe_diff, run_pair, trace_and_box

pytestmark = pytest.mark.gpu


def _check(cfg, tcfg, steps):
    tr, mbr = trace_and_box(tcfg, steps)
    total = 0
    for t, g, o, gs, os_ in run_pair(cfg, tr, mbr):
        assert gs.checking_units == os_.checking_units, f"step {t}: units {gs.checking_units} vs {os_.checking_units}"
        assert gs.hits == os_.hits, f"step {t}: hits {gs.hits} vs {os_.hits}"
        assert gs.leaves == os_.leaves and gs.schema_nodes == os_.schema_nodes, f"step {t}: schema differs"
        assert np.array_equal(g, o), f"step {t}: " + describe_diff(g, o)
        total += len(o)
    return total


def test_uniform_grid_small(built_cuda):
    """Config-1 model at 20k objects: sparse road network, rare meetings."""
    cfg = StcConfig(num_objects=20000, reach_distance=10.0, min_meet_time=5, grid_capacity=200,
                    num_meeting_buckets=200000)
    assert _check(cfg, uniform_grid(20000, seed=3), 25) > 0


def test_hotspot_dense_chain_breaks(built_cuda):
    """Dense hotspots, loaded table (restarts across cleared slots), overflowing
    leaves (grid_amplify 1.2) and dynamic splits/merges."""
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=11)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.2,
                    num_meeting_buckets=1_500_000)
    assert _check(cfg, tc, 15) > 0


def test_serial_schema_replay_matches(built_cuda):
    """The one-thread split/merge replay and the parallel one agree."""
    from stcdb_gb300.pipeline import FLAG_SERIAL_SCHEMA
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=12)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50,
                    num_meeting_buckets=1_500_000, flags=FLAG_SERIAL_SCHEMA)
    assert _check(cfg, tc, 12) > 0


def test_table_full_reports_capacity(built_cuda):
    """A meeting table too small for the live pairs returns STC_ERR_CAPACITY
    (bounded probe walks), never hangs, and the context can be destroyed."""
    from stcdb_gb300.pipeline import Pipeline, StcError
    tr, mbr = trace_and_box(hotspot_grid(20000, n_hotspots=20, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=2), 2)
    cfg = StcConfig(num_objects=20000, reach_distance=10.0, grid_capacity=50, num_meeting_buckets=5000)
    p = Pipeline(cfg, mbr, tr[0])
    with pytest.raises(StcError) as e:
        p.step(tr[0], 0)
    assert e.value.status in (3, 4)
    with pytest.raises(StcError) as e2:
        p.step(tr[1], 1)  # a failed context refuses further steps
    assert e2.value.status == 6
    p.close()


def test_partial_drain(built_cuda):
    """Draining in small pieces returns the same meetings as one drain."""
    import ctypes
    from stcdb_gb300.pipeline import MEETING_DTYPE, Pipeline
    tr, mbr = trace_and_box(hotspot_grid(20000, n_hotspots=20, box_m=3000.0, grid_n=16, sigma_m=150.0, seed=5), 9)
    cfg = StcConfig(num_objects=20000, reach_distance=10.0, min_meet_time=3, grid_capacity=50,
                    num_meeting_buckets=1 << 20)
    with Pipeline(cfg, mbr, tr[0]) as a, Pipeline(cfg, mbr, tr[0]) as b:
        for t in range(9):
            a.step(tr[t], t)
            b.step(tr[t], t)
        whole = a.drain()
        parts = []
        while True:
            buf = np.zeros(37, dtype=MEETING_DTYPE)
            n = ctypes.c_size_t()
            assert b._lib.stc_drain_meetings(b._h, buf.ctypes.data, 37, ctypes.byref(n)) == 0
            parts.append(buf[: n.value])
            if n.value < 37:
                break
        got = np.concatenate(parts)
        assert len(whole) > 37
        from stcdb_gb300.pipeline import sort_meetings
        assert np.array_equal(sort_meetings(whole), sort_meetings(got))


def test_drain_into_pinned_buffer(built_cuda):
    """A page-locked output buffer (one direct copy) and a small pageable one
    (staged, in pieces) return what the default drain returns."""
    import torch
    from stcdb_gb300.pipeline import MEETING_DTYPE, Pipeline, sort_meetings
    tr, mbr = trace_and_box(hotspot_grid(20000, n_hotspots=20, box_m=3000.0, grid_n=16, sigma_m=150.0, seed=6), 9)
    cfg = StcConfig(num_objects=20000, reach_distance=10.0, min_meet_time=3, grid_capacity=50,
                    num_meeting_buckets=1 << 20)
    pinned = torch.empty((1 << 16) * MEETING_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    pout = pinned.numpy().view(MEETING_DTYPE)
    small = np.zeros(16, MEETING_DTYPE)
    total = 0
    with Pipeline(cfg, mbr, tr[0]) as a, Pipeline(cfg, mbr, tr[0]) as b, Pipeline(cfg, mbr, tr[0]) as c:
        for t in range(9):
            for p in (a, b, c):
                p.step(tr[t], t)
            want = sort_meetings(a.drain())
            got = b.drain(pout)
            assert got.base is not None and np.array_equal(sort_meetings(got.copy()), want)
            assert np.array_equal(sort_meetings(c.drain(small)), want)  # too small: falls back to its own buffer
            total += len(want)
    assert total > 16


# Map box with dyadic corners: every quadtree split line, (lo + hi) / 2 at
# every depth, is an exact double, so objects can sit exactly on them.
DYADIC_BOX = np.array([-87.75, 41.75, -87.25, 42.25])


def _degenerate_trace(n, steps, seed):
    """Objects in a 0.004 x 0.004 degree patch around the root's split point,
    random-walking about 3 m a step, except: 150 coincident at the root's
    split point; 150 on its vertical and 150 on its horizontal split line;
    150 on deeper vertical split lines (depths 9-11); 20 at corners of the map
    box."""
    rng = np.random.default_rng(seed)
    cx, cy, h = -87.5, 42.0, 0.002
    base = np.column_stack([rng.uniform(cx - h, cx + h, n), rng.uniform(cy - h, cy + h, n)])
    g = np.arange(n)
    on_point, on_x, on_y, deep = g < 150, (g >= 150) & (g < 300), (g >= 300) & (g < 450), (g >= 450) & (g < 600)
    corner = (g >= 600) & (g < 620)
    lines = cx + np.array([-2.0 ** -10, -2.0 ** -11, -2.0 ** -12, 2.0 ** -12, 2.0 ** -11, 2.0 ** -10])
    out = np.empty((steps, n, 2))
    for t in range(steps):
        if t:
            base = base + rng.normal(0.0, 3e-5, (n, 2))
        p = base.copy()
        p[on_point] = (cx, cy)
        p[on_x, 0] = cx
        p[on_y, 1] = cy
        p[deep, 0] = lines[g[deep] % len(lines)]
        p[corner] = np.column_stack([np.where(g[corner] % 2 == 0, DYADIC_BOX[2], DYADIC_BOX[0]),
                                     np.where(g[corner] % 4 < 2, DYADIC_BOX[3], DYADIC_BOX[1])])
        out[t] = p
    return out


def _check_trace(cfg, tr, mbr):
    total = 0
    for t, g, o, gs, os_ in run_pair(cfg, tr, mbr):
        assert gs.checking_units == os_.checking_units, f"step {t}: units {gs.checking_units} vs {os_.checking_units}"
        assert gs.hits == os_.hits, f"step {t}: hits {gs.hits} vs {os_.hits}"
        assert gs.overflow_objects == os_.overflow_objects, f"step {t}: overflow differs"
        assert gs.leaves == os_.leaves and gs.schema_nodes == os_.schema_nodes, f"step {t}: schema differs"
        assert np.array_equal(g, o), f"step {t}: " + describe_diff(g, o)
        total += len(o)
    return total


def test_degenerate_positions(built_cuda):
    """Coincident objects (every pair within reach; their leaf splits down to
    twice the reach and drops the members past its capacity), objects exactly
    on split lines (the descent's tie rule: a coordinate equal to the split
    goes low) and at the map box's corners, against the oracle step by step."""
    tr = _degenerate_trace(3000, 8, 21)
    cfg = StcConfig(num_objects=3000, reach_distance=10.0, min_meet_time=3, grid_capacity=20, grid_amplify=1.5,
                    num_meeting_buckets=400_000)
    assert _check_trace(cfg, tr, DYADIC_BOX) > 1000


@pytest.mark.parametrize("n", [1, 2])
def test_one_and_two_objects(built_cuda, n):
    """One object (no pairs) and two objects together for five steps, then
    apart: the one meeting is emitted when it ends."""
    tr = np.tile(np.array([[-87.5, 42.0]]), (7, n, 1))
    if n == 2:
        tr[:, 1, 0] += 2e-5        # about 1.7 m apart
        tr[5:, 1, 0] += 0.01       # then about 800 m
    cfg = StcConfig(num_objects=n, reach_distance=10.0, min_meet_time=3, grid_capacity=20, num_meeting_buckets=64)
    assert _check_trace(cfg, tr, DYADIC_BOX) == (1 if n == 2 else 0)
