"""The refinement's launch shape (job_chunk, tile length refine_chunk, blocks
per SM) leaves every result unchanged, and stc_autotune picks a leaf capacity and launch shape
that run."""
import numpy as np
import pytest

from stcdb_gb300.pipeline import MEETING_DTYPE, Pipeline, StcConfig, autotune
from stcdb_gb300.tracegen import hotspot_grid

from parity import trace_and_box

pytestmark = pytest.mark.gpu


def _rows(m):
    a = np.ascontiguousarray(m).view(np.uint32).reshape(-1, MEETING_DTYPE.itemsize // 4)
    return a[np.lexsort(a.T[::-1])] if len(a) else a


def _run(cfg, tr, mbr):
    p = Pipeline(cfg, mbr, tr[0])
    try:
        out = []
        for t in range(len(tr)):
            p.step(tr[t], t)
            out.append((_rows(p.drain()), p.stats().hits, p.stats().taken_buckets))
        return out
    finally:
        p.close()


def test_launch_shape_leaves_results_unchanged(built_cuda):
    tr, mbr = trace_and_box(hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=9), 14)
    base = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.5,
                     num_meeting_buckets=1_500_000)
    want = _run(base, tr, mbr)
    assert sum(len(m) for m, _, _ in want) > 0
    for shape in [dict(job_chunk=1, refine_blocks_per_sm=2, hits_blocks_per_sm=64),
                  dict(job_chunk=64, refine_blocks_per_sm=32, hits_blocks_per_sm=1),
                  dict(refine_chunk=32), dict(refine_chunk=96, job_chunk=3), dict(refine_chunk=4096),
                  dict(refine_chunk=256)]:
        got = _run(StcConfig(**{**base.__dict__, **shape}), tr, mbr)
        for t, ((gm, gh, gb), (wm, wh, wb)) in enumerate(zip(got, want)):
            assert gh == wh and gb == wb, f"step {t}: counters differ with {shape}"
            assert np.array_equal(gm, wm), f"step {t}: meetings differ with {shape}"


@pytest.mark.parametrize("small_hit_buffer", [False, True])
def test_hit_emission_forms_give_the_same_results(built_cuda, small_hit_buffer):
    """The pair tests' two ways of handing over hits (straight to the hit
    buffer, or through a per-warp queue; the library picks by density) give
    the same meetings and counters every step, also when the hit buffer is
    too small and hits are applied inside the pair tests."""
    tr, mbr = trace_and_box(hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=9), 14)
    base = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.5,
                     num_meeting_buckets=1_500_000, hit_capacity=4096 if small_hit_buffer else 0)
    direct = _run(StcConfig(**{**base.__dict__, "flags": 2}), tr, mbr)  # STC_FLAG_DIRECT_HITS
    queued = _run(StcConfig(**{**base.__dict__, "flags": 4}), tr, mbr)  # STC_FLAG_QUEUED_HITS
    assert sum(len(m) for m, _, _ in queued) > 0
    for t, ((gm, gh, gb), (wm, wh, wb)) in enumerate(zip(direct, queued)):
        assert gh == wh and gb == wb, f"step {t}: counters differ"
        assert np.array_equal(gm, wm), f"step {t}: meetings differ"


def test_autotune_picks_a_runnable_setting(built_cuda):
    tr, mbr = trace_and_box(hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=10), 6)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=2.0,
                    num_meeting_buckets=1_500_000)
    chosen, rep = autotune(cfg, mbr, np.stack(tr), capacities=[25, 50, 100])
    assert chosen.grid_capacity in (25, 50, 100)
    assert chosen.job_chunk in (2, 4, 8, 16, 32) and chosen.refine_chunk in (0, 64, 128, 256, 512)
    assert chosen.refine_blocks_per_sm in (4, 8, 16) and chosen.hits_blocks_per_sm in (8, 16, 32)
    assert rep["trials"] == 3 + 4 + 4 + 2 + 2
    assert 0 < rep["best_step_ms"] <= rep["base_step_ms"]
    assert len(_run(chosen, tr, mbr)) == len(tr)
