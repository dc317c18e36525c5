"""GPU parity of the memtable and flush (stc_lsm.cu) against the oracle's
restatement (oracle/stc_lsm.c) fed with the oracle pipeline's emitted
meetings: every flushed block -- CTF metadata, bitmaps, packed keys, sids,
oversize keys, boxes and bitmap -- must be byte-identical."""
import numpy as np
import pytest

from stcdb_gb300.pipeline import Pipeline, StcConfig
from stcdb_gb300.tracegen import hotspot_grid, uniform_grid

from parity import trace_and_box

pytestmark = pytest.mark.gpu


def _same_block(g, o, t):
    gi, gb = g
    oi, ob = o
    assert gi.as_dict() == oi.as_dict(), f"step {t}: block info {gi.as_dict()} vs {oi.as_dict()}"
    assert gb["ctfs"].tobytes() == ob["ctfs"].tobytes(), f"step {t}: CTF metadata differs"
    for k in ("bitmaps", "keys", "sids", "oversize_keys", "oversize_boxes", "oversize_bitmap"):
        a, b = gb[k], ob[k]
        assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"step {t}: {k} differs"


def _run(cfg, tcfg, steps):
    import oracle as orc
    tr, mbr = trace_and_box(tcfg, steps)
    pipe = Pipeline(cfg, mbr, tr[0])
    ref = orc.Oracle(cfg, mbr, tr[0])
    lsm = orc.LsmOracle(cfg.num_objects, cfg.max_meet_time, cfg.ctf_count or 100, cfg.area_restriction or 100.0,
                        cfg.start_time + cfg.min_meet_time, mbr, 1 << 21, bitmap_edge=cfg.bitmap_edge)
    blocks = 0
    try:
        for t in range(steps):
            pipe.step(tr[t], t)
            pipe.drain()
            lsm.append(ref.step(tr[t], t))
            st = pipe.stats()
            if lsm.kv_count() > cfg.kv_restriction:
                lsm.flush(t)
                blocks += 1
                assert st.flushes == blocks, f"step {t}: GPU flushed {st.flushes}, oracle {blocks}"
                _same_block(pipe.read_ctb(), lsm.read(), t)
            assert st.flushes == blocks
            assert st.memtable_keys == lsm.kv_count(), f"step {t}: memtable {st.memtable_keys} vs {lsm.kv_count()}"
        # end of run: flush the rest
        if lsm.kv_count():
            assert pipe.flush()
            lsm.flush(steps - 1)
            blocks += 1
            _same_block(pipe.read_ctb(), lsm.read(), steps)
        assert not pipe.flush()
    finally:
        pipe.close()
        ref.close()
        lsm.close()
    return blocks


def test_flush_hotspot_long_meetings(built_cuda):
    """Dense hotspots; meetings longer than max_meet_time send objects to the
    oversize buffer (and shift the CTF ranges, as in the reference); several
    flushes, 16 CTFs."""
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=11)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, max_meet_time=6, grid_capacity=50,
                    grid_amplify=1.2, num_meeting_buckets=1_500_000, kv_restriction=60_000, ctf_count=16)
    assert _run(cfg, tc, 15) >= 2


@pytest.mark.parametrize("edge", [512, 96])
def test_flush_map_bitmap_edge(built_cuda, edge):
    """A map bitmap other than the reference's 256 x 256 (the stress
    configuration's 512 x 512; 96, not a power of two): the oversize buffer's
    bitmap has edge^2 bits, the rest of the block is unchanged."""
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=11)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, max_meet_time=6, grid_capacity=50,
                    grid_amplify=1.2, num_meeting_buckets=1_500_000, kv_restriction=60_000, ctf_count=16,
                    bitmap_edge=edge)
    assert _run(cfg, tc, 8) >= 1


def test_flush_area_restriction(built_cuda):
    """Objects whose box of all meetings is larger than the area restriction
    (the reference's smallest table entry) go to the oversize buffer."""
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=5)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.2,
                    num_meeting_buckets=1_500_000, kv_restriction=100_000, ctf_count=100,
                    area_restriction=7.24534e-06)
    assert _run(cfg, tc, 12) >= 1


def test_flush_uniform_default_ctfs(built_cuda):
    """Sparse road network, 100 CTFs (10 x 10 slabs), one flush at the end."""
    cfg = StcConfig(num_objects=20000, reach_distance=10.0, min_meet_time=5, grid_capacity=200,
                    num_meeting_buckets=200_000, kv_restriction=1 << 20)
    assert _run(cfg, uniform_grid(20000, seed=3), 25) == 1


def test_flush_rejects_bad_config_and_off_memtable(built_cuda):
    from stcdb_gb300.pipeline import StcError
    tr, mbr = trace_and_box(uniform_grid(2000, seed=1), 1)
    with pytest.raises(StcError):
        Pipeline(StcConfig(num_objects=2000, kv_restriction=1000, ctf_count=10), mbr, tr[0])
    for edge in (100, 2048):  # not a multiple of 32; too large
        with pytest.raises(StcError):
            Pipeline(StcConfig(num_objects=2000, kv_restriction=1000, bitmap_edge=edge), mbr, tr[0])
    with Pipeline(StcConfig(num_objects=2000), mbr, tr[0]) as p:
        with pytest.raises(StcError):
            p.flush()
        with pytest.raises(StcError):
            p.ctb_info()
