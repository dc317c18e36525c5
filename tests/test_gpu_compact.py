"""GPU compaction (stc_compact, stc_compact.cu) against the oracle's
restatement of the reference's merge_dump (oracle/stc_compact.cpp, normal
mode, itself pinned against the reference's own merge_dump by
tests/test_oracle_compact.py): the merged block -- CTF metadata, bitmaps,
packed keys, sids, oversize keys, boxes and bitmap -- must be byte-identical
to the oracle's merge of the same input blocks, queries must answer from it
as the oracle does, and it must survive a round trip through block files."""
import os

import numpy as np
import pytest

from stcdb_gb300.pipeline import QUERY_BOX, QUERY_DTYPE, QUERY_OBJECT, Pipeline, StcConfig, sort_contacts
from stcdb_gb300.tracegen import hotspot_grid

from parity import trace_and_box

pytestmark = pytest.mark.gpu


def _same_block(g, o, what):
    gi, gb = g
    oi, ob = o
    assert gi.as_dict() == oi.as_dict(), f"{what}: block info {gi.as_dict()} vs {oi.as_dict()}"
    assert gb["ctfs"].tobytes() == ob["ctfs"].tobytes(), f"{what}: CTF metadata differs"
    for k in ("bitmaps", "keys", "sids", "oversize_keys", "oversize_boxes", "oversize_bitmap"):
        a, b = gb[k], ob[k]
        assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"{what}: {k} differs"


def _run(max_meet, steps=14, n=30000, edge=0):
    """A run that flushes several blocks and keeps them all."""
    tc = hotspot_grid(n, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=11)
    cfg = StcConfig(num_objects=n, reach_distance=10.0, min_meet_time=3, max_meet_time=max_meet, grid_capacity=50,
                    grid_amplify=1.2, num_meeting_buckets=1_500_000, kv_restriction=60_000, ctf_count=16,
                    ctb_retain=16, bitmap_edge=edge)
    tr, mbr = trace_and_box(tc, steps)
    pipe = Pipeline(cfg, mbr, tr[0])
    for t in range(steps):
        pipe.step(tr[t], t)
        pipe.drain()
    pipe.flush()
    return cfg, mbr, pipe, tr[0]


def _queries(rng, blk, mbr, n_obj=150, n_box=60):
    qs = np.zeros(n_obj + n_box, QUERY_DTYPE)
    pids = np.flatnonzero(blk["sids"] > 0)
    W, H = mbr[2] - mbr[0], mbr[3] - mbr[1]
    for i in range(n_obj):
        qs[i]["kind"], qs[i]["pid"] = QUERY_OBJECT, int(rng.choice(pids))
        qs[i]["t_start"], qs[i]["t_end"] = (0, 0xFFFFFFFF) if i % 2 else (int(rng.integers(0, 8)), int(rng.integers(8, 16)))
    for i in range(n_obj, n_obj + n_box):
        side = 10 ** rng.uniform(-4, -1.8)
        x, y = mbr[0] + rng.random() * (W - side), mbr[1] + rng.random() * (H - side)
        qs[i]["kind"], qs[i]["box"], qs[i]["t_start"], qs[i]["t_end"] = QUERY_BOX, (x, y, x + side, y + side), 0, 0xFFFFFFFF
    return qs


@pytest.mark.parametrize("max_meet,split,edge", [(4096, 4, 0), (6, 5, 0), (6, 1, 0), (6, 5, 512)])
def test_compaction_is_the_oracles(built_cuda, max_meet, split, edge):
    import oracle as orc
    cfg, mbr, pipe, _ = _run(max_meet, edge=edge)
    try:
        infos = [pipe.block_info(i) for i in range(64) if _retained(pipe, i)]
        assert len(infos) >= 4
        blocks = [pipe.read_block(int(i.index)) for i in infos]
        if max_meet == 6:
            assert sum(int(i.oversize_kv_count) for i, _ in blocks) > 0
        first, count = int(infos[0].index), 3
        want = orc.compact(blocks[:count], cfg.num_objects, split, cfg.max_meet_time, mbr, len(infos))
        new, ms = pipe.compact(first, count, split)
        assert new == len(infos) and ms > 0.0
        got = pipe.read_block(new)
        _same_block(got, want, f"merge of {count} blocks into {split}x{split}")
        # the merged block replaced its inputs; queries see it and the rest
        with pytest.raises(Exception):
            pipe.block_info(first)
        rest = blocks[count:]
        qs = _queries(np.random.default_rng(5), blocks[0][1], mbr)
        ref = orc.query_blocks([want] + rest, qs)
        res = pipe.query_batch(qs)
        for i in range(len(qs)):
            assert sort_contacts(res[i]).tobytes() == sort_contacts(ref[i]).tobytes(), f"query {i}"
        assert sum(len(r) for r in ref) > 500
        # merging the merged block with the next one (the span grows)
        want2 = orc.compact([want, rest[0]], cfg.num_objects, split, cfg.max_meet_time, mbr, new + 1)
        new2, _ = pipe.compact(new, 2, split)
        _same_block(pipe.read_block(new2), want2, "second merge")
    finally:
        pipe.close()


def _retained(pipe, i):
    try:
        pipe.block_info(i)
        return True
    except Exception:
        return False


@pytest.mark.parametrize("edge", [0, 512])
def test_compacted_block_files_load_back(built_cuda, tmp_path, edge):
    cfg, mbr, pipe, xy0 = _run(6, edge=edge)
    try:
        new, _ = pipe.compact(0, 3, 7)  # 49 CTFs in a context of 16
        info, blk = pipe.read_block(new)
        d = str(tmp_path)
        pipe.write_ctb(new, d, "c")
        assert os.path.exists(os.path.join(d, f"c_STcL{new}-48")) and not os.path.exists(os.path.join(d, f"c_STcL{new}-49"))
        qs = _queries(np.random.default_rng(9), blk, mbr)
        import oracle as orc
        want = orc.query_blocks([(info, blk)], qs)
        fresh = Pipeline(cfg, mbr, xy0)
        try:
            fresh.load_ctb(new, d, "c")
            li, lb = fresh.read_block(new)
            assert int(li.ctf_count) == 49 and lb["keys"].tobytes() == blk["keys"].tobytes()
            assert lb["oversize_bitmap"].tobytes() == blk["oversize_bitmap"].tobytes()
            assert len(lb["oversize_bitmap"]) == (edge or 256) ** 2 // 8
            got = fresh.query_batch(qs)
            for i in range(len(qs)):
                assert sort_contacts(got[i]).tobytes() == sort_contacts(want[i]).tobytes(), f"query {i}"
        finally:
            fresh.close()
        with pytest.raises(Exception):
            pipe.compact(new, 5, 4)  # not that many blocks after it
        with pytest.raises(Exception):
            pipe.compact(new, 1, 64)  # split too large
    finally:
        pipe.close()
