"""Block files (stc_write_ctb / stc_load_ctb): the files a flushed block is
written to must hold exactly the bytes the reference's writers produce for
that block -- rebuilt here from the oracle's copy of the block and the
reference's struct layout (tests/golden/ref_layout.txt, printed by the
reference's own headers) -- and a context that loads them answers queries as
the context that flushed the block."""
import os

import numpy as np
import pytest

from stcdb_gb300.pipeline import (QUERY_BOX, QUERY_DTYPE, QUERY_OBJECT, Pipeline, StcConfig, sort_contacts)
from stcdb_gb300.tracegen import hotspot_grid

from parity import trace_and_box

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _layout():
    lay = {}
    for line in open(os.path.join(HERE, "golden", "ref_layout.txt")):
        name, off, size = line.split()
        lay[name] = (int(off), int(size))
    return lay


def _put(buf, off, value, dtype):
    a = np.asarray(value, dtype=dtype).tobytes()
    buf[off:off + len(a)] = a


def _ctf_file(ctf, bitmap, lay):
    """CTF::dump_meta: the CTF object (pointers 0) then its bitmap."""
    size = lay["CTF"][0]
    b = bytearray(size)
    _put(b, lay["CTF.ctf_mbr"][0], ctf["mbr"], "<f4")
    for f in ("kv_count", "start_time_min", "start_time_max", "end_time_min", "end_time_max"):
        name = "CTF_kv_capacity" if f == "kv_count" else f
        _put(b, lay["CTF." + name][0], ctf[f], "<u4")
    _put(b, lay["CTF.ctf_bitmap_size"][0], ctf["bitmap_bytes"], "<u4")
    for f in ("key_bit", "id_bit", "duration_bit", "end_bit", "low_x_bit", "low_y_bit", "edge_bit", "mbr_bit",
              "x_grid", "y_grid"):
        _put(b, lay["CTF." + f][0], ctf[f], "<u2")
    return bytes(b) + bitmap[: int(ctf["bitmap_bytes"])].tobytes()


def _ctb_file(info, blk, lay):
    """workbench::dump_CTB_meta after straight_dump: the CTB object (pointers,
    CTF_count and its own times 0), sids, oversize keys, boxes, map bitmap."""
    b = bytearray(lay["CTB"][0])
    ob = lay["CTB.o_buffer"][0]
    _put(b, ob + lay["oversize_buffer.oversize_kv_count"][0], info.oversize_kv_count, "<u4")
    for f in ("start_time_min", "start_time_max", "end_time_min", "end_time_max"):
        _put(b, ob + lay["oversize_buffer." + f][0], getattr(info, "o_" + f), "<u4")
    return (bytes(b) + blk["sids"].astype("<u2").tobytes() + blk["oversize_keys"].astype("<u8").tobytes() +
            blk["oversize_boxes"].astype("<f4").tobytes() + blk["oversize_bitmap"].tobytes())


def _run(tmp_path):
    import oracle as orc
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=11)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, max_meet_time=6, grid_capacity=50,
                    grid_amplify=1.2, num_meeting_buckets=1_500_000, kv_restriction=60_000, ctf_count=16,
                    ctb_retain=4)
    tr, mbr = trace_and_box(tc, 12)
    pipe = Pipeline(cfg, mbr, tr[0])
    ref = orc.Oracle(cfg, mbr, tr[0])
    lsm = orc.LsmOracle(30000, 6, 16, 100.0, 3, mbr, 1 << 21)
    blocks = []
    for t in range(12):
        pipe.step(tr[t], t)
        pipe.drain()
        lsm.append(ref.step(tr[t], t))
        if lsm.kv_count() > cfg.kv_restriction:
            lsm.flush(t)
            blocks.append(lsm.read())
    ref.close()
    lsm.close()
    return cfg, mbr, pipe, blocks, tr[0]


def test_block_files_are_the_references_bytes_and_load_back(built_cuda, tmp_path):
    cfg, mbr, pipe, blocks, xy0 = _run(tmp_path)
    try:
        assert len(blocks) >= 2
        lay = _layout()
        info, blk = blocks[-1]
        idx = int(info.index)
        d = str(tmp_path)
        pipe.write_ctb(idx, d, "6oversize_3600")
        for c in range(int(info.ctf_count)):
            ctf = blk["ctfs"][c]
            meta = open(os.path.join(d, f"6oversize_3600_STcL{idx}-{c}"), "rb").read()
            assert meta == _ctf_file(ctf, blk["bitmaps"][c * 8192:(c + 1) * 8192], lay), f"CTF {c} meta"
            kb = int(ctf["key_bit"]) // 8
            o, n = int(ctf["key_offset"]), int(ctf["kv_count"]) * kb
            keys = open(os.path.join(d, f"6oversize_3600_SSTable_{idx}-{c}"), "rb").read()
            assert keys == blk["keys"][o:o + n].tobytes(), f"CTF {c} keys"
        ctb = open(os.path.join(d, f"6oversize_3600_CTB{idx}"), "rb").read()
        assert ctb == _ctb_file(info, blk, lay)

        # a fresh context loads the files and answers as the flushing one
        rng = np.random.default_rng(4)
        qs = np.zeros(120, QUERY_DTYPE)
        sids = blk["sids"]
        pids = np.flatnonzero(sids > 0)
        for i in range(80):
            qs[i]["kind"], qs[i]["pid"], qs[i]["t_start"], qs[i]["t_end"] = \
                QUERY_OBJECT, int(rng.choice(pids)), 0, 0xFFFFFFFF
        W, H = mbr[2] - mbr[0], mbr[3] - mbr[1]
        for i in range(80, 120):
            side = 10 ** rng.uniform(-4, -1.8)
            x, y = mbr[0] + rng.random() * (W - side), mbr[1] + rng.random() * (H - side)
            qs[i]["kind"], qs[i]["box"], qs[i]["t_start"], qs[i]["t_end"] = \
                QUERY_BOX, (x, y, x + side, y + side), 0, 0xFFFFFFFF
        import oracle as orc
        want = orc.query_blocks([blocks[-1]], qs)
        fresh = Pipeline(cfg, mbr, xy0)
        try:
            fresh.load_ctb(idx, d, "6oversize_3600")
            got = fresh.query_batch(qs)
            for i in range(len(qs)):
                assert sort_contacts(got[i]).tobytes() == sort_contacts(want[i]).tobytes(), f"query {i}"
            assert sum(len(w) for w in want) > 500
            with pytest.raises(Exception):
                fresh.load_ctb(idx + 100, d, "6oversize_3600")  # no such files
        finally:
            fresh.close()
    finally:
        pipe.close()
