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

from blockfiles import ctb_file, ctf_file, layout
from parity import trace_and_box

pytestmark = pytest.mark.gpu


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
        lay = layout()
        info, blk = blocks[-1]
        idx = int(info.index)
        d = str(tmp_path)
        pipe.write_ctb(idx, d, "6oversize_3600")
        for c in range(int(info.ctf_count)):
            ctf = blk["ctfs"][c]
            meta = open(os.path.join(d, f"6oversize_3600_STcL{idx}-{c}"), "rb").read()
            assert meta == ctf_file(ctf, blk["bitmaps"][c * 8192:(c + 1) * 8192], lay), f"CTF {c} meta"
            kb = int(ctf["key_bit"]) // 8
            o, n = int(ctf["key_offset"]), int(ctf["kv_count"]) * kb
            keys = open(os.path.join(d, f"6oversize_3600_SSTable_{idx}-{c}"), "rb").read()
            assert keys == blk["keys"][o:o + n].tobytes(), f"CTF {c} keys"
        ctb = open(os.path.join(d, f"6oversize_3600_CTB{idx}"), "rb").read()
        assert ctb == ctb_file(info, blk, lay)

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
