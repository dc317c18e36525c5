"""Generates tests/golden/compact_pin.npz: three flushed blocks and the block
the reference's own compaction (merge_dump, tools/compaction.cpp:729-1206)
makes of them.

The blocks come from the oracle (a seeded hotspot run through the CPU path
and the memtable flush, three flushes); they are written as the reference's
block files and merged by oracle/_ref/ref_compact (oracle/ref_compact.cpp
linked with the reference's unmodified tools/compaction.cpp, built by
oracle/build_ref.sh), whose output files are parsed back. Only this script
needs the reference checkout.

The inputs keep merge_dump on its defined paths: object 0 is parked outside
the street grid (merge_dump copies object 0's keys into CTFs it cannot fill),
no object is oversize (large area restriction, long max_meet_time), and the
sid bits the flush stores above each CTF key's oid are cleared (merge_dump
decodes the oid without a mask and would index its per-object arrays with
them).

    python tests/golden/make_compact_pin.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

N = 2500
F_IN = 16
SPLIT_OUT = 4
MAX_MEET = 4096
FLUSH_AT = (8, 16, 24)


def make_blocks():
    import oracle
    from stcdb_gb300.pipeline import StcConfig
    from stcdb_gb300.tracegen import TraceConfig, TraceGenerator
    tc = TraceConfig(num_objects=N, grid_n=14, box_m=1300.0, n_hotspots=10, hot_frac=0.7, sigma_m=60.0, seed=31)
    g = TraceGenerator(tc)
    tr = g.steps(FLUSH_AT[-1] + 1)
    mbr = g.map_box(100.0)
    tr[:, 0, 0] = mbr[0] + 1e-6  # object 0 far from every street
    tr[:, 0, 1] = mbr[1] + 1e-6
    cfg = StcConfig(num_objects=N, reach_distance=10.0, min_meet_time=3, max_meet_time=MAX_MEET, grid_capacity=50,
                    grid_amplify=4.0, num_meeting_buckets=1 << 18)
    ref = oracle.Oracle(cfg, mbr, tr[0])
    lsm = oracle.LsmOracle(N, MAX_MEET, F_IN, 1e12, 0, mbr, 1 << 20)
    blocks = []
    for t in range(FLUSH_AT[-1] + 1):
        lsm.append(ref.step(tr[t], t))
        if t in FLUSH_AT:
            lsm.flush(t)
            blocks.append(lsm.read())
    ref.close()
    lsm.close()
    for info, b in blocks:
        assert int(info.oversize_kv_count) == 0 and not (b["sids"] == 1).any()
        assert b["sids"][0] == 0, "object 0 has keys"
        strip_sid_bits(b)
    return blocks, mbr


def strip_sid_bits(b):
    """Clears the bits above the oid field of every CTF key."""
    keys = b["keys"]
    for c in b["ctfs"]:
        kb = int(c["key_bit"]) // 8
        total = 2 * int(c["id_bit"]) + int(c["duration_bit"]) + int(c["end_bit"]) + int(c["mbr_bit"])
        mask = (1 << total) - 1
        o = int(c["key_offset"])
        for k in range(int(c["kv_count"])):
            p = o + k * kb
            v = int.from_bytes(keys[p:p + kb].tobytes(), "little") & mask
            keys[p:p + kb] = np.frombuffer(v.to_bytes(kb, "little"), np.uint8)


def main():
    import oracle
    from blockfiles import layout, parse_ctb_file, parse_ctf_file, write_block
    oracle.build(reference=True)
    if not os.path.exists(oracle.REF_COMPACT):
        raise SystemExit("reference harness not built (no reference checkout here)")
    blocks, mbr = make_blocks()
    lay = layout()
    with tempfile.TemporaryDirectory() as d:
        for i, (info, b) in enumerate(blocks):
            write_block(d, "N", i, info, b, lay, raid=True)
        args = [oracle.REF_COMPACT, str(N), str(F_IN), str(SPLIT_OUT), str(len(blocks)), str(MAX_MEET)]
        args += [repr(float(v)) for v in mbr]
        subprocess.run(args, cwd=d, check=True, stdout=subprocess.DEVNULL)
        F2 = SPLIT_OUT * SPLIT_OUT
        ctb = parse_ctb_file(open(os.path.join(d, "m", "2G_CTB0"), "rb").read(), lay, N)
        ctfs, bitmaps, keys = [], [], []
        for c in range(F2):
            f, bm = parse_ctf_file(open(os.path.join(d, "m", f"2G_STcL0-{c}"), "rb").read(), lay)
            ctfs.append(f)
            bitmaps.append(np.frombuffer(bm, np.uint8))
            keys.append(np.frombuffer(open(os.path.join(d, f"r{c % 2}", f"2G_SSTable_0-{c}"), "rb").read(),
                                      np.uint8))
    out = {"meta": np.array([N, F_IN, SPLIT_OUT, MAX_MEET, len(blocks)], np.uint32),
           "map": np.asarray(mbr, np.float64)}
    for i, (info, b) in enumerate(blocks):
        p = f"in{i}_"
        out[p + "info"] = np.frombuffer(bytes(info), np.uint8).copy()
        for k in ("ctfs", "keys", "sids", "oversize_bitmap"):
            out[p + k] = b[k]
    cf = ("kv_count", "start_time_min", "start_time_max", "end_time_min", "end_time_max", "bitmap_bytes",
          "key_bit", "id_bit", "duration_bit", "end_bit", "low_x_bit", "low_y_bit", "edge_bit", "mbr_bit", "x_grid",
          "y_grid")
    out["out_mbr"] = np.array([f["mbr"] for f in ctfs], np.float32)
    out["out_fields"] = np.array([[f[k] for k in cf] for f in ctfs], np.uint32)
    out["out_bitmaps"] = np.concatenate(bitmaps)
    out["out_keys"] = np.concatenate(keys)
    out["out_sids"] = ctb["sids"]
    out["out_oversize_kv_count"] = np.array([ctb["oversize_kv_count"]], np.uint32)
    out["out_oversize_bitmap"] = ctb["oversize_bitmap"]
    np.savez_compressed(os.path.join(HERE, "compact_pin.npz"), **out)
    kv = out["out_fields"][:, 0]
    print("wrote compact_pin.npz:", len(blocks), "blocks,", int(sum(int(i.ctf_kv_count) for i, _ in blocks)),
          "keys in,", int(kv.sum()), "keys out in", F2, "CTFs")


if __name__ == "__main__":
    main()
