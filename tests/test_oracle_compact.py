"""The oracle's compaction (oracle/stc_compact.cpp).

Reference mode is pinned byte for byte against the reference's own
merge_dump (tests/golden/compact_pin.npz, made by
tests/golden/make_compact_pin.py). The compaction the GPU implements (normal
mode) then keeps every key: the decoded contacts of the merged block are
those of its inputs, each object's sid names the CTF holding its keys, and
object queries answer as over the inputs."""
import ctypes
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = ("kv_count", "start_time_min", "start_time_max", "end_time_min", "end_time_max", "bitmap_bytes", "key_bit",
          "id_bit", "duration_bit", "end_bit", "low_x_bit", "low_y_bit", "edge_bit", "mbr_bit", "x_grid", "y_grid")


def _pin():
    from stcdb_gb300.pipeline import StcCtbInfo
    z = np.load(os.path.join(HERE, "golden", "compact_pin.npz"))
    N, F_in, S, max_meet, m = (int(v) for v in z["meta"])
    blocks = []
    for i in range(m):
        p = f"in{i}_"
        info = StcCtbInfo()
        raw = z[p + "info"].tobytes()  # the fixture predates the info's bitmap_edge (0 reads as 256)
        ctypes.memmove(ctypes.byref(info), raw, min(len(raw), ctypes.sizeof(info)))
        b = {"ctfs": z[p + "ctfs"], "keys": z[p + "keys"], "sids": z[p + "sids"],
             "oversize_keys": np.zeros(0, np.uint64), "oversize_boxes": np.zeros(0, np.float32),
             "oversize_bitmap": z[p + "oversize_bitmap"]}
        b["bitmaps"] = np.zeros(F_in * 8192, np.uint8)
        blocks.append((info, b))
    return z, N, S, max_meet, z["map"], blocks


def _decoded(info, b):
    """(oid, target, duration, absolute end) of every CTF and oversize key."""
    import oracle
    lib = oracle.lib()
    out = []
    box = np.zeros(4, np.float64)
    vals = [ctypes.c_uint32() for _ in range(4)]
    vm = ctypes.c_uint64()
    for ci in range(len(b["ctfs"])):
        c = np.ascontiguousarray(b["ctfs"][ci:ci + 1])
        kb = int(c["key_bit"][0]) // 8
        for k in range(int(c["kv_count"][0])):
            key = np.ascontiguousarray(b["keys"][int(c["key_offset"][0]) + k * kb:][:kb])
            lib.lsm_decode_key(key.ctypes.data, c.ctypes.data, *[ctypes.byref(v) for v in vals], ctypes.byref(vm),
                               box.ctypes.data)
            out.append((vals[0].value, vals[1].value, vals[2].value, vals[3].value + int(c["end_time_min"][0])))
    ok = b["oversize_keys"].reshape(-1, 2)
    for lo, hi in ok:
        out.append((int(hi) >> 26, int(hi) & ((1 << 26) - 1), int(lo) >> 32,
                    (int(lo) & 0xFFFFFFFF) + int(info.o_end_time_min)))
    return sorted(out)


def test_reference_mode_is_the_references_merge(built):
    import oracle
    z, N, S, max_meet, mp, blocks = _pin()
    info, b = oracle.compact(blocks, N, S, max_meet, mp, 0, reference_mode=True)
    assert int(info.ctf_count) == S * S
    assert int(z["out_oversize_kv_count"][0]) == 0 == int(info.oversize_kv_count)
    got_fields = np.array([[int(c[k]) for k in FIELDS] for c in b["ctfs"]], np.uint32)
    assert np.array_equal(got_fields, z["out_fields"])
    assert b["ctfs"]["mbr"].tobytes() == z["out_mbr"].tobytes()
    bms = np.concatenate([b["bitmaps"][c * 8192:c * 8192 + int(t["bitmap_bytes"])] for c, t in enumerate(b["ctfs"])])
    assert bms.tobytes() == z["out_bitmaps"].tobytes()
    assert b["keys"].tobytes() == z["out_keys"].tobytes()
    assert np.array_equal(b["sids"], z["out_sids"])
    assert b["oversize_bitmap"].tobytes() == z["out_oversize_bitmap"].tobytes()
    # the reference leaves the last object of the STR order without a CTF
    n_in = sum(int(i.ctf_kv_count) for i, _ in blocks)
    assert int(info.ctf_kv_count) < n_in


def test_normal_mode_keeps_every_key(built):
    import oracle
    from stcdb_gb300.pipeline import QUERY_DTYPE, QUERY_OBJECT
    z, N, S, max_meet, mp, blocks = _pin()
    info, b = oracle.compact(blocks, N, S, max_meet, mp, 99)
    want = []
    for i, bb in blocks:
        want += _decoded(i, bb)
    assert _decoded(info, b) == sorted(want)
    assert int(info.kv_count) == len(want) and int(info.index) == 99
    # each object's keys sit in the CTF its sid names, objects ascending
    sids = b["sids"]
    for c, t in enumerate(b["ctfs"]):
        kb = int(t["key_bit"]) // 8
        oids = []
        for k in range(int(t["kv_count"])):
            key = int.from_bytes(b["keys"][int(t["key_offset"]) + k * kb:][:kb].tobytes(), "little")
            oids.append((key >> (int(t["id_bit"]) + int(t["duration_bit"]) + int(t["end_bit"]) + int(t["mbr_bit"])))
                        & ((1 << int(t["id_bit"])) - 1))
        assert oids == sorted(oids)
        assert all(int(sids[o]) == c + 2 for o in oids)
        assert int(t["end_time_min"]) == min(int(i.end_time_min) for i, _ in blocks)
        assert int(t["end_time_max"]) == max(int(i.flush_time) for i, _ in blocks)
    # object queries: the same contacts (boxes are re-quantised in the new CTFs)
    rng = np.random.default_rng(3)
    pids = rng.choice(np.flatnonzero(sids >= 2), 200, replace=False)
    qs = np.zeros(len(pids), QUERY_DTYPE)
    qs["kind"], qs["pid"], qs["t_start"], qs["t_end"] = QUERY_OBJECT, pids, 0, 0xFFFFFFFF
    a = oracle.query_blocks(blocks, qs)
    c = oracle.query_blocks([(info, b)], qs)
    key = ("pid", "target", "start", "end")
    for x, y in zip(a, c):
        assert sorted(tuple(int(r[k]) for k in key) for r in x) == sorted(tuple(int(r[k]) for k in key) for r in y)
    assert sum(len(x) for x in a) > 1000


def test_reference_mode_refuses_what_the_reference_cannot_do(built):
    import oracle
    z, N, S, max_meet, mp, blocks = _pin()
    with pytest.raises(RuntimeError):
        oracle.compact(blocks, N, 40, max_meet, mp, 0, reference_mode=True)  # negative last CTF
    oracle.compact(blocks, N, 40, max_meet, mp, 0)  # fine without the reference's sizes
