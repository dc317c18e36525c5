"""The oracle's flush restatement (oracle/stc_lsm.c) against the reference's
own host code for the CTF encoding (fixture tests/golden/ctf_pin.npz, made by
tests/golden/make_ctf_pin.py through oracle/ref_ctf.cpp), plus host-side
properties of a whole flush."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
PIN = os.path.join(HERE, "golden", "ctf_pin.npz")
BIT_FIELDS = ("key_bit", "id_bit", "duration_bit", "end_bit", "low_x_bit", "low_y_bit", "edge_bit", "mbr_bit",
              "x_grid", "y_grid")


def _sets(z):
    return sorted({k.split("_")[0] for k in z.files})


def test_ctf_encoding_matches_reference_host_code(built):
    import oracle
    z = np.load(PIN)
    checked = 0
    for s in _sets(z):
        mp = z[s + "_map"]
        nobj, mmt, _ = (int(v) for v in z[s + "_meta"])
        for i in range(len(z[s + "_ctf_mbr"])):
            c = oracle.ctf_bits(z[s + "_ctf_mbr"][i], mp, nobj, mmt)
            got = [int(c[f][0]) for f in BIT_FIELDS]
            assert got == [int(v) for v in z[s + "_bits"][i]], (s, i)
            assert int(c["bitmap_bytes"][0]) == int(z[s + "_bitmap_size"][i])
            vm = oracle.serialize_mbr(z[s + "_box"][i], c)
            assert vm == int(z[s + "_value_mbr"][i]), (s, i)
            key = oracle.pack_key(int(z[s + "_pid_field"][i]), int(z[s + "_target"][i]), int(z[s + "_dur"][i]),
                                  int(z[s + "_end"][i]), vm, c)
            ref = (int(z[s + "_key_hi"][i]) << 64) | int(z[s + "_key_lo"][i])
            kb = int(c["key_bit"][0]) // 8
            assert key == (ref & ((1 << (8 * kb)) - 1)).to_bytes(kb, "little"), (s, i)
            checked += 1
    assert checked >= 1000


def test_oversize_bitmap_and_times_match_reference_host_code(built):
    import oracle
    z = np.load(PIN)
    for s in _sets(z):
        mp = z[s + "_map"]
        bm = oracle.o_bitmap(z[s + "_oboxes"], mp)
        assert np.array_equal(bm, z[s + "_o_bitmap"]), s
        etm = int(z[s + "_meta"][2])
        starts = z[s + "_oend"].astype(np.int64) + etm - z[s + "_odur"].astype(np.int64)
        assert [int(starts.min()), int(starts.max())] == [int(v) for v in z[s + "_o_times"]]


def test_map_bitmap_edge_scales_the_pinned_256(built):
    """The map bitmap at edges 512 and 1024 (bitmap_edge; the reference fixes
    256 at compile time) against the 256 one pinned above: the cell of a
    coordinate at edge 256 * 2^k is 2^k times its cell at 256 plus a
    remainder (multiplying by a power of two is exact in double), so for
    boxes inside the map the 2^k x 2^k blocks of the larger bitmap OR
    together into the 256 x 256 one."""
    import oracle
    z = np.load(PIN)
    rng = np.random.default_rng(3)
    checked = 0
    for s in _sets(z):
        mp = z[s + "_map"]
        boxes = np.asarray(z[s + "_oboxes"], np.float32).reshape(-1, 4)
        # fixture boxes inside the map, and random ones from points to wide boxes
        inside = boxes[(boxes[:, 0] >= mp[0]) & (boxes[:, 1] >= mp[1]) & (boxes[:, 2] < mp[2]) & (boxes[:, 3] < mp[3])]
        lo = rng.random((200, 2)) * 0.9
        wh = rng.random((200, 2)) ** 4 * 0.09
        rnd = np.concatenate([mp[0] + (mp[2] - mp[0]) * np.stack([lo[:, 0], lo[:, 0] + wh[:, 0]], 1),
                              mp[1] + (mp[3] - mp[1]) * np.stack([lo[:, 1], lo[:, 1] + wh[:, 1]], 1)], 1)
        rnd = rnd[:, [0, 2, 1, 3]].astype(np.float32)
        rnd = rnd[(rnd[:, 2] < mp[2]) & (rnd[:, 3] < mp[3])]
        for bx in (inside, rnd):
            base = np.unpackbits(oracle.o_bitmap(bx, mp, 256), bitorder="little").reshape(256, 256)
            for k in (1, 2):
                e = 256 << k
                big = np.unpackbits(oracle.o_bitmap(bx, mp, e), bitorder="little").reshape(e, e)
                down = big.reshape(256, 1 << k, 256, 1 << k).any(axis=(1, 3))
                assert np.array_equal(down, base.astype(bool)), (s, e)
                checked += int(base.sum())
    assert checked > 1000


def test_live_reference_pin_when_available(built):
    """Re-runs the reference host code on fresh cases where its build exists."""
    import oracle
    if not os.path.exists(oracle.REF_CTF):
        pytest.skip("reference harness not built here")
    import subprocess
    import sys
    import tempfile
    import shutil
    with tempfile.TemporaryDirectory() as d:
        # regenerate into a scratch copy and compare it with the committed fixture
        env = dict(os.environ)
        script = os.path.join(HERE, "golden", "make_ctf_pin.py")
        shutil.copy(script, os.path.join(d, "make_ctf_pin.py"))
        src = open(script).read().replace('os.path.dirname(os.path.dirname(HERE))', repr(os.path.dirname(HERE)))
        open(os.path.join(d, "make_ctf_pin.py"), "w").write(src)
        subprocess.run([sys.executable, os.path.join(d, "make_ctf_pin.py")], check=True, env=env,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        a, b = np.load(os.path.join(d, "ctf_pin.npz")), np.load(PIN)
        assert sorted(a.files) == sorted(b.files)
        for k in a.files:
            assert np.array_equal(a[k], b[k]), k


def _meetings(rng, n_obj, n, t0, t1, mp, long_frac=0.0):
    from oracle import MEETING_DTYPE
    m = np.zeros(n, MEETING_DTYPE)
    a = rng.integers(0, n_obj, n)
    b = (a + rng.integers(1, n_obj, n)) % n_obj
    m["pid_lo"] = np.minimum(a, b)
    m["pid_hi"] = np.maximum(a, b)
    m["end"] = rng.integers(t0, t1, n)
    dur = rng.integers(5, 40, n)
    if long_frac:
        dur[rng.random(n) < long_frac] = 1200
    m["start"] = np.maximum(m["end"].astype(np.int64) - dur, 0)
    W, H = mp[2] - mp[0], mp[3] - mp[1]
    x = mp[0] + 0.05 * W + rng.random(n) * 0.9 * W
    y = mp[1] + 0.05 * H + rng.random(n) * 0.9 * H
    w = rng.random(n) * 2e-4
    h = rng.random(n) * 2e-4
    m["mbr"] = np.stack([x, y, x + w, y + h], 1).astype(np.float32)
    # one meeting per (pair, end)
    _, keep = np.unique(np.stack([m["pid_lo"], m["pid_hi"], m["end"]], 1), axis=0, return_index=True)
    return m[np.sort(keep)]


def test_flush_block_is_consistent(built):
    """Size-independent properties of a whole flush with no meeting longer
    than max_meet_time: key counts, CTF ranges, sids, time limits and that
    every CTF key decodes back to its meeting."""
    import oracle
    rng = np.random.default_rng(7)
    mp = np.array([-87.9412, 41.6437, -87.80, 41.75])
    n_obj, F = 5000, 16
    # key times count from 5000; every end offset fits the 10-bit end field
    m = _meetings(rng, n_obj, 20000, 5000, 5900, mp)
    lo = oracle.LsmOracle(n_obj, 1000, F, 100.0, 5000, mp, 1 << 20)
    lo.append(m)
    assert lo.kv_count() == 2 * len(m)
    lo.flush(5900)
    info, b = lo.read()
    assert info.kv_count == 2 * len(m)
    assert info.oversize_kv_count == 0
    assert info.ctf_kv_count == info.kv_count
    ctfs = b["ctfs"]
    assert int(ctfs["kv_count"].sum()) == info.ctf_kv_count
    assert np.all(np.diff(ctfs["first_key"].astype(np.int64)) == ctfs["kv_count"][:-1])
    sids = b["sids"]
    assert set(np.unique(sids)) <= set(range(0, F + 2))
    # every key of CTF c belongs to an object with sid c + 2 and decodes to one meeting
    long_pairs = set()
    for r in m[(m["end"] - m["start"]) > 1000]:
        long_pairs.add(int(r["pid_lo"]))
        long_pairs.add(int(r["pid_hi"]))
    want = {}
    for r in m:
        for p, q in ((r["pid_lo"], r["pid_hi"]), (r["pid_hi"], r["pid_lo"])):
            want[(int(p), int(q), int(r["end"]) - 5000)] = int(r["end"] - r["start"])
    keys = b["keys"]
    seen = 0
    for c in range(F):
        t = ctfs[c]
        kb = int(t["key_bit"]) // 8
        shift_end = int(t["mbr_bit"])
        for i in range(int(t["kv_count"])):
            off = int(t["key_offset"]) + i * kb
            k = int.from_bytes(keys[off:off + kb].tobytes(), "little")
            endv = (k >> shift_end) & ((1 << int(t["end_bit"])) - 1)
            k2 = k >> (shift_end + int(t["end_bit"]))
            dur = k2 & ((1 << int(t["duration_bit"])) - 1)
            k3 = k2 >> int(t["duration_bit"])
            target = k3 & ((1 << int(t["id_bit"])) - 1)
            pid = (k3 >> int(t["id_bit"])) & ((1 << int(t["id_bit"])) - 1)
            assert sids[pid] == c + 2
            assert want[(pid, target, endv)] == dur
            seen += 1
        if t["kv_count"]:
            assert t["start_time_min"] <= t["start_time_max"]
            assert t["end_time_min"] == 5000 and t["end_time_max"] == 5900
    assert seen == len(want)
    assert not long_pairs
    # the next block's times start at the flush step
    lo.append(_meetings(rng, n_obj, 100, 5901, 5910, mp))
    lo.flush(5910)
    info2, _ = lo.read()
    assert info2.index == 1 and info2.end_time_min == 5900


def test_flush_with_long_meetings(built):
    """Meetings longer than max_meet_time send both objects' keys to the
    oversize buffer. The reference counts such meetings in oversize_oid_count
    and later gives the objects CTF sids when their box is small, so the CTF
    ranges shift into the oversize keys; the block stays well formed."""
    import oracle
    rng = np.random.default_rng(11)
    mp = np.array([-87.9412, 41.6437, -87.80, 41.75])
    n_obj, F = 5000, 16
    m = _meetings(rng, n_obj, 20000, 5000, 5900, mp, long_frac=0.01)
    lo = oracle.LsmOracle(n_obj, 1000, F, 100.0, 5000, mp, 1 << 20)
    lo.append(m)
    lo.flush(5900)
    info, b = lo.read()
    n_long = int(((m["end"] - m["start"]) > 1000).sum())
    assert n_long > 0
    assert info.oversize_oid_count >= n_long
    assert info.ctf_kv_count + info.oversize_kv_count == info.kv_count == 2 * len(m)
    ctfs = b["ctfs"]
    assert int(ctfs["kv_count"].sum()) <= info.kv_count
    assert np.all(np.diff(ctfs["first_key"].astype(np.int64)) == ctfs["kv_count"][:-1])
    ok = b["oversize_keys"].reshape(-1, 2)
    okset = {(int(hi) >> 26, int(hi) & ((1 << 26) - 1), int(lo) & 0xFFFFFFFF) for lo, hi in ok}
    for r in m[(m["end"] - m["start"]) > 1000]:
        assert (int(r["pid_lo"]), int(r["pid_hi"]), int(r["end"]) - 5000) in okset
        assert (int(r["pid_hi"]), int(r["pid_lo"]), int(r["end"]) - 5000) in okset
    order = np.lexsort((ok[:, 0], ok[:, 1]))
    assert np.array_equal(order, np.arange(len(ok)))


def test_area_restriction_moves_objects_to_oversize(built):
    import oracle
    rng = np.random.default_rng(3)
    mp = np.array([-87.9412, 41.6437, -87.80, 41.75])
    m = _meetings(rng, 2000, 5000, 10, 100, mp)
    a = oracle.LsmOracle(2000, 4096, 4, 100.0, 5, mp, 1 << 16)
    b = oracle.LsmOracle(2000, 4096, 4, 1e-9, 5, mp, 1 << 16)
    for o in (a, b):
        o.append(m)
        o.flush(100)
    ia, _ = a.read()
    ib, bb = b.read()
    assert ia.oversize_kv_count == 0
    assert ib.oversize_kv_count > ia.oversize_kv_count
    assert ib.oversize_oid_count > 0


def test_key_decoding_matches_reference_host_code(built):
    """lsm_decode_key = CTF::ctf_get_key_oid + parse_key + new_parse_mbr on
    the stored key bytes (fixture made by the reference's own code)."""
    import ctypes
    import oracle
    z = np.load(PIN)
    lib = oracle.lib()
    n = 0
    for s in _sets(z):
        mp = z[s + "_map"]
        nobj, mmt, _ = (int(v) for v in z[s + "_meta"])
        for i in range(len(z[s + "_ctf_mbr"])):
            c = oracle.ctf_bits(z[s + "_ctf_mbr"][i], mp, nobj, mmt)
            kb = int(c["key_bit"][0]) // 8
            key = ((int(z[s + "_key_hi"][i]) << 64) | int(z[s + "_key_lo"][i])) & ((1 << (8 * kb)) - 1)
            kbytes = np.frombuffer(key.to_bytes(16, "little"), np.uint8).copy()
            f = (ctypes.c_uint32 * 4)()
            vm = ctypes.c_uint64()
            box = np.zeros(4, np.float64)
            lib.lsm_decode_key(kbytes.ctypes.data, c.ctypes.data, ctypes.byref(f, 0), ctypes.byref(f, 4),
                               ctypes.byref(f, 8), ctypes.byref(f, 12), ctypes.byref(vm), box.ctypes.data)
            assert list(f) == [int(v) for v in z[s + "_dec"][i]], (s, i)
            assert vm.value == int(z[s + "_dec_vm"][i]), (s, i)
            assert box.tobytes() == z[s + "_dec_box"][i].tobytes(), (s, i)
            n += 1
    assert n >= 1000


def _truth(m, pid=None, box=None, t1=0, t2=0xFFFFFFFF, etm=5000):
    """(pid, target, start, end) of every directed key matching the query."""
    out = set()
    for r in m:
        for p, q in ((int(r["pid_lo"]), int(r["pid_hi"])), (int(r["pid_hi"]), int(r["pid_lo"]))):
            st, en = int(r["start"]), int(r["end"])
            if not (st < t2 and t1 < en):
                continue
            if pid is not None and p != pid:
                continue
            out.add((p, q, st, en))
    return out


def test_oracle_queries_match_ground_truth(built):
    """Object queries over a block without over-long meetings find exactly
    the directed keys of the object in the window; box queries over the whole
    map find every key; a box query's matches are those whose decoded box
    meets the box."""
    import oracle
    from stcdb_gb300.pipeline import QUERY_BOX, QUERY_DTYPE, QUERY_OBJECT
    rng = np.random.default_rng(21)
    mp = np.array([-87.9412, 41.6437, -87.80, 41.75])
    m = _meetings(rng, 3000, 8000, 5000, 5900, mp)
    lo = oracle.LsmOracle(3000, 1000, 16, 100.0, 5000, mp, 1 << 20)
    lo.append(m)
    lo.flush(5900)
    blocks = [lo.read()]
    qs = np.zeros(40, QUERY_DTYPE)
    pids = rng.choice(np.concatenate([m["pid_lo"], m["pid_hi"]]), 30)
    for i in range(30):
        qs[i]["kind"], qs[i]["pid"] = QUERY_OBJECT, pids[i]
        a = int(rng.integers(4990, 5900))
        qs[i]["t_start"], qs[i]["t_end"] = (a, a + int(rng.integers(1, 400))) if i % 3 else (0, 0xFFFFFFFF)
    for i in range(30, 40):
        qs[i]["kind"], qs[i]["t_start"], qs[i]["t_end"] = QUERY_BOX, 0, 0xFFFFFFFF
        if i == 30:
            qs[i]["box"] = mp
        else:
            x, y = mp[0] + rng.random() * (mp[2] - mp[0]), mp[1] + rng.random() * (mp[3] - mp[1])
            qs[i]["box"] = (x, y, x + 0.005, y + 0.004)
    res = oracle.query_blocks(blocks, qs)
    for i in range(30):
        got = {(int(r["pid"]), int(r["target"]), int(r["start"]), int(r["end"])) for r in res[i]}
        assert got == _truth(m, pid=int(qs[i]["pid"]), t1=int(qs[i]["t_start"]), t2=int(qs[i]["t_end"])), i
    assert len(res[30]) == 2 * len(m)
    for i in range(31, 40):
        b = qs[i]["box"]
        for r in res[i]:
            x0, y0, x1, y1 = r["mbr"]
            assert not (b[0] > x1 or b[2] < x0 or b[1] > y1 or b[3] < y0)
        assert set(map(tuple, res[i][["pid", "target", "end"]].tolist())) <= \
            set(map(tuple, res[30][["pid", "target", "end"]].tolist()))


def test_reference_layout_fixture():
    """The struct layout the block files use (printed by the reference's own
    headers): CTF 80 bytes, CTB 128 with the oversize buffer at 72."""
    lay = {}
    for line in open(os.path.join(HERE, "golden", "ref_layout.txt")):
        name, a, b = line.split()
        lay[name] = (int(a), int(b))
    assert lay["CTF"][0] == 80 and lay["CTB"][0] == 128 and lay["oversize_buffer"][0] == 48
    assert lay["CTF.key_bit"][0] == 56 and lay["CTF.y_grid"][0] == 74 and lay["CTF.ctf_bitmap_size"][0] == 52
    assert lay["CTB.o_buffer"][0] == 72 and lay["oversize_buffer.start_time_min"][0] == 32
