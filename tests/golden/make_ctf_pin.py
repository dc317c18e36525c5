"""Generates tests/golden/ctf_pin.npz from the reference's own host code for
the CTF encoding of a flushed block.

Runs oracle/_ref/ref_ctf (oracle/ref_ctf.cpp linked with the reference's
unmodified tracing/step_merge.cpp, built by oracle/build_ref.sh), which calls
CTF::get_ctf_bits, CTF::serial_mbr, CTF::serial_key,
oversize_buffer::write_o_buffer and, on the packed keys, CTF::parse_key,
CTF::new_parse_mbr and CTF::ctf_get_key_oid on seeded random cases, and
stores inputs and outputs; and the byte layout of the reference's CTF, CTB
and oversize_buffer objects (ref_layout.txt), which its block files hold raw.
Only this script needs the reference checkout.

    python tests/golden/make_ctf_pin.py
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# (map box, num_objects, max_meet_time) sets; the map is a street-grid
# window like the ones the trace generator produces, padded by 100 m.
SETS = [
    ((-87.9412, 41.6437, -87.4556, 42.0060), 10_000_000, 4096),
    ((-87.9412, 41.6437, -87.9000, 41.6800), 100_000, 1000),
    ((-87.9412, 41.6437, -87.5000, 41.9000), 50_000_000, 4096),
]
CASES_PER_SET = 400
OBOXES = 300


def make_cases(rng, mp, n):
    """CTF boxes from a few metres to the whole map, a key box inside each."""
    W, H = mp[2] - mp[0], mp[3] - mp[1]
    cm = np.zeros((n, 4), np.float32)
    bx = np.zeros((n, 4), np.float32)
    for i in range(n):
        fx, fy = 10 ** rng.uniform(-4.5, 0), 10 ** rng.uniform(-4.5, 0)
        if i % 50 == 0:
            fx, fy = 1.0, 1.0
        w, h = W * fx, H * fy
        x0 = mp[0] + rng.uniform(0, W - w)
        y0 = mp[1] + rng.uniform(0, H - h)
        c = np.array([x0, y0, x0 + w, y0 + h], np.float32)
        if c[2] <= c[0] or c[3] <= c[1]:
            c[2] = np.nextafter(c[0], np.float32(np.inf))
            c[3] = np.nextafter(c[1], np.float32(np.inf))
        cm[i] = c
        kind = i % 4
        if kind == 0:
            b = c.copy()                                   # the box that set the CTF box
        else:
            u = np.sort(rng.uniform(0, 1, 2))
            v = np.sort(rng.uniform(0, 1, 2))
            if kind == 3:
                u[1] = u[0]                                # zero width
            b = np.array([c[0] + (c[2] - c[0]) * u[0], c[1] + (c[3] - c[1]) * v[0],
                          c[0] + (c[2] - c[0]) * u[1], c[1] + (c[3] - c[1]) * v[1]], np.float32)
            b = np.clip(b, [c[0], c[1], c[0], c[1]], [c[2], c[3], c[2], c[3]]).astype(np.float32)
        bx[i] = b
    return cm, bx


def main():
    import oracle
    oracle.build(reference=True)
    ref = oracle.REF_CTF
    if not os.path.exists(ref):
        raise SystemExit("reference harness not built (no reference checkout here)")
    rng = np.random.default_rng(2024)
    out = {}
    for si, (mp, nobj, mmt) in enumerate(SETS):
        cm, bx = make_cases(rng, mp, CASES_PER_SET)
        sid = rng.integers(0, 102, CASES_PER_SET).astype(np.uint64)
        pid = rng.integers(0, nobj, CASES_PER_SET).astype(np.uint64)
        pid_field = (sid << np.uint64(26)) | pid
        target = rng.integers(0, nobj, CASES_PER_SET).astype(np.uint32)
        dur = rng.integers(0, mmt + 1, CASES_PER_SET).astype(np.uint32)
        end = rng.integers(0, mmt, CASES_PER_SET).astype(np.uint32)
        # oversize boxes strictly inside the map
        W, H = mp[2] - mp[0], mp[3] - mp[1]
        ob = np.zeros((OBOXES, 4), np.float32)
        for i in range(OBOXES):
            w, h = W * rng.uniform(0, 0.05), H * rng.uniform(0, 0.05)
            x0, y0 = mp[0] + rng.uniform(0.001, 0.94) * W, mp[1] + rng.uniform(0.001, 0.94) * H
            ob[i] = (x0, y0, x0 + w, y0 + h)
        odur = rng.integers(0, 5000, OBOXES).astype(np.uint32)
        oend = rng.integers(5000, 9000, OBOXES).astype(np.uint32)
        etm = 100
        with tempfile.TemporaryDirectory() as d:
            ip, op = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
            with open(ip, "wb") as f:
                f.write(np.asarray(mp, np.float64).tobytes())
                f.write(struct.pack("<III", nobj, mmt, CASES_PER_SET))
                for i in range(CASES_PER_SET):
                    f.write(cm[i].tobytes() + bx[i].tobytes())
                    f.write(struct.pack("<QIII", int(pid_field[i]), int(target[i]), int(dur[i]), int(end[i])))
                f.write(struct.pack("<II", etm, OBOXES))
                for i in range(OBOXES):
                    f.write(ob[i].tobytes() + struct.pack("<II", int(odur[i]), int(oend[i])))
            subprocess.run([ref, ip, op], check=True)
            raw = open(op, "rb").read()
        rec = np.dtype([("bits", "<u2", (10,)), ("bitmap_size", "<u4"), ("value_mbr", "<u8"),
                        ("key_lo", "<u8"), ("key_hi", "<u8"), ("dec", "<u4", (4,)), ("dec_vm", "<u8"),
                        ("dec_box", "<f8", (4,))])
        n = CASES_PER_SET * rec.itemsize
        r = np.frombuffer(raw[:n], rec)
        tail = raw[n:]
        obm = np.frombuffer(tail[:8192], np.uint8)
        osmin, osmax = struct.unpack("<II", tail[8192:8200])
        p = f"s{si}_"
        out.update({p + "map": np.asarray(mp, np.float64), p + "meta": np.array([nobj, mmt, etm], np.uint32),
                    p + "ctf_mbr": cm, p + "box": bx, p + "pid_field": pid_field, p + "target": target,
                    p + "dur": dur, p + "end": end, p + "bits": r["bits"].copy(),
                    p + "bitmap_size": r["bitmap_size"].copy(), p + "value_mbr": r["value_mbr"].copy(),
                    p + "key_lo": r["key_lo"].copy(), p + "key_hi": r["key_hi"].copy(),
                    p + "dec": r["dec"].copy(), p + "dec_vm": r["dec_vm"].copy(), p + "dec_box": r["dec_box"].copy(),
                    p + "oboxes": ob, p + "odur": odur, p + "oend": oend, p + "o_bitmap": obm.copy(),
                    p + "o_times": np.array([osmin, osmax], np.uint32)})
    np.savez_compressed(os.path.join(HERE, "ctf_pin.npz"), **out)
    print("wrote ctf_pin.npz with", len(SETS), "sets")
    # byte layout of the reference's CTF / CTB / oversize_buffer objects
    layout = subprocess.run([ref, "layout"], check=True, capture_output=True, text=True).stdout
    with open(os.path.join(HERE, "ref_layout.txt"), "w") as f:
        f.write(layout)
    print("wrote ref_layout.txt")


if __name__ == "__main__":
    main()
