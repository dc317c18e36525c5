"""The reference's block files, built from and parsed into the stc_read_ctb
layout. CTF::dump_meta writes the CTF object raw and then its bitmap,
CTF::dump_keys the packed keys, workbench::dump_CTB_meta the CTB object raw
and then the sids, oversize keys, boxes and map bitmap
(tracing/step_merge.cpp:644-658, tracing/workbench.cpp:597-635). The struct
layout is the one the reference's own headers print (golden/ref_layout.txt,
made by golden/make_ctf_pin.py). Pointer fields are written as 0 and ignored
when parsing."""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CTF_FIELDS = ("kv_count", "start_time_min", "start_time_max", "end_time_min", "end_time_max")
BIT_FIELDS = ("key_bit", "id_bit", "duration_bit", "end_bit", "low_x_bit", "low_y_bit", "edge_bit", "mbr_bit",
              "x_grid", "y_grid")


def layout() -> dict:
    lay = {}
    for line in open(os.path.join(HERE, "golden", "ref_layout.txt")):
        name, off, size = line.split()
        lay[name] = (int(off), int(size))
    return lay


def _put(buf, off, value, dtype):
    a = np.asarray(value, dtype=dtype).tobytes()
    buf[off:off + len(a)] = a


def _get(data, off, dtype, count=1):
    return np.frombuffer(data, dtype=dtype, count=count, offset=off)


def _ref_name(f):
    return "CTF_kv_capacity" if f == "kv_count" else f


def ctf_file(ctf, bitmap, lay) -> bytes:
    """CTF::dump_meta: the CTF object then its bitmap."""
    b = bytearray(lay["CTF"][0])
    _put(b, lay["CTF.ctf_mbr"][0], ctf["mbr"], "<f4")
    for f in CTF_FIELDS:
        _put(b, lay["CTF." + _ref_name(f)][0], ctf[f], "<u4")
    _put(b, lay["CTF.ctf_bitmap_size"][0], ctf["bitmap_bytes"], "<u4")
    for f in BIT_FIELDS:
        _put(b, lay["CTF." + f][0], ctf[f], "<u2")
    return bytes(b) + np.asarray(bitmap[: int(ctf["bitmap_bytes"])], np.uint8).tobytes()


def parse_ctf_file(data: bytes, lay) -> tuple:
    """(dict of the CTF's fields, its bitmap bytes)."""
    f = {"mbr": _get(data, lay["CTF.ctf_mbr"][0], "<f4", 4).copy()}
    for k in CTF_FIELDS:
        f[k] = int(_get(data, lay["CTF." + _ref_name(k)][0], "<u4")[0])
    f["bitmap_bytes"] = int(_get(data, lay["CTF.ctf_bitmap_size"][0], "<u4")[0])
    for k in BIT_FIELDS:
        f[k] = int(_get(data, lay["CTF." + k][0], "<u2")[0])
    size = lay["CTF"][0]
    return f, data[size:size + f["bitmap_bytes"]]


def ctb_file(info, blk, lay, ctb_times=(0, 0, 0, 0)) -> bytes:
    """workbench::dump_CTB_meta after straight_dump: the CTB object (its own
    times 0 unless given), sids, oversize keys, boxes, map bitmap."""
    b = bytearray(lay["CTB"][0])
    for f, v in zip(("start_time_min", "start_time_max", "end_time_min", "end_time_max"), ctb_times):
        _put(b, lay["CTB." + f][0], v, "<u4")
    ob = lay["CTB.o_buffer"][0]
    _put(b, ob + lay["oversize_buffer.oversize_kv_count"][0], info.oversize_kv_count, "<u4")
    for f in ("start_time_min", "start_time_max", "end_time_min", "end_time_max"):
        _put(b, ob + lay["oversize_buffer." + f][0], getattr(info, "o_" + f), "<u4")
    return (bytes(b) + blk["sids"].astype("<u2").tobytes() + blk["oversize_keys"].astype("<u8").tobytes() +
            blk["oversize_boxes"].astype("<f4").tobytes() + blk["oversize_bitmap"].tobytes())


def parse_ctb_file(data: bytes, lay, num_objects: int, bitmap_edge: int = 256) -> dict:
    ob = lay["CTB.o_buffer"][0]
    out = {f: int(_get(data, lay["CTB." + f][0], "<u4")[0])
           for f in ("start_time_min", "start_time_max", "end_time_min", "end_time_max")}
    n = int(_get(data, ob + lay["oversize_buffer.oversize_kv_count"][0], "<u4")[0])
    for f in ("start_time_min", "start_time_max", "end_time_min", "end_time_max"):
        out["o_" + f] = int(_get(data, ob + lay["oversize_buffer." + f][0], "<u4")[0])
    off = lay["CTB"][0]
    out["oversize_kv_count"] = n
    out["sids"] = _get(data, off, "<u2", num_objects).copy()
    off += 2 * num_objects
    out["oversize_keys"] = _get(data, off, "<u8", 2 * n).copy()
    off += 16 * n
    out["oversize_boxes"] = _get(data, off, "<f4", 4 * n).copy()
    off += 16 * n
    nb = bitmap_edge * bitmap_edge // 8
    out["oversize_bitmap"] = np.frombuffer(data[off:off + nb], np.uint8).copy()
    return out


def ctf_keys(ctf, keys) -> bytes:
    kb = int(ctf["key_bit"]) // 8
    o, n = int(ctf["key_offset"]), int(ctf["kv_count"]) * kb
    return keys[o:o + n].tobytes()


def write_block(d: str, prefix: str, index: int, info, blk, lay, raid: bool = False) -> None:
    """All files of one block: in d, or (raid) the CTB and CTF files in d/m
    and the key files in d/r0, d/r1 by CTF parity, as workbench::load_CTF_keys
    looks for them (tracing/workbench.cpp:302-305)."""
    meta = os.path.join(d, "m") if raid else d
    os.makedirs(meta, exist_ok=True)
    with open(os.path.join(meta, f"{prefix}_CTB{index}"), "wb") as f:
        f.write(ctb_file(info, blk, lay))
    for c in range(int(info.ctf_count)):
        ctf = blk["ctfs"][c]
        with open(os.path.join(meta, f"{prefix}_STcL{index}-{c}"), "wb") as f:
            f.write(ctf_file(ctf, blk["bitmaps"][c * 8192:(c + 1) * 8192], lay))
        kd = os.path.join(d, f"r{c % 2}") if raid else d
        os.makedirs(kd, exist_ok=True)
        with open(os.path.join(kd, f"{prefix}_SSTable_{index}-{c}"), "wb") as f:
            f.write(ctf_keys(ctf, blk["keys"]))
