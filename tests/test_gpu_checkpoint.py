"""Checkpoint / restore (stc_checkpoint, stc_restore): a run checkpointed
mid-way, destroyed and restored from the file continues exactly as the
uninterrupted run -- the same meetings every step (including those still
undrained at the checkpoint), the same memtable and the same flushed
blocks -- and a damaged file is refused."""
import os

import numpy as np
import pytest

from stcdb_gb300.pipeline import Pipeline, StcConfig, StcError
from stcdb_gb300.tracegen import hotspot_grid

from parity import as_tuples, trace_and_box

pytestmark = pytest.mark.gpu

STEPS, CUT = 14, 6


def _cfg():
    return StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, max_meet_time=6, grid_capacity=50,
                     grid_amplify=1.2, num_meeting_buckets=1_500_000, kv_restriction=60_000, ctf_count=16)


def _record(pipe, t, out, drain=True):
    st = pipe.stats()
    rec = {"memtable": st.memtable_keys, "flushes": st.flushes, "leaves": st.leaves,
           "nodes": st.schema_nodes, "live": st.taken_buckets}
    if drain:
        rec["meetings"] = as_tuples(pipe.drain()).tobytes()
    out[t] = rec
    return st


def test_restore_continues_the_run(built_cuda, tmp_path):
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=11)
    tr, mbr = trace_and_box(tc, STEPS)
    want, blocks_a = {}, {}
    with Pipeline(_cfg(), mbr, tr[0]) as a:
        seen = 0
        for t in range(STEPS):
            a.step(tr[t], t)
            st = _record(a, t, want)
            if st.flushes > seen:
                seen = st.flushes
                info, b = a.read_ctb()
                blocks_a[t] = (info.as_dict(), {k: v.tobytes() for k, v in b.items()})
    assert len(blocks_a) >= 2 and any(t > CUT for t in blocks_a)

    path = str(tmp_path / "run.ckpt")
    with Pipeline(_cfg(), mbr, tr[0]) as b:
        for t in range(CUT + 1):
            b.step(tr[t], t)
            if t < CUT:
                b.drain()
        b.checkpoint(path)  # step CUT's meetings are still undrained
    got, blocks_b = {}, {}
    r = Pipeline.restore(path)
    try:
        assert r.cfg == _cfg().resolved()
        _record(r, CUT, got)
        seen = r.stats().flushes
        for t in range(CUT + 1, STEPS):
            r.step(tr[t], t)
            st = _record(r, t, got)
            if st.flushes > seen:
                seen = st.flushes
                info, blk = r.read_ctb()
                blocks_b[t] = (info.as_dict(), {k: v.tobytes() for k, v in blk.items()})
    finally:
        r.close()
    for t in range(CUT, STEPS):
        assert got[t] == want[t], f"step {t} differs after the restore"
    for t, blk in blocks_b.items():
        assert blk == blocks_a[t], f"block flushed at step {t} differs"
    assert blocks_b

    # a damaged file is refused
    data = bytearray(open(path, "rb").read())
    data[len(data) // 2] ^= 0x5A
    bad = str(tmp_path / "bad.ckpt")
    open(bad, "wb").write(bytes(data))
    with pytest.raises(StcError):
        Pipeline.restore(bad)
    with pytest.raises(StcError):
        Pipeline.restore(str(tmp_path / "missing.ckpt"))
    assert os.path.getsize(path) > 1_500_000 * 32
