"""stc_step_window (each step replayed from a captured CUDA graph) against the
plain step-by-step pipeline: uneven windows, pageable and page-locked host
input and device input, flushes
inside windows (the graph is captured again after each), a change of the
slice count between windows. Meetings, statistics and every flushed block
must be identical."""
import numpy as np
import pytest

from stcdb_gb300.pipeline import FLAG_COPY_INPUT, MEETING_DTYPE, Pipeline, StcConfig
from stcdb_gb300.tracegen import hotspot_grid

from parity import trace_and_box

pytestmark = pytest.mark.gpu


def _rows(meetings):
    a = np.ascontiguousarray(meetings).view(np.uint32).reshape(-1, MEETING_DTYPE.itemsize // 4)
    return a[np.lexsort(a.T[::-1])] if len(a) else a


def _blocks(p):
    n = p.stats().flushes
    out = []
    for i in range(max(0, n - 8), n):  # the context keeps the last 8 blocks
        info, arrays = p.read_block(i)
        out.append((info.as_dict(), {k: v.view(np.uint8).tobytes() for k, v in arrays.items()}))
    return out


# replayed graphs; direct launches, whose descent reads page-locked host
# input from the host pages; direct launches with that input copied in
# (STC_FLAG_COPY_INPUT)
@pytest.mark.parametrize("graphs,flags", [(1, 0), (2, 0), (2, FLAG_COPY_INPUT)])
def test_windows_match_plain_steps(built_cuda, graphs, flags):
    import torch
    steps = 24
    tc = hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=11)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, max_meet_time=6, grid_capacity=50,
                    grid_amplify=1.2, num_meeting_buckets=1_500_000, kv_restriction=60_000, ctf_count=16)
    tr, mbr = trace_and_box(tc, steps)
    tr = np.ascontiguousarray(tr, dtype=np.float64)

    plain = Pipeline(cfg, mbr, tr[0])
    try:
        got_plain = []
        for t in range(steps):
            plain.step(tr[t], t)
            got_plain.append(plain.drain())
        ps = plain.stats()
        plain_blocks = _blocks(plain)
    finally:
        plain.close()

    from dataclasses import replace
    win = Pipeline(replace(cfg, window_graphs=graphs, flags=flags), mbr, tr[0])
    dev = torch.from_numpy(tr).cuda()
    # page-locked host input (read by the descent, or copied by DMA) besides
    # pageable host input (staged by the driver)
    pinned = torch.from_numpy(tr).pin_memory().numpy()
    try:
        got_win = []
        t0 = 0
        # (steps, slices, input: pageable host, page-locked host, device)
        for w, slices, src in [(1, 1, "host"), (4, 1, "device"), (7, 3, "pinned"), (2, 3, "device"), (6, 1, "host"),
                               (4, 2, "pinned")]:
            win.set_step_slices(slices)
            out = np.empty(2_000_000, MEETING_DTYPE)
            if src == "device":
                got = win.step_window((dev[t0].data_ptr(), w), t0, out)
            elif src == "pinned":
                got = win.step_window(pinned[t0:t0 + w], t0, out)
            else:
                got = win.step_window(tr[t0:t0 + w], t0, out)
            got_win.append(got.copy())
            t0 += w
        assert t0 == steps
        ws = win.stats()
        win_blocks = _blocks(win)
    finally:
        win.close()

    a, b = _rows(np.concatenate(got_plain)), _rows(np.concatenate(got_win))
    assert len(a) > 0 and a.shape == b.shape and np.array_equal(a, b)
    assert ps.flushes >= 2 and ws.flushes == ps.flushes
    assert ws.memtable_keys == ps.memtable_keys and ws.hits == ps.hits and ws.leaves == ps.leaves
    assert len(win_blocks) == len(plain_blocks)
    for (gi, ga), (pi, pa) in zip(win_blocks, plain_blocks):
        assert gi == pi
        for k in pa:
            assert ga[k] == pa[k], f"block array {k} differs"


def _plain_run(cfg, tr, mbr, steps):
    p = Pipeline(cfg, mbr, tr[0])
    try:
        got = []
        for t in range(steps):
            p.step(tr[t], t)
            got.append(p.drain().copy())
        return got
    finally:
        p.close()


def test_window_output_too_small_reports_capacity(built_cuda):
    """A full output buffer stops the window with STC_ERR_CAPACITY; the
    context stays usable, the meetings that did not fit stay pending, and
    everything equals plain steps up to the last step that ran."""
    from stcdb_gb300.pipeline import StcError
    tr, mbr = trace_and_box(hotspot_grid(20000, n_hotspots=20, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=4), 12)
    tr = np.ascontiguousarray(tr, dtype=np.float64)
    cfg = StcConfig(num_objects=20000, reach_distance=10.0, min_meet_time=3, grid_capacity=50,
                    num_meeting_buckets=1_000_000)
    plain = _plain_run(cfg, tr, mbr, 12)
    cum = np.cumsum([len(m) for m in plain])
    fill = int(np.argmax(cum > 1))  # the step whose meetings overflow a one-record buffer
    assert cum[fill] > 1
    p = Pipeline(cfg, mbr, tr[0])
    try:
        out = np.empty(1, MEETING_DTYPE)
        with pytest.raises(StcError) as e:
            p.step_window(tr, 0, out)
        assert e.value.status == 3  # STC_ERR_CAPACITY
        last = p.stats().step
        assert fill <= last <= fill + 1  # at most one step beyond the one that filled the buffer
        rest = p.drain()
        got = np.concatenate([out[:1], rest])
        want = np.concatenate(plain[:last + 1])
        assert np.array_equal(_rows(got), _rows(want))
        # the context goes on: the remaining steps equal the plain run's
        more = p.step_window(tr[last + 1:], last + 1, np.empty(2_000_000, MEETING_DTYPE))
        assert np.array_equal(_rows(more), _rows(np.concatenate(plain[last + 1:])))
    finally:
        p.close()


@pytest.mark.parametrize("graphs", [1, 2])
def test_window_small_emit_buffer(built_cuda, graphs):
    """A window whose emit buffer passes half full holds the pipeline for a
    step and empties the buffer; the meetings equal the plain run's."""
    from dataclasses import replace
    steps = 20
    tr, mbr = trace_and_box(hotspot_grid(30000, n_hotspots=30, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=6),
                            steps)
    tr = np.ascontiguousarray(tr, dtype=np.float64)
    cfg = StcConfig(num_objects=30000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.2,
                    num_meeting_buckets=1_500_000, kv_restriction=40_000, ctf_count=16)
    plain = _plain_run(cfg, tr, mbr, steps)
    peak = max(len(m) for m in plain)
    assert peak > 0
    small = replace(cfg, emit_capacity=3 * peak, window_graphs=graphs)
    p = Pipeline(small, mbr, tr[0])
    try:
        got = p.step_window(tr, 0, np.empty(2_000_000, MEETING_DTYPE)).copy()
        assert p.stats().pending == 0
    finally:
        p.close()
    assert np.array_equal(_rows(got), _rows(np.concatenate(plain)))


def test_page_locked_input_path(built_cuda):
    """Without graphs, page-locked host input is read by each step's descent
    (no input copies: window_copy_ms stays 0); with STC_FLAG_COPY_INPUT, or
    while a request loop is attached, it is copied in as before."""
    import torch
    from dataclasses import replace
    steps = 8
    tc = hotspot_grid(20000, n_hotspots=20, box_m=3000.0, grid_n=16, sigma_m=120.0, seed=12)
    cfg = StcConfig(num_objects=20000, reach_distance=10.0, min_meet_time=3, grid_capacity=50, grid_amplify=1.5,
                    num_meeting_buckets=1_000_000, kv_restriction=50_000, window_graphs=2)
    tr, mbr = trace_and_box(tc, steps)
    pinned = torch.from_numpy(np.ascontiguousarray(tr, dtype=np.float64)).pin_memory().numpy()
    out = np.empty(1_000_000, MEETING_DTYPE)
    for flags, serve, copies in [(0, False, False), (FLAG_COPY_INPUT, False, True), (0, True, True)]:
        p = Pipeline(replace(cfg, flags=flags), mbr, tr[0])
        srv = p.server() if serve else None
        try:
            p.step_window(pinned[0:2], 0, out)  # the first window after the context's own step 0
            p.step_window(pinned[2:steps], 2, out)
            ms = p.stats().window_copy_ms
            assert (ms > 0) == copies, (flags, serve, ms)
        finally:
            if srv is not None:
                srv.stop()
            p.close()
