"""The device trace generator (stc_trace_dev_*) writes the host generator's
positions bit for bit: the same start positions, the same walk over many
steps whether written one step per call or many, the same map box."""
import numpy as np
import pytest

from stcdb_gb300.tracegen import DeviceTraceGenerator, TraceConfig, TraceGenerator, hotspot_grid, uniform_grid

pytestmark = pytest.mark.gpu

CONFIGS = [
    uniform_grid(30000, seed=3),
    hotspot_grid(40000, n_hotspots=50, seed=9, grid_n=30, box_m=3000.0, sigma_m=100.0),
    # a 4x4 grid walked at up to 90 m/s: several turns per step, boundary nodes
    TraceConfig(num_objects=5000, grid_n=4, box_m=60.0, jitter_m=5.0, speed_lo=20.0, speed_hi=90.0,
                n_hotspots=3, hot_frac=0.5, sigma_m=10.0, seed=77),
    hotspot_grid(1_000_000, n_hotspots=1000, seed=1),
]
CHUNKS = [1, 1, 7, 16]  # steps per call: 25 steps in all


@pytest.mark.parametrize("ci", range(len(CONFIGS)))
def test_device_walk_is_the_host_walk(built_cuda, ci):
    import torch
    cfg = CONFIGS[ci]
    N = cfg.num_objects
    host = TraceGenerator(cfg)
    want = host.steps(sum(CHUNKS))
    buf = torch.empty((sum(CHUNKS), N, 2), dtype=torch.float64, device="cuda:0")
    with DeviceTraceGenerator(cfg, 0) as dev:
        assert np.array_equal(dev.map_box(100.0), host.map_box(100.0))
        t = 0
        for c in CHUNKS:
            dev.next_into(buf[t].data_ptr(), c)
            t += c
            assert dev.step == t
        assert dev.last_ms > 0.0
    got = buf.cpu().numpy()
    for s in range(t):
        assert got[s].tobytes() == want[s].tobytes(), f"step {s} differs"


def test_rejects_bad_arguments(built_cuda):
    import torch
    with pytest.raises(ValueError):
        DeviceTraceGenerator(TraceConfig(num_objects=10, grid_n=1), 0)
    with pytest.raises(ValueError):
        DeviceTraceGenerator(TraceConfig(num_objects=0), 0)
    buf = torch.empty(2 * 100 + 2, dtype=torch.float64, device="cuda:0")
    with DeviceTraceGenerator(TraceConfig(num_objects=100), 0) as dev:
        with pytest.raises(RuntimeError):
            dev.next_into(buf.data_ptr() + 8)  # positions must start on 16 bytes
        assert dev.step == 0
        dev.next_into(buf.data_ptr())
        assert dev.step == 1
