"""The seeded trace generator is deterministic and keeps objects on the map."""
import numpy as np

from stcdb_gb300.tracegen import TraceGenerator, hotspot_grid, uniform_grid


def test_deterministic(built):
    a = TraceGenerator(hotspot_grid(5000, n_hotspots=10, seed=4)).steps(5)
    b = TraceGenerator(hotspot_grid(5000, n_hotspots=10, seed=4)).steps(5)
    c = TraceGenerator(hotspot_grid(5000, n_hotspots=10, seed=5)).steps(5)
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def test_inside_map_and_speed(built):
    g = TraceGenerator(uniform_grid(20000, seed=2))
    tr = g.steps(20)
    box = g.map_box(0.0)
    assert (tr[..., 0] >= box[0]).all() and (tr[..., 0] <= box[2]).all()
    assert (tr[..., 1] >= box[1]).all() and (tr[..., 1] <= box[3]).all()
    # metres moved per step stay within the speed range (corners cut distance short)
    dpml0 = 1.2020818910678718e-05
    dpm_lat = 360.0 / 40076000.0
    d = np.hypot(np.diff(tr[..., 0], axis=0) / dpml0, np.diff(tr[..., 1], axis=0) / dpm_lat)
    assert d.max() <= 15.0 + 1e-6
