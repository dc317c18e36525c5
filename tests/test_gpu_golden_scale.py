"""The GPU pipeline against fixtures made at the benchmark's own scale by the
reference's single-threaded CPU implementation (tests/golden/make_golden_scale.py):
the 10M-object uniform benchmark workload (its first 12 steps), the hotspot
model at 1M objects (the hotspot-1M workload) and its density-preserving
downscale to 100k objects. Per step the emitted meetings (pid_lo, pid_hi,
start, end) must hash-identically equal the reference's, with the same count,
and the step must make the same number of checking units."""
import hashlib
import os

import numpy as np
import pytest

from golden.make_golden import stc_config, trace_config, tuples_digest
from golden.make_golden_scale import SCALE_CASES, fixture_path
from stcdb_gb300.pipeline import Pipeline

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["hotspot_100k_scaled", "hotspot_1m", "uniform_10m"])
def test_gpu_matches_reference_at_scale(built_cuda, name):
    import torch
    from stcdb_gb300.tracegen import DeviceTraceGenerator
    case = SCALE_CASES[name]
    fx = dict(np.load(fixture_path(name)))
    steps, n = case["steps"], case["trace"]["num_objects"]
    # positions from the device walker, which is bit-identical to the host
    # walker that fed the reference; the digest of all steps proves it here
    with DeviceTraceGenerator(trace_config(case["trace"]), 0) as gen:
        mbr = gen.map_box(100.0)
        xy = torch.empty((steps, n, 2), dtype=torch.float64, device="cuda:0")
        gen.next_into(xy.data_ptr(), steps)
    assert np.array_equal(mbr, fx["mbr"])
    h = hashlib.sha256()
    for t in range(steps):
        h.update(np.ascontiguousarray(xy[t].cpu().numpy(), dtype="<f8").tobytes())
    assert h.hexdigest() == str(fx["trace_sha256"]), "positions differ from the fixture's trace"
    with Pipeline(stc_config(case), mbr, xy[0].cpu().numpy()) as p:
        for t in range(steps):
            p.step_device(xy[t].data_ptr(), t)
            m = p.drain()
            s = p.stats()
            r = np.stack([m["pid_lo"], m["pid_hi"], m["start"], m["end"]], 1) if len(m) else np.zeros((0, 4))
            assert s.checking_units == fx["units"][t], f"step {t}: checking units"
            assert len(r) == fx["counts"][t], f"step {t}: {len(r)} vs reference {fx['counts'][t]}"
            assert tuples_digest(r) == str(fx["digests"][t]), f"step {t}: meeting set differs"
            assert s.ambiguous_tests == 0
    assert fx["counts"].sum() > 0
