"""GPU pipeline against the fixtures produced by the reference's own CPU
implementation (tests/golden/make_golden.py): per-step meeting sets
(pid_lo, pid_hi, start, end) hash-identical, and the same checking units."""
import os

import numpy as np
import pytest

from golden.make_golden import CASES, make_trace, stc_config, trace_digest, tuples_digest
from stcdb_gb300.pipeline import FLAG_SERIAL_SCHEMA, Pipeline

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("name,flags,slices", [("c1_uniform_100k", 0, 0), ("uniform_20k_small", 0, 0),
                                               ("hotspot_30k", 0, 0), ("hotspot_30k", FLAG_SERIAL_SCHEMA, 0),
                                               ("hotspot_30k", 0, 5)])
def test_gpu_matches_reference(built_cuda, name, flags, slices):
    from dataclasses import replace
    case = CASES[name]
    fx = dict(np.load(os.path.join(HERE, "golden", name + ".npz")))
    trace, mbr = make_trace(case)
    assert trace_digest(trace) == str(fx["trace_sha256"]), "trace generator differs on this host"
    cfg = replace(stc_config(case), flags=flags, step_slices=slices)
    with Pipeline(cfg, mbr, trace[0]) as p:
        for t in range(case["steps"]):
            p.step(trace[t], t)
            m = p.drain()
            s = p.stats()
            r = np.stack([m["pid_lo"], m["pid_hi"], m["start"], m["end"]], 1) if len(m) else np.zeros((0, 4))
            assert len(r) == fx["counts"][t], f"step {t}: {len(r)} vs reference {fx['counts'][t]}"
            assert s.checking_units == fx["units"][t], f"step {t}: checking units"
            assert tuples_digest(r) == str(fx["digests"][t]), f"step {t}: meeting set differs"
            assert s.ambiguous_tests == 0
