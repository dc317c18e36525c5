"""The oracle (C restatement of the reference CPU path) against fixtures
generated by the reference's own CPU implementation (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from golden.make_golden import CASES, make_trace, stc_config, trace_digest, tuples_digest

HERE = os.path.dirname(os.path.abspath(__file__))


def load(name):
    return dict(np.load(os.path.join(HERE, "golden", name + ".npz")))


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference(built, name):
    import oracle
    case = CASES[name]
    fx = load(name)
    trace, mbr = make_trace(case)
    assert trace_digest(trace) == str(fx["trace_sha256"]), "trace generator is not reproducible"
    cfg = stc_config(case)
    o = oracle.Oracle(cfg, mbr, trace[0])
    rows = []
    for t in range(case["steps"]):
        m = o.step(trace[t], t)
        r = np.stack([m["pid_lo"], m["pid_hi"], m["start"], m["end"]], 1) if len(m) else np.zeros((0, 4), np.uint32)
        assert len(r) == fx["counts"][t], f"step {t}: {len(r)} vs reference {fx['counts'][t]}"
        assert o.stats().checking_units == fx["units"][t], f"step {t}: checking units differ"
        assert tuples_digest(r) == str(fx["digests"][t]), f"step {t}: meeting set differs"
        rows.append(r)
    o.close()
    if "rows" in fx:
        # the oracle also reproduces the reference's emission order (bucket order)
        assert np.array_equal(np.concatenate(rows).astype(np.uint32), fx["rows"])


def test_fixture_shapes():
    fx = load("c1_uniform_100k")
    assert fx["counts"].shape == (100,) and fx["counts"].sum() == len(fx["rows"]) > 10000
    assert fx["counts"][:6].sum() == 0  # nothing can end before min_meet_time + 1 steps


def test_oracle_matches_reference_scaled_hotspots(built):
    """The density-preserving 100k downscale of the hotspot model (fixture
    from tests/golden/make_golden_scale.py): dense leaves at the minimum
    width, a loaded table, splits and merges."""
    import oracle
    from golden.make_golden_scale import SCALE_CASES, fixture_path
    case = SCALE_CASES["hotspot_100k_scaled"]
    fx = dict(np.load(fixture_path("hotspot_100k_scaled")))
    trace, mbr = make_trace(case)
    assert trace_digest(trace) == str(fx["trace_sha256"])
    o = oracle.Oracle(stc_config(case), mbr, trace[0])
    try:
        for t in range(case["steps"]):
            m = o.step(trace[t], t)
            r = np.stack([m["pid_lo"], m["pid_hi"], m["start"], m["end"]], 1) if len(m) else np.zeros((0, 4))
            assert len(r) == fx["counts"][t], f"step {t}"
            assert o.stats().checking_units == fx["units"][t], f"step {t}: checking units differ"
            assert tuples_digest(r) == str(fx["digests"][t]), f"step {t}: meeting set differs"
    finally:
        o.close()


def test_scale_fixture_shapes():
    from golden.make_golden_scale import SCALE_CASES, fixture_path
    for name, case in SCALE_CASES.items():
        fx = dict(np.load(fixture_path(name)))
        steps = case["steps"]
        assert fx["counts"].shape == (steps,) and fx["units"].shape == (steps,) and fx["digests"].shape == (steps,)
        assert fx["counts"][:case["cfg"]["min_meet_time"] + 1].sum() == 0  # nothing ends before min_meet + 1
        assert fx["counts"].sum() > 0 and (fx["units"] >= case["trace"]["num_objects"]).all()
