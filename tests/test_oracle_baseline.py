"""The benchmark-configuration fixtures (tests/golden/baseline_*.npz) match
the oracle as it stands: one right-hand side of each case is recomputed on
the CPU (the 3-D case takes a few seconds)."""
import tempfile

import numpy as np
import pytest

import baseline_cases as bc


@pytest.mark.parametrize("name", ["c1", "c2", "c3"])
def test_fixture_rhs_matches_oracle(name):
    fx = bc.load(name)
    with tempfile.TemporaryDirectory() as tmp:
        o = bc.oracle_tank(bc.spec(name, tmp))
    y = bc.modal_state(o.n1, o.n2, o.n3_add, o.omega, frac=bc.ENVELOPE.get(name, 0.2))
    k = o.solveHOS2({key: a for key, a in zip(bc.KEYS, y)}, bc.RHS_DT, bc.RHS_T)
    for i, key in enumerate(bc.KEYS):
        if name in bc.SAMPLED:
            bc.compare_summary(fx, "rhs_" + key, k[key], 100 + i, 1e-13)
        else:
            ref = fx["rhs_" + key]
            assert np.max(np.abs(k[key] - ref)) <= 1e-13 * max(np.max(np.abs(ref)), 1e-300), key


def test_summary_detects_a_planted_error():
    """The sampled record of a large array catches a change of one part in
    1e9 spread over the array and a single changed entry in the sample."""
    rng = np.random.default_rng(0)
    a = rng.standard_normal(200_000)
    fx = bc.summarize("x", a, 5)
    bc.compare_summary(fx, "x", a, 5, 1e-14)
    with pytest.raises(AssertionError):
        bc.compare_summary(fx, "x", a * (1 + 1e-9), 5, 1e-10)
    b = a.copy()
    b[fx["x_idx"][7]] += 1e-6
    with pytest.raises(AssertionError):
        bc.compare_summary(fx, "x", b, 5, 1e-10)
