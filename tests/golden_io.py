"""Golden fixtures of the oracle (tests/golden/*.npz): one right-hand side
on a seeded state and one RK4(5) step from the initial condition of each
small case.  tests/golden/make_golden.py writes them."""
import os

import numpy as np

from oracle.hos_oracle import Tank

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def seeded_state(o, seed=11, amp=1e-3):
    rng = np.random.default_rng(seed)
    n1, n2, n3a = o.n1, o.n2, o.n3_add
    decay = np.exp(-0.15 * np.arange(n1))[:, None] * np.exp(-0.3 * np.arange(n2))[None, :]
    da = np.exp(-0.2 * np.arange(n3a))[:, None] * np.ones((1, n2))
    G2 = amp * rng.standard_normal((n1, n2)) * decay * o.omega
    G2[0, 0] = 0.0
    return dict(G1=amp * rng.standard_normal((n1, n2)) * decay, G2=G2,
                a_add_1=amp * rng.standard_normal((n3a, n2)) * da, a_add_2=np.zeros((n3a, n2)),
                a_add_ramp=amp * rng.standard_normal((n3a, n2)) * da, a_add_3=np.zeros((n3a, n2)),
                a1st=amp * rng.standard_normal((n1, n2)) * decay,
                eta1st=amp * rng.standard_normal((n1, n2)) * decay,
                a2nd=np.zeros((n1, n2)), eta2nd=np.zeros((n1, n2)))


def run_fixture_case(case):
    o = Tank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"])
    out = {}
    y = seeded_state(o)
    k = o.solveHOS2({a: b.copy() for a, b in y.items()}, 0.02, 1.3)
    for key in o.STATE_KEYS:
        out["rhs_" + key] = k[key]
    o2 = Tank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"])
    res, err, deta, _ = o2.runge4_adapt2(0.0, *[a.copy() for a in o2.state_tuple()], o2.delt)
    for key, v in res.items():
        out["step_" + key] = v
    out["step_err"] = np.array([err])
    out["step_deta"] = deta
    return out


def load_fixture(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}
