"""The filtering branch of check_slope (initial_condition.f90:687-716) on the
GPU against the oracle: a right-hand side of a steep free surface
(max |eta_x| > 8 on the dealiased grid) makes check_slope cut the modes
beyond 0.7 n of eta and phis (filtering.f90:37-86, 334-360)."""
import numpy as np
import pytest

import cases
from oracle.hos_oracle import Tank as OTank

pytestmark = pytest.mark.gpu

KEYS = ("G1", "G2", "a_add_1", "a_add_2", "a_add_ramp", "a_add_3", "a1st", "eta1st", "a2nd", "eta2nd")


def _steep_case(name, amp_hi):
    case = cases.ALL[name]
    o = OTank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"])
    n1, n2, n3a = o.n1, o.n2, o.n3_add
    G1 = np.zeros((n1, n2))
    G1[3, 0] = 0.05
    G1[n1 - 5, 0] = amp_hi                   # slope amp_hi * kx(n1 - 5) along x
    if n2 > 1:
        G1[2, 1] = 0.02
        G1[1, n2 - 3] = amp_hi                # and along y
    G2 = np.zeros((n1, n2))
    G2[2, 0] = 0.01
    G2[n1 - 6, 0] = 0.002
    y = [G1, G2] + [np.zeros((n3a, n2)) for _ in range(4)] + [np.zeros((n1, n2)) for _ in range(4)]
    return case, o, y


@pytest.mark.parametrize("name,amp", [("reg1d", 0.6), ("reg3d", 1.0)])
def test_check_slope_filters_like_oracle(lib, name, amp):
    import hosnwt
    case, o, y = _steep_case(name, amp)
    eta = o.fourier.F2S(y[0])
    phis = o.fourier.F2S(y[1] / np.where(o.omega > 0, o.omega, 1.0))
    # oracle: one right-hand side sets etax / etay, then the filter
    o.solveHOS2({k: a.copy() for k, a in zip(KEYS, y)}, 0.0, 0.0)
    assert np.max(np.abs(o.etax)) > 8.0
    o.eta, o.phis = eta.copy(), phis.copy()
    hit = o.check_slope()
    assert hit
    g = hosnwt.Tank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"])
    g.solveHOS2(y, 0.0, 0.0, 0.0, 0.0)
    d = g.diagnostics()
    assert abs(d[3] - np.max(np.abs(o.etax))) <= 1e-10 * np.max(np.abs(o.etax))
    if case["n2"] > 1:
        assert abs(d[4] - np.max(np.abs(o.etay))) <= 1e-10 * np.max(np.abs(o.etay))
    g.set_state(eta, phis)
    f = g.check_slope()
    assert f == (3 if case["n2"] > 1 else 1)
    ge, gp, _ = g.get_state()
    g.close()
    for got, ref in ((ge, o.eta), (gp, o.phis)):
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    # the cut removed the steep modes
    m = o.fourier.S2F(ge)
    assert np.max(np.abs(m[int(0.7 * case["n1"]):, :])) <= 1e-12 * np.max(np.abs(m))
