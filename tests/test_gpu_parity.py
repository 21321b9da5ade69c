"""GPU parity of the CUDA hot path against the CPU oracle, through the C ABI.

Tolerances (FP64 end to end, different summation orders):
  transforms                    max abs diff <= 1e-13 * max|ref| (x sqrt(N) slack)
  one right-hand side           max abs diff <= 1e-10 * max|ref|
  one RK4(5) step               max abs diff <= 1e-11 * max|ref|
  time loop                     max|d eta| / Hs <= 1e-9 and probe relative error <= 1e-8
"""
import numpy as np
import pytest

import cases
from oracle.hos_oracle import Tank as OTank

pytestmark = pytest.mark.gpu


def _gtank(case, probes=None):
    import hosnwt
    return hosnwt.Tank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"],
                       case["p2"], probes=probes)


def _otank(case, probes=None):
    return OTank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"],
                 probes=probes)


def _rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


@pytest.mark.parametrize("name", ["reg1d", "reg3d", "wide3d"])
def test_transforms(lib, name):
    case = cases.ALL[name]
    g = _gtank(case)
    o = _otank(case)
    F = o.fourier
    rng = np.random.default_rng(1)
    shapes = {"n": (o.n1, o.n2), "big": (o.nd1, o.nd2), "add": (o.n3_add, o.n2)}
    for grid, shp in shapes.items():
        for csx in ("cos", "sin"):
            for csy in ("cos", "sin"):
                a = rng.standard_normal(shp)
                for direction in (1, -1):
                    if grid == "n":
                        ref = F.S2F(a, csx, csy) if direction == 1 else F.F2S(a, csx, csy)
                    elif grid == "big":
                        ref = F.S2F_big(a, csx, csy) if direction == 1 else F.F2S_big(a, csx, csy)
                    else:
                        ref = F.S2F_add(a, csx, csy) if direction == 1 else F.F2S_add(a, csx, csy)
                    got = g.transform(grid, direction, csx, csy, a)
                    assert _rel(got, ref) < 1e-13 * np.sqrt(max(shp)), (grid, csx, csy, direction)


def _state(o, rng, amp=1e-3):
    """A smooth random RK state of the oracle's shapes."""
    n1, n2, n3a = o.n1, o.n2, o.n3_add
    decay = np.exp(-0.15 * np.arange(n1))[:, None] * np.exp(-0.3 * np.arange(n2))[None, :]
    G1 = amp * rng.standard_normal((n1, n2)) * decay
    G2 = amp * rng.standard_normal((n1, n2)) * decay * o.omega
    G2[0, 0] = 0.0
    da = np.exp(-0.2 * np.arange(n3a))[:, None] * np.ones((1, n2))
    y = dict(G1=G1, G2=G2, a_add_1=amp * rng.standard_normal((n3a, n2)) * da,
             a_add_2=np.zeros((n3a, n2)), a_add_ramp=amp * rng.standard_normal((n3a, n2)) * da,
             a_add_3=np.zeros((n3a, n2)), a1st=amp * rng.standard_normal((n1, n2)) * decay,
             eta1st=amp * rng.standard_normal((n1, n2)) * decay, a2nd=np.zeros((n1, n2)),
             eta2nd=np.zeros((n1, n2)))
    if o.inp["i_wmk"] >= 2:
        y["a_add_2"] = 0.1 * amp * rng.standard_normal((n3a, n2)) * da
        y["a2nd"] = 0.1 * amp * rng.standard_normal((n1, n2)) * decay
        y["eta2nd"] = 0.1 * amp * rng.standard_normal((n1, n2)) * decay
    if o.inp["i_wmk"] == 3:
        y["a_add_3"] = 0.01 * amp * rng.standard_normal((n3a, n2)) * da
    return y


@pytest.mark.parametrize("name", ["reg1d", "reg1d_m5", "reg3d", "slosh", "jonswap1d", "wide3d", "reg1d_w2",
                                  "reg3d_w2", "reg1d_w3", "reg3d_w3"])
def test_solveHOS2(lib, name):
    case = cases.ALL[name]
    g = _gtank(case)
    o = _otank(case)
    rng = np.random.default_rng(7)
    y = _state(o, rng)
    t, dt = 1.3, 0.02
    alpha_prev, pos_top = o._alpha[0], o._pos[0][o.n3 - 1, 0]
    ref = o.solveHOS2({k: v.copy() for k, v in y.items()}, dt, t)
    got = g.solveHOS2([y[k] for k in o.STATE_KEYS], dt, t, alpha_prev, pos_top)
    for key, arr in zip(o.STATE_KEYS, got):
        r = ref[key]
        if np.max(np.abs(r)) == 0.0:
            assert np.max(np.abs(arr)) == 0.0, key
        else:
            assert _rel(arr, r) < 1e-10, (key, _rel(arr, r))


@pytest.mark.parametrize("name", ["reg1d", "reg3d", "slosh", "reg1d_w2", "reg3d_w2", "reg1d_w3", "reg3d_w3"])
def test_runge4_adapt2(lib, name):
    case = cases.ALL[name]
    o = _otank(case)
    o.advance_to(0.6, o.delt)  # a nontrivial state; the last step was accepted
    st = [a.copy() for a in o.state_tuple()]
    h = 0.8 * o.delt
    t0 = o.time_cur
    res, err, deta, _ = o.runge4_adapt2(t0, *[a.copy() for a in st], h)
    g = _gtank(case)
    # the reference's module globals alpha / pos1st hold the wavemaker law of
    # the last stage (t0); one right-hand side at t0 sets them on the device
    g.solveHOS2(_zero_state(o), 0.0, t0, 0.0, 0.0)
    g_arrs, g_err = g.runge4_adapt2(t0, *st, h)
    keys = ("eta", "phis", "a_add_1", "a_add_2", "a_add_ramp", "a_add_3", "eta1st", "eta2nd", "a1st", "a2nd")
    for k, a in zip(keys, g_arrs):
        r = res[k]
        if np.max(np.abs(r)) == 0.0:
            assert np.max(np.abs(a)) == 0.0, k
        else:
            assert _rel(a, r) < 1e-10, (k, _rel(a, r))
    assert abs(g_err - err) <= 1e-6 * max(err, 1e-12) + 1e-14


def _zero_state(o):
    n1, n2, n3a = o.n1, o.n2, o.n3_add
    return [np.zeros((n1, n2)), np.zeros((n1, n2))] + [np.zeros((n3a, n2))] * 4 + [np.zeros((n1, n2))] * 4


@pytest.mark.parametrize("name", ["reg1d", "jonswap1d", "reg3d", "reg1d_w2", "reg3d_w2", "reg1d_w3", "reg3d_w3"])
def test_time_loop_probes(lib, name):
    case = dict(cases.ALL[name])
    inp = dict(case["inp"])
    inp["T_stop"] = 2.0
    case["inp"] = inp
    probes = [(5.0, 0.0), (10.0, 0.0)] if case["n2"] == 1 else [(5.0, 5.0), (10.0, 12.0)]
    g = _gtank(case, probes)
    o = _otank(case, probes)
    recs_o = o.run()
    recs_g = g.simulate()
    assert len(recs_o) == len(recs_g)
    to = np.array([r[0] for r in recs_o])
    tg = np.array([r[0] for r in recs_g])
    assert np.max(np.abs(to - tg)) < 1e-12
    po = np.array([r[1] for r in recs_o]) * o.h
    pg = np.array([r[1] for r in recs_g]) * o.h
    Hs = 2 * inp.get("amp_mono", 0.025) if inp["icase"] == 2 else inp["Hs"]
    assert np.max(np.abs(po - pg)) / Hs <= 1e-9
    eta_g, _, _ = g.get_state()
    assert np.max(np.abs(eta_g - o.eta)) * o.h / Hs <= 1e-9
