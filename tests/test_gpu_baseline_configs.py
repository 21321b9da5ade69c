"""GPU parity on the benchmark tank configurations themselves, through the C
ABI, against the oracle's fixtures (tests/golden/baseline_*.npz):

  c1  regular_2d      (n1 = 257, M = 3): RHS, RK4(5) step, the whole 30 s run
  c2  irregular_2d    (n1 = 1025, M = 5, p1 = 5, 512 components): RHS, step,
                      the first 10 s of the time loop
  c3  directional_3d  (513 x 257, M = 5, p = 4): RHS, step (sampled entries,
                      max |.|, sum of squares and random projections), the
                      first simulated second of the time loop
  c5  steep_3d        (1025 x 513, M = 7, p = 7): RHS, step (sampled)

Tolerances (FP64, different summation orders):
  one right-hand side / one RK4(5) step   <= 1e-10 relative to max |ref|
  error estimate of the step              <= 1e-6 relative
  time loop                               max |d eta| / Hs <= 1e-9 over the
                                          records and at the end; probe
                                          error <= 1e-8 of max |probe|
"""
import tempfile

import numpy as np
import pytest

import baseline_cases as bc

pytestmark = pytest.mark.gpu
RTOL = 1e-10


def _rel(a, b):
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(np.asarray(a) - b)) / scale)


@pytest.mark.parametrize("name", ["c1", "c2", "c3", "c5"])
def test_rhs(lib, name):
    fx = bc.load(name)
    with tempfile.TemporaryDirectory() as tmp:
        w = bc.spec(name, tmp)
        o = bc.oracle_tank(w)
        g = bc.gpu_tank(w)
    y = bc.modal_state(o.n1, o.n2, o.n3_add, o.omega, frac=bc.ENVELOPE.get(name, 0.2))
    got = g.solveHOS2(y, bc.RHS_DT, bc.RHS_T, float(fx["rhs_alpha_prev"][0]), float(fx["rhs_pos_top"][0]))
    g.close()
    worst = 0.0
    for i, (key, arr) in enumerate(zip(bc.KEYS, got)):
        if name in bc.SAMPLED:
            worst = max(worst, bc.compare_summary(fx, "rhs_" + key, arr, 100 + i, RTOL))
            continue
        ref = fx["rhs_" + key]
        if np.max(np.abs(ref)) == 0.0:
            assert np.max(np.abs(arr)) == 0.0, key
        else:
            assert _rel(arr, ref) <= RTOL, (key, _rel(arr, ref))
            worst = max(worst, _rel(arr, ref))
    print(f"rhs {name}: worst relative deviation {worst:.2e} (gate {RTOL:.0e})")


@pytest.mark.parametrize("name", ["c1", "c2", "c3", "c5"])
def test_step(lib, name):
    fx = bc.load(name)
    with tempfile.TemporaryDirectory() as tmp:
        w = bc.spec(name, tmp)
        o = bc.oracle_tank(w)
        g = bc.gpu_tank(w)
    st = bc.physical_state(o, frac=bc.ENVELOPE.get(name, 0.2))
    # the wavemaker state the first stage's volume correction reads: one
    # right-hand side at the step's start time
    g.solveHOS2(bc.zero_state(o), 0.0, bc.STEP_T0, 0.0, 0.0)
    h = float(fx["step_h"][0])
    arrs, err = g.runge4_adapt2(bc.STEP_T0, *st, h)
    g.close()
    ref_err = float(fx["step_err"][0])
    assert abs(err - ref_err) <= 1e-6 * max(ref_err, 1e-12) + 1e-14, (err, ref_err)
    worst = 0.0
    for i, (key, arr) in enumerate(zip(bc.STEP_KEYS, arrs)):
        if name in bc.SAMPLED:
            worst = max(worst, bc.compare_summary(fx, "step_" + key, arr, 200 + i, RTOL))
            continue
        ref = fx["step_" + key]
        if np.max(np.abs(ref)) == 0.0:
            assert np.max(np.abs(arr)) == 0.0, key
        else:
            assert _rel(arr, ref) <= RTOL, (key, _rel(arr, ref))
            worst = max(worst, _rel(arr, ref))
    print(f"step {name}: worst relative deviation {worst:.2e} (gate {RTOL:.0e}); error estimate "
          f"{abs(err - ref_err) / max(ref_err, 1e-12):.2e}")


@pytest.mark.parametrize("name", ["c1", "c2", "c3"])
def test_time_loop(lib, name):
    fx = bc.load(name)
    with tempfile.TemporaryDirectory() as tmp:
        w = bc.spec(name, tmp)
        inp = dict(w["inp"], T_stop=float(fx["loop_T_stop"][0]))
        g = bc.gpu_tank(w, inp)
    recs = g.simulate()
    eta, _, _ = g.get_state()
    g.close()
    t_ref, p_ref = fx["loop_t"], fx["loop_probes"]
    assert len(recs) == len(t_ref)
    t = np.array([r[0] for r in recs])
    p = np.array([r[1] for r in recs])
    assert np.max(np.abs(t - t_ref)) < 1e-12
    h, Hs = float(fx["h"][0]), float(fx["Hs"][0])
    dp = np.max(np.abs(p - p_ref))
    assert dp * h / Hs <= 1e-9
    assert dp / np.max(np.abs(p_ref)) <= 1e-8
    if name in bc.SAMPLED:
        # the final eta as a sampled record: max |d eta| / Hs <= 1e-9 is a
        # deviation of 1e-9 Hs / (h max |eta_ref|) relative to max |eta_ref|
        ref_max = float(fx["loop_eta_max"][0])
        de = bc.compare_summary(fx, "loop_eta", eta, 300, 1e-9 * Hs / (h * ref_max))
        de_hs = de * ref_max * h / Hs
    else:
        de_hs = np.max(np.abs(eta - fx["loop_eta"])) * h / Hs
        assert de_hs <= 1e-9
    print(f"loop {name}: {len(recs)} records, max |d probe| h/Hs {dp * h / Hs:.2e}, "
          f"relative {dp / np.max(np.abs(p_ref)):.2e}; eta {de_hs:.2e} of Hs")
