"""Parity of the CUDA path with the oracle across the reference's branches:
wavemaker geometry, ramp laws (including the ramp-down after T_stop), HOS
order and partial dealiasing, file wave input with cut-offs and repeated
harmonics, no absorbing zone, and the end-of-ramp correction."""
import os

import numpy as np
import pytest

from oracle.hos_oracle import Tank as OTank, default_input

pytestmark = pytest.mark.gpu


def _pair(inp, n1=65, n2=1, n3=17, M=3, p1=3, p2=1, probes=None, wave_dir="."):
    import hosnwt
    g = hosnwt.Tank(inp, n1, n2, n3, M, p1, p2, probes=probes, wave_dir=wave_dir)
    o = OTank(inp, n1, n2, n3, M, p1, p2, probes=probes, wave_files_dir=wave_dir)
    return g, o


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def _rhs_check(g, o, t, dt=0.01, seed=3, tol=1e-10):
    rng = np.random.default_rng(seed)
    n1, n2, n3a = o.n1, o.n2, o.n3_add
    decay = np.exp(-0.2 * np.arange(n1))[:, None] * np.exp(-0.4 * np.arange(n2))[None, :]
    G2 = 1e-3 * rng.standard_normal((n1, n2)) * decay * o.omega
    G2[0, 0] = 0.0
    y = dict(G1=1e-3 * rng.standard_normal((n1, n2)) * decay, G2=G2,
             a_add_1=1e-3 * rng.standard_normal((n3a, n2)), a_add_2=np.zeros((n3a, n2)),
             a_add_ramp=1e-3 * rng.standard_normal((n3a, n2)), a_add_3=np.zeros((n3a, n2)),
             a1st=1e-3 * rng.standard_normal((n1, n2)) * decay, eta1st=1e-3 * rng.standard_normal((n1, n2)) * decay,
             a2nd=np.zeros((n1, n2)), eta2nd=np.zeros((n1, n2)))
    alpha_prev, pos_top = o._alpha[0], o._pos[0][o.n3 - 1, 0]
    ref = o.solveHOS2({k: v.copy() for k, v in y.items()}, dt, t)
    got = g.solveHOS2([y[k] for k in o.STATE_KEYS], dt, t, alpha_prev, pos_top)
    for key, arr in zip(o.STATE_KEYS, got):
        r = ref[key]
        if np.max(np.abs(r)) == 0.0:
            assert np.max(np.abs(arr)) == 0.0, key
        else:
            assert _rel(arr, r) < tol, (key, _rel(arr, r))


@pytest.mark.parametrize("iramp", [0, 1, 2, 21, 4, 41, 11, 33])
def test_ramp_laws(lib, iramp):
    inp = default_input(iramp=iramp, Tramp=2.0, T_stop=4.0, toler=1e-7, f_out=10.0)
    g, o = _pair(inp)
    T = o.Tscale
    for t_phys in (0.3, 1.1, 1.9, 3.0, 4.5, 5.5, 7.0):  # inside, after the ramp, ramp-down, stopped
        _rhs_check(g, o, t_phys / T)


@pytest.mark.parametrize("igeom", [1, 2])
def test_wavemaker_geometry(lib, igeom):
    inp = default_input(igeom=igeom, d_hinge=1.5, T_stop=10.0, toler=1e-7, f_out=10.0)
    g, o = _pair(inp)
    _rhs_check(g, o, 1.0)


@pytest.mark.parametrize("M,p1", [(1, 1), (2, 2), (4, 4), (5, 3), (7, 7), (4, 2)])
def test_hos_orders(lib, M, p1):
    inp = default_input(T_stop=10.0, toler=1e-7, f_out=10.0)
    g, o = _pair(inp, M=M, p1=p1)
    _rhs_check(g, o, 0.7)


def test_3d_partial_dealiasing_y(lib):
    inp = default_input(T_stop=10.0, theta_mono=10.0, ylen=20.0, toler=1e-7, f_out=4.0, nu_mono=0.7)
    g, o = _pair(inp, n1=33, n2=17, n3=9, M=4, p1=4, p2=2)
    _rhs_check(g, o, 0.9)


def test_no_absorbing_zone(lib):
    inp = default_input(iabsnb=0, T_stop=10.0, toler=1e-7, f_out=10.0)
    g, o = _pair(inp)
    _rhs_check(g, o, 0.8)


def test_file_waves_cutoff_and_repeated_harmonics(lib, tmp_path):
    import workloads
    harmo = np.array([20, 20, 25, 30, 31, 40, 90, 200])  # two components share harmonic 20
    amp = np.array([0.004, 0.002, 0.005, 0.003, 0.003, 0.002, 0.001, 0.001])
    phase = np.linspace(0.1, 5.0, harmo.size)
    angle = np.zeros(harmo.size)
    # clock 32 Hz, rnum 9: f = harmo / 16 Hz; cut-offs drop 0.125 Hz (harmo 2) and 12.5 Hz
    workloads.write_wave_files(str(tmp_path), "W", harmo, 32.0, 9, amp, angle, phase, 5.0, 30.0, 2.0,
                               0.5, 6.0)
    inp = default_input(icase=3, file_name="W", T_stop=10.0, toler=1e-7, f_out=10.0)
    g, o = _pair(inp, wave_dir=str(tmp_path))
    assert len(o.freq_w) == 5  # harmonic 20 is one group; above 4 Hz (90) wmk_ini drops, 200 is cut
    _rhs_check(g, o, 1.3)


def test_end_of_ramp_correction(lib):
    """A time loop whose steps cross Tramp exercises the one-off
    a1st_add -= a_add_ramp correction (HOS-NWT.f90:546-550)."""
    inp = default_input(iramp=1, Tramp=0.35, T_stop=0.6, toler=1e-7, f_out=10.0)
    g, o = _pair(inp, probes=[(5.0, 0.0)])
    ro = o.run()
    rg = g.simulate()
    assert len(ro) == len(rg)
    po = np.array([r[1] for r in ro])
    pg = np.array([r[1] for r in rg])
    assert np.max(np.abs(po - pg)) <= 1e-9 * max(np.max(np.abs(po)), 1e-12)
    assert getattr(o, "_endramp", 0) == 1
