"""CPU tests of the oracle: FFTW conventions, libgfortran RAND, analytic
known answers of the reference's physics and the committed golden fixtures."""
import os

import numpy as np
import pytest

from oracle import hos_oracle as H

import cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _direct(kind, x):
    """FFTW r2r definitions written as explicit sums (FFTW manual, 'What
    FFTW Really Computes')."""
    n = len(x)
    j = np.arange(n)
    y = np.zeros(n)
    for k in range(n):
        if kind == "REDFT00":
            y[k] = x[0] + (-1) ** k * x[n - 1] + 2 * np.sum(x[1:n - 1] * np.cos(np.pi * j[1:n - 1] * k / (n - 1)))
        elif kind == "RODFT00":
            y[k] = 2 * np.sum(x * np.sin(np.pi * (j + 1) * (k + 1) / (n + 1)))
        elif kind == "REDFT10":
            y[k] = 2 * np.sum(x * np.cos(np.pi * (j + 0.5) * k / n))
        elif kind == "REDFT01":
            y[k] = x[0] + 2 * np.sum(x[1:] * np.cos(np.pi * j[1:] * (k + 0.5) / n))
        elif kind == "RODFT10":
            y[k] = 2 * np.sum(x * np.sin(np.pi * (j + 0.5) * (k + 1) / n))
        elif kind == "RODFT01":
            y[k] = (-1) ** k * x[n - 1] + 2 * np.sum(x[:n - 1] * np.sin(np.pi * (j[:n - 1] + 1) * (k + 0.5) / n))
    return y


@pytest.mark.parametrize("kind", ["REDFT00", "RODFT00", "REDFT10", "REDFT01", "RODFT10", "RODFT01"])
@pytest.mark.parametrize("n", [5, 17, 34, 61])
def test_r2r_matches_fftw_definitions(kind, n):
    x = np.random.default_rng(n).standard_normal(n)
    got = H._r2r(x[:, None], 0, kind)[:, 0]
    assert np.max(np.abs(got - _direct(kind, x))) < 1e-12 * n


def test_s2f_f2s_roundtrip():
    F = H.Fourier(17, 9, 34, 18, 16)
    rng = np.random.default_rng(3)
    for csx in ("cos", "sin"):
        for csy in ("cos", "sin"):
            a = rng.standard_normal((17, 9))
            if csx == "sin":
                a[0, :] = a[-1, :] = 0
            if csy == "sin":
                a[:, 0] = a[:, -1] = 0
            assert np.allclose(F.F2S(F.S2F(a, csx, csy), csx, csy), a, atol=1e-13)
    b = rng.standard_normal((16, 9))
    b[:, 0] = b[:, -1] = 0
    for csz in ("cos", "sin"):
        assert np.allclose(F.F2S_add(F.S2F_add(b, csz, "sin"), csz, "sin"), b, atol=1e-13)


def test_gfortran_rand_sequence():
    v = H.gfortran_rand_sequence(513, 3)
    # libgfortran RAND after SRAND(513) (seed of the Benchmark inputs)
    assert [float(x) for x in v] == [0.004014730453491211, 0.4788851737976074, 0.6255302429199219]
    # the same values from the published Park-Miller generator with the
    # 24-bit mask libgfortran applies
    s = 513
    for x in v:
        s = (16807 * s) % 2147483647
        assert np.float32(((s - 1) & ~511) / np.float32(2147483646.0)) == x


def test_dichoto_dispersion():
    k = H.wave_number_adim_r(0.5, 1e-15)
    assert abs(k * np.tanh(k) - (2 * np.pi * 0.5) ** 2) < 1e-12


def test_read_input(tmp_path):
    p = os.path.join(GOLDEN, "input_HOS-NWT.dat")
    d = H.read_input(p)
    assert d["xlen"] == 50.0 and d["icase"] == 2 and d["file_name"] == "J010_14"
    assert d["toler"] == 1e-7 and d["pro_file"] == "prob.inp" and d["i_sw"] == 0


def test_linear_sloshing_known_answer():
    """icase 1: a small standing wave oscillates at the linear frequency
    sqrt(g k tanh(k h)); the nonlinear correction is O(k a)."""
    a = 5e-5
    inp = H.default_input(icase=1, islosh=3, aslosh=a, T_stop=6.0, toler=1e-8, f_out=2.0, iabsnb=0)
    t = H.Tank(inp, n1=33, n2=1, n3=9, mHOS=3, p1=3, probes=[(0.0, 0.0)])
    recs = t.run()
    T = np.array([r[0] for r in recs]) * t.Tscale
    P = np.array([r[1][0] for r in recs]) * t.h
    k = 3 * np.pi / 50.0
    w = np.sqrt(9.81 * k * np.tanh(k * 5.0))
    assert np.max(np.abs(P - a * np.cos(w * T))) / a < 5e-5


def test_volume_conserved_with_wavemaker():
    inp = H.default_input(T_stop=4.0, amp_mono=0.02, toler=1e-7, f_out=4.0)
    t = H.Tank(inp, n1=33, n2=1, n3=9, mHOS=3, p1=3)
    t.run()
    # the mean mode is set to the displaced volume of the paddle each step
    assert abs(t.volume()) < 1e-3


def test_linear_wavemaker_amplitude():
    """A small regular wave from the flap: far-field amplitude within the
    band the transfer function (TF_adim_new) predicts."""
    inp = H.default_input(T_stop=12.0, amp_mono=0.0025, nu_mono=1.0, toler=1e-6, f_out=20.0, xlen=25.0)
    t = H.Tank(inp, n1=129, n2=1, n3=17, mHOS=1, p1=1, probes=[(3.0, 0.0), (4.0, 0.0)])
    recs = t.run()
    T = np.array([r[0] for r in recs]) * t.Tscale
    P = np.array([r[1] for r in recs]) * t.h
    m = T > 8.0
    amp = 0.5 * (P[m].max(axis=0) - P[m].min(axis=0))
    assert np.all(np.abs(amp / 0.0025 - 1.0) < 0.15)


@pytest.mark.parametrize("name", ["reg1d", "reg3d", "jonswap1d", "slosh"])
def test_golden_fixtures(name):
    """The oracle still reproduces the committed fixtures (one RHS and one
    RK step of each small case)."""
    import cases
    from golden_io import load_fixture, run_fixture_case
    fx = load_fixture(name)
    got = run_fixture_case(cases.ALL[name])
    for key, ref in fx.items():
        assert np.allclose(got[key], ref, rtol=0, atol=1e-12 * max(np.max(np.abs(ref)), 1e-300)), key


# --------------------------------------------------------------------------
# The oracle against the reference's own result files (Benchmark/*/Ref_data,
# stored by tests/golden/make_ref_benchmarks.py): the probe records are
# printed with 5 significant digits, so each value must agree within about
# half a unit of its last printed digit.

def _digit_unit(v):
    a = np.abs(v)
    return np.where(a > 0, 10.0 ** (np.floor(np.log10(np.where(a > 0, a, 1.0))) - 4), 1e-20)


def _ref_fixture(name):
    return np.load(os.path.join(os.path.dirname(__file__), "golden", name))


def _run_records(case, fx, T_end=None, wave_dir="."):
    from oracle.hos_oracle import Tank
    probes = [tuple(p) for p in fx["probes"]]
    o = Tank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"], probes=probes,
             wave_files_dir=wave_dir)
    recs = o.run(T_end=T_end)
    return np.array([[r[0] * o.Tscale] + list(np.asarray(r[1]) * o.h) for r in recs])


def test_oracle_matches_reference_sloshing_record():
    """Benchmark/Sloshing: the 4th natural mode (0.2 m) over 20 s, 401 records."""
    fx = _ref_fixture("ref_sloshing.npz")
    assert [int(v) for v in fx["numerics"]] == [129, 1, 33, 1, 1, 1]
    got = _run_records(cases.REF_SLOSHING, fx)
    ref = fx["records"]
    assert got.shape == ref.shape
    assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 0.6 * _digit_unit(ref[:, 0]) + 1e-9)
    err = np.abs(got[:, 1:] - ref[:, 1:]) / (_digit_unit(ref[:, 1:]) + 1e-12)
    assert np.max(err[:, [0, 2]]) <= 0.6, np.max(err)
    assert np.max(np.abs(got[:, 2])) < 1e-12  # the node of the mode


def test_oracle_matches_reference_regular3d_record():
    """Benchmark/Regular_3D: a 30 deg Dalrymple wave, M = 3 on 256 x 32 modes;
    the first second (11 records of the 401) on the CPU."""
    fx = _ref_fixture("ref_regular3d.npz")
    assert [int(v) for v in fx["numerics"]] == [256, 32, 16, 3, 3, 3]
    case = cases.REF_REGULAR_3D
    got = _run_records(case, fx, T_end=1.0)
    ref = fx["records"][:len(got)]
    assert len(got) == 11
    assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 0.6 * _digit_unit(ref[:, 0]) + 1e-9)
    err = np.abs(got[:, 1:] - ref[:, 1:]) / (_digit_unit(ref[:, 1:]) + 1e-14)
    assert np.max(err) <= 0.6, np.max(err)


def test_oracle_matches_reference_irreg2d_record(tmp_path):
    """Benchmark/Irreg_2D: a 4348-component file wave with the second-order
    wavemaker (i_wmk = 2), M = 3 on 512 modes; the first two seconds (61
    records of the 1502) on the CPU."""
    fx = _ref_fixture("ref_irreg2d.npz")
    assert [int(v) for v in fx["numerics"]] == [512, 1, 32, 3, 3, 1]
    cases.write_ref_wave_files(fx, str(tmp_path))
    got = _run_records(cases.REF_IRREG_2D, fx, T_end=2.0, wave_dir=str(tmp_path))
    ref = fx["records"][:len(got)]
    assert len(got) == 61
    assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 0.6 * _digit_unit(ref[:, 0]) + 1e-9)
    err = np.abs(got[:, 1:] - ref[:, 1:]) / (_digit_unit(ref[:, 1:]) + 1e-14)
    assert np.max(err) <= 0.6, np.max(err)


def test_oracle_matches_reference_irreg3d_record(tmp_path):
    """Benchmark/Irreg_3D: an Edinburgh Designs .txt wave read by the OCEAN
    reader (icase 31), i_wmk = 2, M = 3 on 256 x 32 modes; the first second
    (11 records of the 2561) on the CPU."""
    fx = _ref_fixture("ref_irreg3d.npz")
    assert [int(v) for v in fx["numerics"]] == [256, 32, 16, 3, 3, 3]
    cases.write_ref_txt(fx, str(tmp_path))
    got = _run_records(cases.REF_IRREG_3D, fx, T_end=1.0, wave_dir=str(tmp_path))
    ref = fx["records"][:len(got)]
    assert len(got) == 11
    assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 0.6 * _digit_unit(ref[:, 0]) + 1e-9)
    err = np.abs(got[:, 1:] - ref[:, 1:]) / (_digit_unit(ref[:, 1:]) + 1e-14)
    assert np.max(err) <= 0.6, np.max(err)
