"""The CUDA path against the reference's own result files.

Benchmark/Sloshing, Regular_3D, Irreg_2D and Irreg_3D ship probe records
written by the reference HOS-NWT (tests/golden/ref_*.npz, made by
tests/golden/make_ref_benchmarks.py).  The whole runs (20 s to 256 s) go
through the C ABI; every probe value must agree with the reference's record
within about half a unit of its last printed digit (5 significant digits).
"""
import os

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _digit_unit(v):
    a = np.abs(v)
    return np.where(a > 0, 10.0 ** (np.floor(np.log10(np.where(a > 0, a, 1.0))) - 4), 1e-20)


def _records(case, fx, wave_dir="."):
    import hosnwt
    probes = [tuple(p) for p in fx["probes"]]
    g = hosnwt.Tank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"],
                    probes=probes, wave_dir=wave_dir)
    inf = g.info()
    recs = g.simulate()
    return np.array([[t * inf["Tscale"]] + list(np.asarray(p) * case["inp"]["h"]) for t, p in recs])


def _fixture(name):
    return np.load(os.path.join(os.path.dirname(__file__), "golden", name))


def test_sloshing_matches_reference_record(lib):
    fx = _fixture("ref_sloshing.npz")
    got = _records(cases.REF_SLOSHING, fx)
    ref = fx["records"]
    assert got.shape == ref.shape
    assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 0.6 * _digit_unit(ref[:, 0]) + 1e-9)
    err = np.abs(got[:, 1:] - ref[:, 1:]) / (_digit_unit(ref[:, 1:]) + 1e-12)
    assert np.max(err[:, [0, 2]]) <= 0.6, np.max(err)


def test_regular3d_matches_reference_record(lib):
    """Nonlinear (M = 3) 3-D tank with Dalrymple wavemaking over 40 s."""
    fx = _fixture("ref_regular3d.npz")
    got = _records(cases.REF_REGULAR_3D, fx)
    ref = fx["records"]
    assert got.shape == ref.shape
    assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 0.6 * _digit_unit(ref[:, 0]) + 1e-9)
    err = np.abs(got[:, 1:] - ref[:, 1:]) / (_digit_unit(ref[:, 1:]) + 1e-14)
    assert np.max(err) <= 0.6, (np.max(err), np.unravel_index(np.argmax(err), err.shape))


def test_irreg2d_matches_reference_record(lib, tmp_path):
    """4348-component file wave, second-order wavemaker (i_wmk = 2), M = 3,
    512 modes, 1502 records over 50 s."""
    fx = _fixture("ref_irreg2d.npz")
    cases.write_ref_wave_files(fx, str(tmp_path))
    got = _records(cases.REF_IRREG_2D, fx, str(tmp_path))
    ref = fx["records"]
    assert got.shape == ref.shape, (got.shape, ref.shape)
    assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 0.6 * _digit_unit(ref[:, 0]) + 1e-9)
    err = np.abs(got[:, 1:] - ref[:, 1:]) / (_digit_unit(ref[:, 1:]) + 1e-14)
    assert np.max(err) <= 0.6, (np.max(err), np.unravel_index(np.argmax(err), err.shape))


def test_irreg3d_matches_reference_record(lib, tmp_path):
    """Edinburgh Designs .txt wave (OCEAN reader, icase 31), second-order
    wavemaker, M = 3, 256 x 32 modes, 2561 records over 256 s."""
    fx = _fixture("ref_irreg3d.npz")
    cases.write_ref_txt(fx, str(tmp_path))
    got = _records(cases.REF_IRREG_3D, fx, str(tmp_path))
    ref = fx["records"]
    assert got.shape == ref.shape, (got.shape, ref.shape)
    assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 0.6 * _digit_unit(ref[:, 0]) + 1e-9)
    err = np.abs(got[:, 1:] - ref[:, 1:]) / (_digit_unit(ref[:, 1:]) + 1e-14)
    assert np.max(err) <= 0.6, (np.max(err), np.unravel_index(np.argmax(err), err.shape))
