"""Output files of the time loop (hosnwt_run): probes.dat, vol_energy.dat and
3d.dat in the reference's formats, their values against the device API and
the oracle, and check_slope's slope measure."""
import os
import re

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

D13 = re.compile(r"^( {1,2}-?0\.\d{5}D[+-]\d{2})+$")


def _case(T):
    case = dict(cases.ALL["reg1d"])
    inp = dict(case["inp"])
    inp["T_stop"] = T
    case["inp"] = inp
    return case


def test_run_writes_reference_formats(lib, tmp_path):
    import hosnwt
    from oracle.hos_oracle import Tank as OTank
    case = _case(1.0)
    probes = [(5.0, 0.0), (10.0, 0.0)]
    g = hosnwt.Tank(case["inp"], case["n1"], 1, case["n3"], case["mHOS"], case["p1"], 1, probes=probes)
    g.run(str(tmp_path))
    lines = open(os.path.join(tmp_path, "probes.dat")).read().splitlines()
    head = [ln for ln in lines if ln.startswith("#")]
    assert len(head) == 59  # write_input: 12 section lines + 47 values
    assert head[1] == "#        Length(m) of the wavetank::          xlen::    5.0000000000000000E+01"
    assert lines[len(head)] == 'TITLE="Probes elevation records versus time"'
    recs = lines[len(head) + 2:]
    assert all(D13.match(r) for r in recs)
    vals = np.array([[float(x.replace("D", "E")) for x in re.findall(r"-?0\.\d{5}D[+-]\d{2}", r)] for r in recs])
    o = OTank(case["inp"], case["n1"], 1, case["n3"], case["mHOS"], case["p1"], 1, probes=probes)
    en = []
    ro = o.run(on_output=lambda t: en.append(t.energy()))
    assert vals.shape == (len(ro), 3)
    t_ref = np.array([r[0] for r in ro]) * o.Tscale
    p_ref = np.array([r[1] for r in ro]) * o.h
    assert np.allclose(vals[:, 0], t_ref, rtol=1e-5, atol=1e-12)
    assert np.allclose(vals[:, 1:], p_ref, rtol=1e-4, atol=1e-9)
    ve = open(os.path.join(tmp_path, "vol_energy.dat")).read().splitlines()
    rows = [ln for ln in ve if not ln.startswith("#") and not ln.startswith("TITLE") and not ln.startswith("VARIABLES")]
    assert len(rows) == len(ro)
    got = np.array([[float(x) for x in r.split()] for r in rows])
    ref = np.array(en)
    assert np.allclose(got[:, 2], ref[:, 0], rtol=1e-4, atol=1e-14), (got[:, 2], ref[:, 0])
    assert np.allclose(got[:, 3], ref[:, 1], rtol=1e-4, atol=1e-14), (got[:, 3], ref[:, 1])


def test_diagnostics_match_oracle(lib):
    import hosnwt
    from oracle.hos_oracle import Tank as OTank
    case = _case(1.0)
    g = hosnwt.Tank(case["inp"], case["n1"], 1, case["n3"], case["mHOS"], case["p1"], 1)
    o = OTank(case["inp"], case["n1"], 1, case["n3"], case["mHOS"], case["p1"], 1)
    g.simulate(T_end=0.5)
    o.run(T_end=0.5)
    dg = g.diagnostics()
    assert abs(dg[0] - o.volume()) <= 1e-10 + 1e-8 * abs(o.volume())
    ep, ek = o.energy()
    assert abs(dg[1] - ep) <= 1e-9 * abs(ep) + 1e-16
    assert abs(dg[2] - ek) <= 1e-8 * abs(ek) + 1e-16
    assert abs(dg[3] - np.max(np.abs(o.etax))) <= 1e-9 * np.max(np.abs(o.etax)) + 1e-16
    assert g.check_slope() == 0


ZONE0 = re.compile(r"^ZONE SOLUTIONTIME = [ \d.-]{6}, I=[ \d]{4}, J=[ \d]{4}$")
ZONE = re.compile(r"^ZONE SOLUTIONTIME = [ \d.-]{6}, D=\(1,2\), I=[ \d]{4}, J=[ \d]{4}$")
ES = r"[ -]\d\.\d{5}E[+-]\d{2} "
ROW0 = re.compile(r"^[ \d.-]{10} [ \d.-]{10} " + ES + ES + "$")
ROW = re.compile(r"^" + ES + ES + "$")


def test_run_writes_3d_dat(lib, tmp_path):
    """3d.dat of a 3-D tank (output.f90:291-345, tecplot = 11): the first zone
    holds x, y, eta, phis; later zones eta and eta minus the target wave;
    eta against the oracle at every output time."""
    import hosnwt
    from oracle.hos_oracle import Tank as OTank
    case = dict(cases.ALL["reg3d"])
    inp = dict(case["inp"])
    inp["T_stop"] = 1.0
    inp["i3d"] = 1
    args = (inp, case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"])
    g = hosnwt.Tank(*args)
    g.run(str(tmp_path))
    lines = open(os.path.join(tmp_path, "3d.dat")).read().splitlines()
    head = [ln for ln in lines if ln.startswith("#")]
    assert len(head) == 59
    body = lines[len(head):]
    assert body[0] == ' TITLE=" 3D free surface elevation "'
    assert body[1] == 'VARIABLES="x","y","eta","phis"'
    n1, n2 = case["n1"], case["n2"]
    zones = []
    i = 2
    while i < len(body):
        assert (ZONE0 if not zones else ZONE).match(body[i]), body[i]
        rows = body[i + 1:i + 1 + n1 * n2]
        rx = ROW0 if not zones else ROW
        assert all(rx.match(r) for r in rows), rows[0]
        zones.append(np.array([[float(x) for x in r.split()] for r in rows]))
        i += 1 + n1 * n2
    o = OTank(*args)
    etas = []
    o.run(on_output=lambda t: etas.append(t.eta.copy()))
    assert len(zones) == len(etas)
    h = inp["h"]
    assert np.allclose(zones[0][:, 0], np.tile(o.cx, n2) * h, atol=6e-6)
    for z, e in zip(zones, etas):
        eta = e.reshape(-1, order="F") * h
        got = z[:, 2] if z.shape[1] == 4 else z[:, 0]
        assert np.allclose(got, eta, rtol=2e-5, atol=1e-9 * max(1.0, np.max(np.abs(eta)))), np.max(np.abs(got - eta))
