"""Step control on the device (hosnwt_advance with the CUDA-graph loop)
against the host loop of HOS-NWT.f90:498-571 (HOSNWT_DEVICE_LOOP=0).

The two runs are separate processes, since the library reads the variable
once when it loads.  Each runs the time loop of a 2-D and a 3-D tank and
prints the probe records, the accepted and rejected step counts per output
interval and the final state.  The two loops differ only in where pow() of
dt_correc is evaluated (the device's pow may differ from the host's in the
last bit), so one of them may take an extra remainder step of a few ulps
where time_cur + (time_next - time_cur) falls just short of time_next;
these tanks' steps are clamped at 0.95 dt_stab, so nothing else changes.
Checked: the same output times, probes and final eta within 1e-10 of their
max |.| (the time-loop gate is 1e-9), and step counts within one per
interval.  A NaN planted in the state must stop the device loop with
HOSNWT_ERR_NAN and leave the time where it was.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import json, sys
import numpy as np
sys.path[:0] = [ROOT, ROOT + "/hos-nwt_gb300", ROOT + "/tests"]
import hosnwt, cases
out = {}
for name, T in (("reg1d_w2", 3.0), ("reg3d", 2.0)):
    case = cases.ALL[name]
    inp = dict(case["inp"], T_stop=T)
    probes = [(5.0, 0.0), (10.0, 0.0)] if case["n2"] == 1 else [(5.0, 5.0), (10.0, 12.0)]
    g = hosnwt.Tank(inp, case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"], probes=probes)
    inf = g.info()
    delt, T_stop, dout = inf["delt"], inf["T_stop"], inf["delt_out"]
    recs, counts = [], []
    # the output loop of HOS-NWT.f90:446-581, as Tank.simulate runs it
    while g.info()["time_cur"] < T_stop + dout:
        t = g.info()["time_cur"]
        recs.append([t] + list(g.probes()))
        if abs(t - T_stop) <= 2.2e-16:
            break
        delt, na, nr = g.advance(min(t + dout, T_stop + dout), delt)
        counts.append([na, nr])
    eta, phis, _ = g.get_state()
    out[name] = {"recs": recs, "counts": counts, "eta": eta.ravel(order="F").tolist(), "h": delt}
    g.close()
print(json.dumps(out))
"""


def _run(device_loop):
    env = dict(os.environ)
    env.pop("HOSNWT_DEVICE_LOOP", None)
    if not device_loop:
        env["HOSNWT_DEVICE_LOOP"] = "0"
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + SCRIPT], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_device_loop_matches_host_loop(lib):
    dev, host = _run(True), _run(False)
    for name in host:
        a, b = dev[name], host[name]
        ca, cb = np.array(a["counts"]), np.array(b["counts"])
        assert ca.shape == cb.shape, name
        assert np.max(np.abs(ca - cb)) <= 1, (name, a["counts"], b["counts"])
        ra, rb = np.array(a["recs"]), np.array(b["recs"])
        assert ra.shape == rb.shape, name
        assert np.max(np.abs(ra[:, 0] - rb[:, 0])) <= 1e-12, name
        scale = max(np.max(np.abs(rb[:, 1:])), 1e-300)
        assert np.max(np.abs(ra[:, 1:] - rb[:, 1:])) <= 1e-10 * scale, (name, np.max(np.abs(ra[:, 1:] - rb[:, 1:])))
        ea, eb = np.array(a["eta"]), np.array(b["eta"])
        assert np.max(np.abs(ea - eb)) <= 1e-10 * max(np.max(np.abs(eb)), 1e-300), name


def test_device_loop_stops_on_nan(lib):
    import hosnwt
    import cases
    case = cases.ALL["reg1d"]
    g = hosnwt.Tank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"])
    inf = g.info()
    h, _, _ = g.advance(5 * inf["delt"], inf["delt"])
    t0 = g.info()["time_cur"]
    eta, phis, _ = g.get_state()
    eta[3, 0] = np.nan
    g.set_state(eta, phis)
    with pytest.raises(hosnwt.HosError, match="NAN"):
        g.advance(t0 + 10 * h, h)
    assert g.info()["time_cur"] == t0
    g.close()
