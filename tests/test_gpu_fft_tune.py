"""The FFT layout tuner (fft.cu: fft_tune_run) changes only how the
double-float passes spread their lines over CTAs and threads, never the
arithmetic of a line: one RK4(5) step of the directional 3-D benchmark
tank must give the same bits with the tuner on (the default) and off
(HOSNWT_FFT_TUNE=0).  Each run is a separate process, since the library
reads the variable once when it loads."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import hashlib, json, sys, tempfile
import numpy as np
sys.path[:0] = [ROOT, ROOT + "/hos-nwt_gb300", ROOT + "/tests"]
import baseline_cases as bc
with tempfile.TemporaryDirectory() as tmp:
    w = bc.spec("c3", tmp)
    o = bc.oracle_tank(w)
    g = bc.gpu_tank(w)
st = bc.physical_state(o, frac=0.2)
g.solveHOS2(bc.zero_state(o), 0.0, bc.STEP_T0, 0.0, 0.0)
arrs, err = g.runge4_adapt2(bc.STEP_T0, *st, g.info()["delt"])
g.close()
h = hashlib.sha256()
for a in arrs:
    h.update(np.ascontiguousarray(a).tobytes())
print(json.dumps({"sha": h.hexdigest(), "err": err}))
"""


def _run(tune):
    env = dict(os.environ)
    env.pop("HOSNWT_FFT_TUNE", None)
    env.pop("HOSNWT_FFT_DF", None)
    if not tune:
        env["HOSNWT_FFT_TUNE"] = "0"
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + SCRIPT], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_tuned_layout_gives_the_same_bits(lib):
    a, b = _run(True), _run(False)
    assert a["sha"] == b["sha"]
    assert a["err"] == b["err"]
