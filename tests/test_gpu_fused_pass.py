"""The opt-in fused two-level pass (HOSNWT_FUSED_PASS=1, two_level_fused in
xform.cu) against the oracle.

The library reads the switch once when it loads, so the parity tests and the
reference's Irreg_2D record run again in a child pytest process with the
switch set: the transforms of every grid and kind, one right-hand side, one
RK4(5) step and the 2 s time loops, at the tolerances of those tests."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fused_pass_parity(lib):
    env = dict(os.environ, HOSNWT_FUSED_PASS="1")
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
           os.path.join(HERE, "test_gpu_parity.py"),
           os.path.join(HERE, "test_gpu_reference_records.py") + "::test_irreg2d_matches_reference_record"]
    r = subprocess.run(cmd, env=env, cwd=os.path.dirname(HERE), capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert " passed" in r.stdout and "failed" not in r.stdout
