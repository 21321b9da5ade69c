"""The FFT transform passes (fft.cu) against the oracle, through the C ABI.

Six 3-D tanks whose axis lengths D = N - 1 cover the FFT plans: powers of
two, Rader's algorithm for prime D (641 = 2^7 5 + 1, 257 = 2^8 + 1), the
generic odd radix (61, 19, 11, 97, 79, 13, 43) and Bluestein's chirp
convolution for lengths with a large prime factor (2051 = 7 293, and the
prime 4099, whose 4098 = 2 3 683 rules Rader out).  Every kind (cos / sin along x
and y, S2F and F2S) on the free-surface and dealiased grids is compared with
the oracle's transforms at 1e-13 * sqrt(N) of max |ref|.  Each run is a
separate process with HOSNWT_FFT = 1 (FFT passes wherever a plan exists),
0 (the sum passes only) or unset (the library's choice), since the library
reads the variable once when it loads; the FFT passes run their complex DFT
in double-float (the default) and, with HOSNWT_FFT_DF = 0, in FP64.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (n1, n2, p1, p2): x / y lengths D of the free-surface and dealiased grids
SIZES = [
    (513, 257, 4, 4),   # 512, 256 | 1281 = 3 7 61, 641 prime
    (257, 129, 3, 3),   # 256, 128 | 513 = 3^3 19, 257 prime
    (257, 65, 5, 5),    # 256, 64  | 770 = 2 5 7 11, 194 = 2 97
    (514, 33, 3, 3),    # 513, 32  | 1027 = 13 79, 65 = 5 13
    (65, 513, 3, 7),    # 64, 512  | 129 = 3 43, 2051 = 7 293 (Bluestein)
    (1025, 33, 7, 3),   # 1024, 32 | 4099 prime (Bluestein), 65
]

SCRIPT = r"""
import json, sys
import numpy as np
sys.path[:0] = [ROOT, ROOT + "/hos-nwt_gb300"]
import hosnwt
from oracle.hos_oracle import Fourier, default_input
rng = np.random.default_rng(11)
worst = 0.0
worst_rel = 0.0
for n1, n2, p1, p2 in SIZES:
    M = max(p1, p2, 3)
    inp = default_input(T_stop=5.0, amp_mono=0.02, nu_mono=0.7, theta_mono=10.0, ylen=20.0, toler=1e-7)
    g = hosnwt.Tank(inp, n1, n2, 9, M, p1, p2)
    nd1, nd2 = ((p1 + 1) * n1) // 2, ((p2 + 1) * n2) // 2
    F = Fourier(n1, n2, nd1, nd2, 16)
    for grid, shp in (("n", (n1, n2)), ("big", (nd1, nd2))):
        for csx in ("cos", "sin"):
            for csy in ("cos", "sin"):
                for direction in (1, -1):
                    a = rng.standard_normal(shp)
                    if grid == "n":
                        ref = F.S2F(a, csx, csy) if direction == 1 else F.F2S(a, csx, csy)
                    else:
                        ref = F.S2F_big(a, csx, csy) if direction == 1 else F.F2S_big(a, csx, csy)
                    got = g.transform(grid, direction, csx, csy, a)
                    rel = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
                    tol = 1e-13 * np.sqrt(max(shp))
                    if not rel < tol:
                        print(json.dumps({"fail": [n1, n2, p1, p2, grid, csx, csy, direction, rel, tol]}))
                        sys.exit(1)
                    worst = max(worst, rel / tol)
                    worst_rel = max(worst_rel, rel)
    g.close()
print(json.dumps({"worst_fraction_of_tol": worst, "worst_rel": worst_rel}))
"""


@pytest.mark.parametrize("mode", ["1", "1-fp64", "0", "auto"])
def test_fft_transforms_match_oracle(lib, mode):
    env = dict(os.environ)
    env.pop("HOSNWT_FFT", None)
    env.pop("HOSNWT_FFT_DF", None)
    if mode == "1-fp64":
        env["HOSNWT_FFT_DF"] = "0"
        mode = "1"
    if mode != "auto":
        env["HOSNWT_FFT"] = mode
    src = f"ROOT = {ROOT!r}\nSIZES = {SIZES!r}\n" + SCRIPT
    r = subprocess.run([sys.executable, "-c", src], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
    out = json.loads(r.stdout.strip().splitlines()[-1])
    print(mode, out)
    assert out["worst_fraction_of_tol"] < 1.0


NAN_SCRIPT = r"""
import json, sys
import numpy as np
sys.path[:0] = [ROOT, ROOT + "/hos-nwt_gb300"]
import hosnwt
from oracle.hos_oracle import Fourier, default_input
n1, n2, p1, p2 = 513, 257, 4, 4
inp = default_input(T_stop=5.0, amp_mono=0.02, nu_mono=0.7, theta_mono=10.0, ylen=20.0, toler=1e-7)
g = hosnwt.Tank(inp, n1, n2, 9, 4, p1, p2)
nd1, nd2 = ((p1 + 1) * n1) // 2, ((p2 + 1) * n2) // 2
F = Fourier(n1, n2, nd1, nd2, 16)
rng = np.random.default_rng(5)
out = {}
for bad in (np.nan, np.inf):
    a = rng.standard_normal((nd1, nd2))
    a[7, 11] = bad
    got = g.transform("big", 1, "cos", "cos", a)
    clean = a.copy()
    clean[7, 11] = 0.0
    ref = F.S2F_big(clean, "cos", "cos")
    # the x pass spreads the bad entry over column 11, the y pass over every
    # row: the whole output becomes non-finite; a clean transform after it
    # is exact again (no state is left behind)
    out[str(bad)] = bool(np.all(~np.isfinite(got)))
    again = g.transform("big", 1, "cos", "cos", clean)
    out[str(bad) + "_after"] = float(np.max(np.abs(again - ref)) / np.max(np.abs(ref)))
g.close()
print(json.dumps(out))
"""


def test_fft_passes_propagate_nan_and_inf(lib):
    env = dict(os.environ)
    env["HOSNWT_FFT"] = "1"
    env.pop("HOSNWT_FFT_DF", None)
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + NAN_SCRIPT], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
    out = json.loads(r.stdout.strip().splitlines()[-1])
    for bad in ("nan", "inf"):
        assert out[bad], (bad, out)
        assert out[bad + "_after"] < 1e-13 * 23, (bad, out)
