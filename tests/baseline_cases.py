"""The benchmark tank configurations as parity cases (fixtures written by
tests/golden/make_baseline_fixtures.py from the oracle).

  c1  regular_2d      n1 = 257, n3 = 33, M = 3, p1 = 3 (the whole 30 s run)
  c2  irregular_2d    n1 = 1025, n3 = 65, M = 5, p1 = 5, 512 components,
                      seed 513 (one right-hand side, one RK4(5) step, the
                      first 10 s of the time loop)
  c3  directional_3d  513 x 257, n3 = 33, M = 5, p1 = p2 = 4 (one right-hand
                      side, one RK4(5) step)
  c5  steep_3d        1025 x 513, n3 = 33, M = 7, p1 = p2 = 7 (one right-hand
                      side, one RK4(5) step)

The right-hand side and the step start from a seeded synthetic state: random
modal amplitudes under a Gaussian envelope over the lower modes, drawn from
PCG64.random (uniform doubles: the bit stream numpy keeps stable across
versions).  Arrays too large to commit (the 3-D cases) are stored as a
seeded sample of entries, their max |.| and sum of squares, and projections
on seeded random vectors, all size-independent checks.
"""
from __future__ import annotations

import os

import numpy as np

import workloads
from oracle.hos_oracle import Tank as OTank

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KEYS = ("G1", "G2", "a_add_1", "a_add_2", "a_add_ramp", "a_add_3", "a1st", "eta1st", "a2nd", "eta2nd")
STEP_KEYS = ("eta", "phis", "a_add_1", "a_add_2", "a_add_ramp", "a_add_3", "eta1st", "eta2nd", "a1st", "a2nd")
RHS_T, RHS_DT = 1.3, 0.02        # stage time and stage step of the right-hand side case
STEP_T0 = 1.3                    # start time of the step case
NSAMPLE = 2048                   # sampled entries per array (sampled fixtures)
NPROJ = 4                        # random projections per array


def spec(name, directory):
    """Workload spec of case `name`; wave files go to `directory`."""
    if name == "c1":
        return workloads.regular_2d()
    if name == "c2":
        return workloads.irregular_2d(directory)
    if name == "c3":
        return workloads.directional_3d(directory)
    if name == "c5":
        return workloads.steep_3d(directory)
    raise KeyError(name)


SAMPLED = ("c3", "c5")  # cases stored as size-independent records
# width of the modal envelope (fraction of n): the M = 7 tank needs a milder
# spectrum, since the order-M terms grow like (k eta)^M
ENVELOPE = {"c5": 0.05}


def oracle_tank(w):
    return OTank(w["inp"], w["n1"], w["n2"], w["n3"], w["mHOS"], w["p1"], w["p2"],
                 wave_files_dir=w["wave_dir"], probes=w["probes"])


def gpu_tank(w, inp=None):
    import hosnwt
    return hosnwt.Tank(inp or w["inp"], w["n1"], w["n2"], w["n3"], w["mHOS"], w["p1"], w["p2"],
                       probes=w["probes"], wave_dir=w["wave_dir"])


def _uniform(rng, shape):
    return 2.0 * rng.random(shape) - 1.0


def _envelope(n, frac):
    return np.exp(-(np.arange(n) / max(frac * n, 1.0)) ** 2)


def modal_state(n1, n2, n3a, omega, seed=2024, amp=1e-3, frac=0.2):
    """The 10 modal arrays of solveHOS2 (G1, G2, a_add_1, a_add_2,
    a_add_ramp, a_add_3, a1st, eta1st, a2nd, eta2nd); first-order
    wavemaker: the second- and third-order arrays are zero."""
    rng = np.random.Generator(np.random.PCG64(seed))
    env = _envelope(n1, frac)[:, None] * _envelope(n2, frac)[None, :]
    enva = _envelope(n3a, 0.3)[:, None] * _envelope(n2, frac)[None, :]
    G1 = amp * _uniform(rng, (n1, n2)) * env
    G2 = amp * _uniform(rng, (n1, n2)) * env * omega
    G2[0, 0] = 0.0
    a1 = amp * _uniform(rng, (n3a, n2)) * enva
    ar = amp * _uniform(rng, (n3a, n2)) * enva
    a1st = amp * _uniform(rng, (n1, n2)) * env
    e1st = amp * _uniform(rng, (n1, n2)) * env
    z = np.zeros((n1, n2))
    za = np.zeros((n3a, n2))
    return [G1, G2, a1, za.copy(), ar, za.copy(), a1st, e1st, z.copy(), z.copy()]


def physical_state(o, seed=2025, amp=1e-3, frac=0.2):
    """The 10 arrays of runge4_adapt2 (eta, phis, a_add_1, a_add_2,
    a_add_ramp, a_add_3, eta1st, eta2nd, a1st, a2nd): eta and phis in space
    (F2S of seeded modes), the rest as in modal_state."""
    m = modal_state(o.n1, o.n2, o.n3_add, o.omega, seed, amp, frac)
    eta = o.fourier.F2S(m[0])
    phis = o.fourier.F2S(m[1] / np.where(o.omega > 0, o.omega, 1.0))
    return [eta, phis, m[2], m[3], m[4], m[5], m[7], m[9], m[6], m[8]]


def zero_state(o):
    n1, n2, n3a = o.n1, o.n2, o.n3_add
    return [np.zeros((n1, n2)), np.zeros((n1, n2))] + [np.zeros((n3a, n2)) for _ in range(4)] + \
        [np.zeros((n1, n2)) for _ in range(4)]


def sample_index(size, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.sort(rng.choice(size, size=min(NSAMPLE, size), replace=False)).astype(np.int64)


def projection_vectors(size, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return _uniform(rng, (NPROJ, size))


def summarize(prefix, arr, seed):
    """Size-independent record of a large array: sampled entries, max |.|,
    sum of squares, projections and the projections' magnitude bounds."""
    a = np.asarray(arr, dtype=np.float64).ravel(order="F")
    idx = sample_index(a.size, seed)
    v = projection_vectors(a.size, seed + 1)
    return {prefix + "_idx": idx, prefix + "_val": a[idx], prefix + "_max": np.array([np.max(np.abs(a))]),
            prefix + "_ss": np.array([float(a @ a)]), prefix + "_proj": v @ a,
            prefix + "_pbound": np.abs(v) @ np.abs(a)}


def compare_summary(fx, prefix, arr, seed, rtol):
    """Check `arr` against the record `summarize` wrote; returns the largest
    relative deviation (of the sampled entries and of max |.|, relative to
    the reference's max |.|; of the projections, relative to their bound)."""
    a = np.asarray(arr, dtype=np.float64).ravel(order="F")
    ref_max = float(fx[prefix + "_max"][0])
    if ref_max == 0.0:
        assert np.max(np.abs(a)) == 0.0, prefix
        return 0.0
    idx = fx[prefix + "_idx"]
    assert np.array_equal(idx, sample_index(a.size, seed)), prefix
    d = np.max(np.abs(a[idx] - fx[prefix + "_val"])) / ref_max
    d = max(d, abs(np.max(np.abs(a)) - ref_max) / ref_max)
    v = projection_vectors(a.size, seed + 1)
    dp = np.max(np.abs(v @ a - fx[prefix + "_proj"]) / np.maximum(fx[prefix + "_pbound"], 1e-300))
    worst = max(d, dp)
    assert worst <= rtol, (prefix, d, dp)
    return worst


def load(name):
    with np.load(os.path.join(GOLDEN, f"baseline_{name}.npz")) as z:
        return {k: z[k] for k in z.files}
