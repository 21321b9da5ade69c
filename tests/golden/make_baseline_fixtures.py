"""Write the oracle fixtures of the benchmark tank configurations
(tests/golden/baseline_{c1,c2,c3,c5}.npz; cases in tests/baseline_cases.py):

  python tests/golden/make_baseline_fixtures.py [--threads N] [c1 c2 c3 c5]
  python tests/golden/make_baseline_fixtures.py [--threads N] --loop-only c3

Per case: one solveHOS2 on a seeded modal state, one runge4_adapt2 on a
seeded physical state (after one right-hand side at the step's start time,
which sets the wavemaker state the step's first volume correction reads),
and, for c1, c2 and c3, the time loop from the initial condition with the
probe records (c3: its first simulated second, the final eta as a sampled
record).  --loop-only adds the loop records to an existing fixture.  The
oracle's transforms use N threads (default 1); c5 and the c3 loop take
tens of minutes.
"""
import os
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "hos-nwt_gb300"), os.path.dirname(HERE)):
    sys.path.insert(0, p)

import numpy as np  # noqa: E402

import baseline_cases as bc  # noqa: E402

LOOP_T = {"c1": None, "c2": 10.0, "c3": 1.0}   # simulated seconds of the time loop (None: the whole run)


def rhs_case(name, w, out, full):
    o = bc.oracle_tank(w)
    y = bc.modal_state(o.n1, o.n2, o.n3_add, o.omega, frac=bc.ENVELOPE.get(name, 0.2))
    out["rhs_alpha_prev"] = np.array([o._alpha[0]])
    out["rhs_pos_top"] = np.array([o._pos[0][o.n3 - 1, 0]])
    k = o.solveHOS2({key: a.copy() for key, a in zip(bc.KEYS, y)}, bc.RHS_DT, bc.RHS_T)
    for i, key in enumerate(bc.KEYS):
        if full:
            out["rhs_" + key] = k[key]
        else:
            out.update(bc.summarize("rhs_" + key, k[key], 100 + i))


def step_case(name, w, out, full):
    o = bc.oracle_tank(w)
    zero = bc.zero_state(o)
    o.solveHOS2({key: a for key, a in zip(bc.KEYS, zero)}, 0.0, bc.STEP_T0)
    st = bc.physical_state(o, frac=bc.ENVELOPE.get(name, 0.2))
    h = 0.8 * o.delt
    res, err, deta, _ = o.runge4_adapt2(bc.STEP_T0, *[a.copy() for a in st], h)
    out["step_h"] = np.array([h])
    out["step_err"] = np.array([err])
    for i, key in enumerate(bc.STEP_KEYS):
        if full:
            out["step_" + key] = res[key]
        else:
            out.update(bc.summarize("step_" + key, res[key], 200 + i))


def loop_case(name, w, out, T):
    inp = dict(w["inp"])
    if T is not None:
        inp["T_stop"] = T
    w = dict(w, inp=inp)
    o = bc.oracle_tank(w)
    recs = o.run()
    out["loop_t"] = np.array([r[0] for r in recs])
    out["loop_probes"] = np.array([r[1] for r in recs])
    if name in bc.SAMPLED:
        out.update(bc.summarize("loop_eta", o.eta, 300))
    else:
        out["loop_eta"] = o.eta
    out["loop_T_stop"] = np.array([inp["T_stop"]])
    out["h"] = np.array([o.h])
    out["Hs"] = np.array([w["Hs"]])


def make(name):
    t0 = time.perf_counter()
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        w = bc.spec(name, tmp)
        full = name not in bc.SAMPLED
        rhs_case(name, w, out, full)
        step_case(name, w, out, full)
        if name in LOOP_T:
            loop_case(name, w, out, LOOP_T[name])
    np.savez_compressed(os.path.join(HERE, f"baseline_{name}.npz"), **out)
    print(name, f"{time.perf_counter() - t0:.1f} s", flush=True)


def add_loop(name):
    """Add the time-loop records to an existing fixture, keeping its others."""
    t0 = time.perf_counter()
    path = os.path.join(HERE, f"baseline_{name}.npz")
    out = dict(np.load(path))
    with tempfile.TemporaryDirectory() as tmp:
        loop_case(name, bc.spec(name, tmp), out, LOOP_T[name])
    np.savez_compressed(path, **out)
    print(name, f"loop {time.perf_counter() - t0:.1f} s", flush=True)


if __name__ == "__main__":
    args = sys.argv[1:]
    if args[:1] == ["--threads"]:
        import oracle.hos_oracle as ho
        ho.set_workers(int(args[1]))
        args = args[2:]
    if args[:1] == ["--loop-only"]:
        for n in args[1:]:
            add_loop(n)
    else:
        for n in (args or ["c1", "c2", "c3", "c5"]):
            make(n)
