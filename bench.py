"""Benchmark of the HOS-NWT hot path: RK4(5) steps per second of one wave
tank, by default the steep 3-D directional tank (1025 x 513 modes, n3 = 33,
M = 7, p1 = p2 = 7, dealiased grid 4100 x 2052; 50 m x 30 m x 5 m, snake
flap, JONSWAP Hs = 0.15 m, Tp = 1.3 s, gamma = 5, cos^2s spreading s = 15;
synthetic seeded phases and directions), the largest benchmark
configuration, run on the plain path (FP64 state, right-hand side and RK
stages; the FFT passes' complex DFT in double-float, HOSNWT_FFT_DF=0 for
FP64).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl cuda|reference]
                  [--workload steep_3d|directional_3d|irregular_2d|regular_2d|...]

One step = one attempted RK4(5) step of runge4_adapt2 (five nonlinear
right-hand sides, error estimate) under the step control of HOS-NWT.f90's
time loop: each timed call of hosnwt_advance takes the tank one accepted
step further, its attempts (rejections included) and the step-size update
running on the device.  `value` = attempts per second, measured with CUDA
events on the library's stream with the state resident on the device, the
L2 cache flushed between calls (a 256 MiB write outside the timed events);
`e2e` is the same metric through hosnwt_runge4_adapt2 on pinned host arrays
(host-to-device copy of the 10 state arrays and device-to-host copy of the
results inside each timed call) with the same step control on the host.  Under torchrun every rank runs its own
replica tank (the path does not shard); value = total steps/s.

--impl reference times the CPU restatement of the reference (the oracle:
numpy/scipy FP64, its transforms threaded over every host core; the Fortran
reference cannot be built on these hosts) on the same tank: whole steps
when they fit in a few minutes, else a bounded sample of right-hand sides
scaled to steps (the line's cpu_baseline.sample says which).

Other workloads (--workload): directional_3d (3-D tank, 513 x 257, M = 5,
p = 4), irregular_2d (2-D JONSWAP tank, n1 = 1025, M = 5), regular_2d (2-D
regular-wave tank, n1 = 257, M = 3), ensemble (64 independent 2-D tanks),
tc_gemm (the surrogate's tensor-core contraction), surrogate (the offline
FNO).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "hos-nwt_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

import workloads  # noqa: E402

METRIC = "RK4(5) steps/s (sim-s/wall-s reported alongside)"
UNIT = "steps/s"


WORKLOAD_TEXT = {
    "directional_3d": "directional_3d: 3-D directional JONSWAP tank 50 m x 30 m x 5 m, snake flap hinged 2.0 m "
                      "above the bottom, Hs=0.08 m Tp=1.2 s gamma=3.3, cos^2s spreading s=10, n1=513 n2=257 "
                      "n3=33 M=5 p1=p2=4, RK4(5) tol 1e-7",
    "steep_3d": "steep_3d: 3-D directional JONSWAP tank 50 m x 30 m x 5 m, snake flap hinged 2.0 m above "
                "the bottom, Hs=0.15 m Tp=1.3 s gamma=5, cos^2s spreading s=15, n1=1025 n2=513 n3=33 M=7 "
                "p1=p2=7, RK4(5) tol 1e-7",
    "irregular_2d": "irregular_2d: 2-D JONSWAP tank 50 m x 5 m, flap, 512 components, "
                    "n1=1025 n3=65 M=5 p1=5, RK4(5) tol 1e-7",
    "regular_2d": "regular_2d: 2-D regular wave T=1.0 s H=0.05 m, tank 50 m x 5 m, flap hinged 2.0 m above "
                  "the bottom, 3 s ramp, n1=257 n3=33 M=3 p1=3, RK4(5) tol 1e-7",
}
SINGLE_TANK = ("directional_3d", "steep_3d", "irregular_2d", "regular_2d")


def _single_tank(name, directory):
    if name == "directional_3d":
        return workloads.directional_3d(directory)
    if name == "steep_3d":
        return workloads.steep_3d(directory)
    if name == "irregular_2d":
        return workloads.irregular_2d(directory)
    return workloads.regular_2d()


def _workload_config(w):
    """The workload's `config`: the same dict in both arms."""
    cfg = {"workload": WORKLOAD_TEXT[w["name"]],
           "n1": w["n1"], "n2": w["n2"], "n3": w["n3"], "mHOS": w["mHOS"], "p1": w["p1"], "p2": w["p2"],
           "l2": "flushed between steps (256 MiB write outside the timed events)",
           "parallelism": "replicas"}
    if w["name"] == "irregular_2d":
        cfg.update({"wave_components": 512, "seed": 513})
    if w["name"] == "directional_3d":
        cfg.update({"seed": 2025})
    if w["name"] == "steep_3d":
        cfg.update({"seed": 200})
    return cfg


def _tank_info(info):
    """Sizes and step of the tank the library built (beside `config`)."""
    return {"nd1": info["nd1"], "nd2": info["nd2"], "n3_add": info["n3_add"], "dt_nondim": info["delt"],
            "dt_s": info["delt"] * info["Tscale"]}


def _host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for i, n in enumerate(names):
                    if r[5 + i].lower().startswith("active"):
                        reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


class NvmlClocks:
    """SM clock and clock-event reasons read through NVML (libnvidia-ml,
    read-only queries) every few milliseconds in a thread, so that a timed
    region of tens of milliseconds still gets samples under load."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index=0, period_s=0.002):
        self.index, self.period = index, period_s
        self.sm, self.reasons, self.max_mhz = [], set(), None
        self.lib = None

    def __enter__(self):
        import ctypes
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return self
            h = ctypes.c_void_p()
            if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.index), ctypes.byref(h)) != 0:
                lib.nvmlShutdown()
                return self
            mx = ctypes.c_uint()
            if lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:
                self.max_mhz = float(mx.value)
            self.lib, self.h = lib, h
            self.get_reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
            self.stop = threading.Event()
            self.t = threading.Thread(target=self._run, daemon=True)
            self.t.start()
        except Exception:
            self.lib = None
        return self

    def _run(self):
        import ctypes
        c, r = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop.is_set():
            if self.lib.nvmlDeviceGetClockInfo(self.h, 1, ctypes.byref(c)) == 0:  # NVML_CLOCK_SM
                self.sm.append(float(c.value))
            if self.get_reasons(self.h, ctypes.byref(r)) == 0:
                for bit, name in self.REASONS.items():
                    if r.value & bit:
                        self.reasons.add(name)
            self.stop.wait(self.period)

    def __exit__(self, *a):
        if self.lib is not None:
            self.stop.set()
            self.t.join(timeout=5)
            self.lib.nvmlShutdown()


def _clocks(smi, nv):
    """Clock record of the timed region: the NVML samples (dense) with the
    nvidia-smi ones (200 ms apart) as a cross-check."""
    out = smi.summary()
    if nv.sm:
        out = {"sm_mhz": statistics.median(nv.sm), "sm_max_mhz": nv.max_mhz or out.get("sm_max_mhz"),
               "reasons": sorted(set(out.get("reasons", [])) - {"unavailable"} | nv.reasons),
               "samples": len(nv.sm), "source": "nvml every 2 ms",
               "nvidia_smi": {"sm_mhz": out.get("sm_mhz"), "samples": out.get("samples", 0)}}
    return out


def _measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "of measured"
    return 6800.0, "of fallback"


def _fp64_step(fmas, ms, peak_gflops):
    """FP64 rate of a whole step: the FMAs of its transform passes (counted
    by the library as it builds the step graph) over the step's device
    time, against the FP64 peak measured live."""
    g = 2.0 * fmas / (ms * 1e-3) / 1e9
    return {"transform_fmas_per_step": fmas, "achieved_gflops": g, "peak_gflops": peak_gflops,
            "frac": g / peak_gflops}


def _fused_pass():
    """The library runs 2-D x passes as one fused kernel when
    HOSNWT_FUSED_PASS=1, else as the two-launch pass pair."""
    return os.environ.get("HOSNWT_FUSED_PASS", "0")[:1] == "1"


# ncu summaries (profiles/) of the roofline transform of each workload
PROFILE_OF = {"directional_3d": "roofline_transform_directional_3d.md",
              "steep_3d": "roofline_transform_steep_3d.md",
              "irregular_2d": "roofline_transform_irregular_2d.md"}


def _profile_traffic(name):
    """Per-launch DRAM traffic of the roofline transform from the committed
    ncu summary of this workload, if present."""
    fn = PROFILE_OF.get(name)
    p = os.path.join(ROOT, "profiles", fn) if fn else None
    if not p or not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def _oracle(w, threads):
    import oracle.hos_oracle as ho
    ho.set_workers(threads)
    return ho.Tank(w["inp"], w["n1"], w["n2"], w["n3"], w["mHOS"], w["p1"], w["p2"],
                   wave_files_dir=w["wave_dir"])


STATE_OUT = ("eta", "phis", "a_add_1", "a_add_2", "a_add_ramp", "a_add_3", "eta1st", "eta2nd", "a1st", "a2nd")


def _rhs_state(o):
    """The modal state of the first stage of runge4_adapt2 from the tank's
    current physical state (runge_kutta.f90:125-141)."""
    eta, phis, a1, a2, ar, a3, e1, e2, a1st, a2nd = o.state_tuple()
    F = o.fourier
    return dict(G1=F.S2F(eta), G2=F.S2F(phis) * o.omega, a_add_1=a1, a_add_2=a2, a_add_ramp=ar, a_add_3=a3,
                a1st=a1st, eta1st=e1, a2nd=a2nd, eta2nd=e2)


def _time_rhs(o, y, h):
    t0 = time.perf_counter()
    o.solveHOS2({k: v.copy() for k, v in y.items()}, h, 0.0)
    return time.perf_counter() - t0


def _oracle_rate(w, steps, warmup, budget_s):
    """Steps/s of the oracle on the tank of `w`, its transforms on every host
    core: whole RK4(5) steps when `steps + warmup` of them fit in
    `budget_s`, else a bounded sample of right-hand-side evaluations (a step
    is five of them plus stage combinations that cost under one percent of
    a step at these sizes), scaled to steps.  Returns (value, sample text,
    cores, h)."""
    cores = _host_cores()
    o = _oracle(w, cores)
    h = o.delt
    y = _rhs_state(o)
    t_rhs = _time_rhs(o, y, h)  # warm-up (transform plans) and the size of a step
    if 5.0 * t_rhs * (steps + warmup) <= budget_s:
        st = list(o.state_tuple())
        t = 0.0
        for _ in range(warmup):
            res, err, deta, _ = o.runge4_adapt2(t, *st, h)
            st = [res[k] for k in STATE_OUT]
            t += h
        n, t0 = 0, time.perf_counter()
        while n < steps:
            res, err, deta, _ = o.runge4_adapt2(t, *st, h)
            st = [res[k] for k in STATE_OUT]
            t += h
            n += 1
        el = time.perf_counter() - t0
        return n / el, f"{n} RK4(5) steps after {warmup} warm-up steps, {el:.1f} s", cores, h
    n, tot = 0, 0.0
    while n < max(2, steps) and (n < 2 or tot < budget_s):
        tot += _time_rhs(o, y, h)
        n += 1
    return n / (5.0 * tot), (f"{n} right-hand sides (solveHOS2) after one warm-up, {tot:.1f} s, scaled to "
                             f"steps at 5 per RK4(5) step"), cores, h


def cpu_baseline(w, budget_s=30.0):
    """The oracle (numpy/scipy FP64, transforms threaded over the host's
    cores) on a bounded sample of the same tank."""
    v, sample, cores, _ = _oracle_rate(w, 400, 0, budget_s)
    return {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{w['name']} tank (n1={w['n1']}, n2={w['n2']}, M={w['mHOS']}), numpy/scipy oracle on "
                      f"{cores} threads: {sample}"}


def run_reference(args, w):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    v, sample, cores, h = _oracle_rate(w, args.steps, args.warmup, 240.0)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": _workload_config(w),
            "sim_s_per_wall_s": v * h * math.sqrt(w["inp"]["h"] / 9.81),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{sample}; transforms on {cores} threads (CPU restatement of the "
                                       "Fortran reference; it is not buildable here: no gfortran/FFTW)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_cuda(args, w):
    import torch
    import hosnwt

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device (the product has no CPU path)")
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    tank = hosnwt.Tank(w["inp"], w["n1"], w["n2"], w["n3"], w["mHOS"], w["p1"], w["p2"],
                       probes=w["probes"], wave_dir=w["wave_dir"])
    info = tank.info()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    # roofline of the dominant work: a FOURIER_2_SPACE_BIG of the n1 x n2
    # extended modes (both passes; batch of four in a 2-D tank), the shape of
    # the HOS order loop, replayed back to back in a CUDA graph
    n1, n2, nd1, nd2 = info["n1"], info["n2"], info["nd1"], info["nd2"]
    batch = 1 if n2 > 1 else 4
    ms_tl = tank.time_transform("big", -1, "cos", "cos", (n1, n2), (nd1, nd2), batch=batch, nrep=20)

    def l2_flush():
        flush.zero_()
        torch.cuda.synchronize()

    # the time loop of HOS-NWT.f90:498-571 one accepted step at a time: each
    # hosnwt_advance to time_cur + h runs the RK4(5) attempts (rejections
    # included) and the step-size control on the device, and the L2 flush
    # sits between the calls; a "step" of the metric is one attempted
    # RK4(5) step, as in the reference's loop
    h = info["delt"]

    def one_step(h):
        t = tank.info()["time_cur"]
        h_new, na, nr = tank.advance(t + h, h)
        return h_new, na + nr

    for _ in range(args.warmup):
        h, _ = one_step(h)
    l2_flush()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    attempts = 0
    with ClockSampler(local) as clk, NvmlClocks(local) as nv:
        info0 = tank.info()
        ms0, t_sim0 = info0["device_ms"], info0["time_cur"]
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            l2_flush()
            h, n = one_step(h)
            attempts += n
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        info = tank.info()
        dev_ms = info["device_ms"] - ms0
        sim_s = (info["time_cur"] - t_sim0) * info["Tscale"]
    if dist is not None:
        t = torch.tensor([dev_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms = float(t.item())
        dist.barrier()
    value = world * attempts / (dev_ms * 1e-3)

    # e2e: the drop-in call (hosnwt_runge4_adapt2, runge_kutta.f90:81) on
    # pinned host arrays, its copies inside the call, driven by the same
    # step control on the host: each attempt copies the state to the work
    # arrays, and an accepted attempt swaps them (HOS-NWT.f90:498-571)
    na = info["n3_add"]
    shapes = [(n1, n2)] * 2 + [(na, n2)] * 4 + [(n1, n2)] * 4
    state, work = [], []
    for s in shapes * 2:
        buf = torch.empty(s[0] * s[1], dtype=torch.float64, pin_memory=True)
        (state if len(state) < len(shapes) else work).append(buf.numpy().reshape(s, order="F"))
    tank.get_rk_state(state)
    toler, dt_stab, dout = info["toler"], info["dt_stab"], info["delt_out"]
    clock = {"t": info["time_cur"], "h": h}

    def e2e_attempt():
        nonlocal state, work
        for a, b in zip(work, state):
            np.copyto(a, b)
        err = tank.runge4_adapt2_inplace(clock["t"], work, clock["h"])
        hr = clock["h"]
        if err > toler and hr > 0.001 * 0.95 * dt_stab:
            corr = float(np.float32(0.9)) * (err / toler) ** -0.25
        else:
            state, work = work, state
            clock["t"] += hr
            corr = 2.0 if abs(err) < np.finfo(np.float64).eps else 0.9 * (err / toler) ** -0.25
        hr = min(hr * corr, 0.95 * dt_stab, dout)
        clock["h"] = max(hr, 0.0001 * 0.95 * dt_stab, 0.0001 * dout)

    for _ in range(max(1, args.warmup)):
        e2e_attempt()
    e2e_s = 0.0
    for _ in range(args.steps):
        l2_flush()
        t0 = time.perf_counter()
        e2e_attempt()
        e2e_s += time.perf_counter() - t0
    if dist is not None:
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * args.steps / e2e_s
    io_bytes = 8 * sum(s[0] * s[1] for s in shapes)

    ms = ms_tl
    # the FFT passes (and with them the double-float DFT) run in 3-D tanks;
    # 2-D tanks take the FP64 sum passes
    df = os.environ.get("HOSNWT_FFT_DF", "1")[:1] != "0" and n2 > 1
    alg_bytes = 16.0 * nd1 * nd2 * batch  # 8-byte read + 8-byte write per output element
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    peak, peak_src = _measured_peaks()
    fp64_peak = hosnwt.fp64_peak_gflops()
    traffic = _profile_traffic(w["name"])

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dev_ms / attempts, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": _workload_config(w), "tank": _tank_info(info),
                "sim_s_per_wall_s": sim_s / (dev_ms * 1e-3),
                "attempted_steps": attempts, "accepted_steps": args.steps,
                "wall_ms_per_step": 1e3 * wall / attempts,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": io_bytes,
                        "d2h_bytes_per_step": io_bytes},
                "gpu_launches": (info["kernels_per_step"] + 3) * attempts,
                "fp64_step": _fp64_step(info["fmas_per_step"], dev_ms / attempts, fp64_peak),
                "clocks": _clocks(clk, nv),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic,
                             "peak_source": peak_src,
                             "kernel": f"the transform passes of {batch} x FOURIER_2_SPACE_BIG of {n1} x {n2} "
                                       f"modes to the {nd1} x {nd2} grid",
                             "ms_per_launch": ms,
                             "timing": "the transform's launches, 20 replays in one CUDA graph, CUDA events on "
                                       "the library's stream",
                             "note": ("not HBM bound: the passes' DFT runs in double-float on the FP32 pipe "
                                      "(bound by instruction issue); fp64_step gives the step's transform work "
                                      "in FP64 instructions against the FP64 peak" if df else
                                      "FP64-pipe bound, not HBM bound: GB300 runs FP64 at about 1.2 TFLOP/s; "
                                      "fp64_step gives the step's transform FMAs against the FP64 peak")},
                "arithmetic": ("FP64 state, right-hand side and RK stages; the FFT passes' complex DFT in "
                               "double-float (pairs of FP32, 48-bit significand)" if df else
                               "FP64 throughout" + (" (HOSNWT_FFT_DF=0)" if n2 > 1 else
                                                    " (a 2-D tank: FP64 sum passes)")),
                }
        if world == 1:
            line["cpu_baseline"] = cpu_baseline(w)
        print(json.dumps(line), flush=True)
    tank.close()
    if dist is not None:
        dist.destroy_process_group()


def run_ensemble(args):
    """Pattern 2: 64 independent 2-D tanks of uneven n1 / M, advanced by the
    same simulated time one after another and then all together
    (hosnwt_advance_many, one stream per tank).  Reports aggregate simulated
    tank-seconds per wall-second of both and their ratio.  Under torchrun
    the tanks are split into contiguous cost-balanced blocks, one per rank
    (ensemble.shard); the ranks exchange nothing while the tanks run, and
    the wall times are the maximum over ranks (strong scaling: the ensemble
    is fixed as ranks are added)."""
    import torch
    import hosnwt
    import ensemble
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device (the product has no CPU path)")
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    all_specs = workloads.ensemble()
    sim_s = args.sim_seconds
    start, stop = ensemble.shard(all_specs, rank, world, sim_s)
    specs = all_specs[start:stop]
    tanks = [hosnwt.Tank(s["inp"], s["n1"], 1, s["n3"], s["mHOS"], s["p1"], 1, probes=s["probes"])
             for s in specs]
    infos = [t.info() for t in tanks]
    # warm-up: every tank a short stretch alone
    h = [i["delt"] for i in infos]
    for k, t in enumerate(tanks):
        h[k], _, _ = t.advance(0.05 / infos[k]["Tscale"], h[k])
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    steps0 = sum(t.info()["n_rhs"] for t in tanks)
    for k, t in enumerate(tanks):
        inf = t.info()
        h[k], _, _ = t.advance(inf["time_cur"] + sim_s / inf["Tscale"], h[k])
    torch.cuda.synchronize()
    seq = time.perf_counter() - t0
    steps_seq = sum(t.info()["n_rhs"] for t in tanks) - steps0
    n_mid = [t.info()["n_rhs"] for t in tanks]
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    tn = [t.info()["time_cur"] + sim_s / t.info()["Tscale"] for t in tanks]
    if tanks:
        h = list(hosnwt.advance_many(tanks, tn, h))
    torch.cuda.synchronize()
    bat = time.perf_counter() - t0
    steps_bat = sum(t.info()["n_rhs"] for t in tanks) - steps0 - steps_seq
    # FP64 work of the batched run: each tank's attempted steps times the
    # transform FMAs of its step graph
    n_end = [t.info()["n_rhs"] for t in tanks]
    fmas_bat = sum((n_end[k] - n_mid[k]) // 5 * tanks[k].info()["fmas_per_step"] for k in range(len(tanks)))
    summaries = [{"tank": start + k, "n1": specs[k]["n1"], "mHOS": specs[k]["mHOS"],
                  "time_s": t.info()["time_cur"] * t.info()["Tscale"], "rhs": n_end[k]}
                 for k, t in enumerate(tanks)]
    if dist is not None:
        v = torch.tensor([seq, bat, float(fmas_bat), float(steps_seq), float(steps_bat)], device="cuda",
                         dtype=torch.float64)
        mx = v.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(v, op=dist.ReduceOp.SUM)
        seq, bat = float(mx[0]), float(mx[1])
        fmas_bat, steps_seq, steps_bat = float(v[2]), int(v[3]), int(v[4])
    gathered = ensemble.gather_summaries(summaries, start, len(all_specs))
    fp64_peak = hosnwt.fp64_peak_gflops()
    if rank == 0:
        n_all = len(all_specs)
        line = {"metric": "ensemble tank-sim-s/wall-s (64 independent 2-D tanks)", "value": n_all * sim_s / bat,
                "unit": "tank-sim-s/wall-s", "n_gpus": world, "higher_is_better": True, "dtype": "f64",
                "scaling": "strong", "data": "synthetic",
                "config": {"workload": "ensemble: 64 x 2-D JONSWAP tanks, n1 in {129..2049}, M in {3,5,7}, "
                                       "p1=M, tol 1e-7, per-tank adaptive dt", "sim_seconds_per_tank": sim_s,
                           "parallelism": f"tank blocks over {world} rank(s), no collective while running"},
                "sequential_value": n_all * sim_s / seq, "batched_over_sequential": seq / bat,
                "rk_steps": {"sequential": steps_seq // 5, "batched": steps_bat // 5},
                "wall_s": {"sequential": seq, "batched": bat},
                "tanks_reported": sum(1 for s in gathered if s is not None),
                "fp64_batched": {"transform_fmas": fmas_bat, "achieved_gflops": 2.0 * fmas_bat / bat / 1e9,
                                 "peak_gflops": fp64_peak * world,
                                 "frac": 2.0 * fmas_bat / bat / 1e9 / (fp64_peak * world),
                                 "note": "the transform FMAs alone; the batched run is bound by the FP64 "
                                         "pipes, so its ratio to the sequential run is capped by how "
                                         "much FP64 work the sequential tanks leave idle"}}
        print(json.dumps(line), flush=True)
    for t in tanks:
        t.close()
    if dist is not None:
        dist.destroy_process_group()


GEMM_SHAPES = [
    # (name, M, N, K)
    ("square 8192^3 (tensor-bound)", 8192, 8192, 8192),
    ("surrogate channel mix on the 2052 x 1028 dealiased grid (32 -> 32 channels)", 2052 * 1028, 32, 32),
    ("surrogate truncated x transform as a contraction (1028 x 32 lines, 64 modes, 2052 points "
     "zero-padded to K = 2056, the multiple of 8 that TMA row strides need)", 1028 * 32, 64, 2056),
]


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), float(d.get("bf16_tflops", 1900.0)), "of measured"
    return 6800.0, 1900.0, "of fallback"


def run_tc_gemm(args):
    """The surrogate's tensor-core contraction (tc_gemm.cu: TMA, tcgen05.mma,
    TMEM accumulator) on its shapes: D = A B^T with A (M x K), B (N x K)
    BF16, FP32 accumulate, FP32 out; CUDA events on the launching stream,
    `--steps` launches after `--warmup`.  Beside it, torch.matmul (cuBLAS)
    on the same BF16 operands, for reference only."""
    import torch
    import hosnwt
    hbm, bf16, src = _peaks()
    st = torch.cuda.current_stream()
    rows = []
    for name, M, N, K in GEMM_SHAPES:
        g = torch.Generator(device="cuda").manual_seed(M + N + K)
        A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
        B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
        D = torch.empty(M, N, device="cuda", dtype=torch.float32)
        err = torch.zeros(1, dtype=torch.int32, device="cuda")

        def ours():
            hosnwt.tc_gemm(A, B, out=D, err=err, stream=st.cuda_stream)

        def cublas():
            torch.matmul(A, B.T)

        res = {}
        for tag, fn in (("tc_gemm", ours), ("cublas", cublas)):
            for _ in range(max(3, args.warmup)):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(args.steps):
                fn()
            e1.record(st)
            torch.cuda.synchronize()
            res[tag] = e0.elapsed_time(e1) / args.steps
        assert int(err.item()) == 0, "tc_gemm: a wait timed out"
        ref = (A[:256].float() @ B.float().T)
        assert (D[:256] - ref).abs().max().item() <= 1e-5 * (A[:256].float().abs() @ B.float().abs().T).max().item()
        flops = 2.0 * M * N * K
        alg_bytes = 2.0 * (M * K + N * K) + 4.0 * M * N
        ai = flops / alg_bytes
        ms = res["tc_gemm"]
        tflops = flops / (ms * 1e-3) / 1e12
        gbs = alg_bytes / (ms * 1e-3) / 1e9
        tensor_bound = ai > bf16 * 1e3 / hbm
        rows.append({"shape": name, "M": M, "N": N, "K": K, "ms": ms, "tflops": tflops, "gbs": gbs,
                     "bound": "tensor" if tensor_bound else "hbm",
                     "frac": tflops / bf16 if tensor_bound else gbs / hbm,
                     "cublas_ms": res["cublas"],
                     "cublas_note": "torch.matmul, BF16 out"})
        del A, B, D
        torch.cuda.empty_cache()
    print(json.dumps({"metric": "tc_gemm throughput (surrogate contractions)", "unit": "TFLOP/s | GB/s",
                      "peaks": {"bf16_tflops": bf16, "hbm_gbs": hbm, "source": src},
                      "steps": args.steps, "warmup": args.warmup, "dtype": "bf16 in, f32 accumulate",
                      "shapes": rows}), flush=True)


def run_profile_gemm(args):
    """One tc_gemm launch per shape of GEMM_SHAPES between cudaProfilerStart
    and cudaProfilerStop, for `ncu --profile-from-start off -k regex:k_tc_gemm`."""
    import torch
    import hosnwt
    st = torch.cuda.current_stream()
    ops = []
    for name, M, N, K in GEMM_SHAPES:
        A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
        B = torch.randn(N, K, device="cuda").to(torch.bfloat16)
        D = torch.empty(M, N, device="cuda", dtype=torch.float32)
        ops.append((A, B, D))
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    for A, B, D in ops:
        hosnwt.tc_gemm(A, B, out=D, err=err, stream=st.cuda_stream)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    assert int(err.item()) == 0
    print(json.dumps({"profile_gemm": [s[0] for s in GEMM_SHAPES]}), flush=True)


def run_surrogate(args):
    """The surrogate for the orders 4..7 of W (pattern 4), offline: a 2-D
    irregular tank (n1 = 513, M = 7, p1 = 7) runs on the plain FP64 GPU
    path; snapshots of eta, phizm(1..3) and phizm(4..7) (hosnwt_hos_terms)
    are taken every 0.1 s from 5 to 45 s of one wave realisation (seed 513)
    for training and from 20 to 40 s of another (seed 600) for testing.  A
    4-layer, 32-channel FNO with 64 cosine modes is trained on the tensor
    cores (BF16 in, FP32 accumulate) and its held-out error is reported,
    relative to the orders 4..7 part and to the whole W."""
    import torch
    import hosnwt
    import surrogate

    def make(seed, tmp):
        w = workloads.irregular_2d(tmp, seed=seed, n1=513, n3=33, mHOS=7, p1=7, T_stop=60.0)
        return hosnwt.Tank(w["inp"], w["n1"], 1, w["n3"], w["mHOS"], w["p1"], 1, probes=w["probes"],
                           wave_dir=w["wave_dir"])

    t0 = time.perf_counter()
    with tempfile.TemporaryDirectory() as tmp:
        tank = make(513, tmp)
    nd = tank.info()["nd1"]
    Xtr, Ytr, Wtr, _ = surrogate.collect(tank, 5.0, 45.0, 0.1, tank.info()["delt"])
    # plain M = 7 step time on this tank (device-resident, CUDA events)
    h = tank.info()["delt"]
    for _ in range(3):
        tank.step(h)
    torch.cuda.synchronize()
    ms0 = tank.info()["device_ms"]
    for _ in range(20):
        tank.step(h)
    step_ms = (tank.info()["device_ms"] - ms0) / 20
    tank.close()
    with tempfile.TemporaryDirectory() as tmp:
        tank = make(600, tmp)
    Xte, Yte, Wte, _ = surrogate.collect(tank, 20.0, 40.0, 0.1, tank.info()["delt"])
    tank.close()
    t_collect = time.perf_counter() - t0
    model = surrogate.build_fno(nd)
    iters = max(args.steps, 1) * 40
    losses, t_train, sc = surrogate.train(model, Xtr, Ytr, iters=iters, batch=32, lr=3e-3)
    pred = surrogate.predict(model, Xte, sc)
    err = pred - Yte
    rel_hi = float(np.linalg.norm(err) / np.linalg.norm(Yte))
    rel_w = float(np.linalg.norm(err) / np.linalg.norm(Wte))
    share = float(np.linalg.norm(Yte) / np.linalg.norm(Wte))
    per_snap = np.linalg.norm(err, axis=1) / np.maximum(np.linalg.norm(Wte, axis=1), 1e-300)
    # inference time of one field and of the five of an RK4(5) step
    xs, ys = sc
    times = {}
    for b in (1, 5):
        Xt = torch.tensor(Xte[:b] / xs, dtype=torch.float32, device="cuda")
        with torch.no_grad():
            for _ in range(3):
                model(Xt)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(20):
                model(Xt)
            e1.record()
            torch.cuda.synchronize()
        times[b] = e0.elapsed_time(e1) / 20
    surrogate.check_kernel_flags()
    print(json.dumps({
        "metric": "surrogate (orders 4..7 of W): held-out relative error", "value": rel_hi,
        "unit": "||pred - W_4..7|| / ||W_4..7||", "higher_is_better": False, "dtype": "bf16 in, f32 accumulate",
        "data": "synthetic: snapshots of the plain FP64 GPU solver",
        "config": {"workload": "surrogate: 2-D irregular JONSWAP tank, n1=513 n3=33 M=7 p1=7, Hs=0.10 m Tp=1.4 s; "
                               "train seed 513 t=5..45 s, test seed 600 t=20..40 s, every 0.1 s",
                   "nd1": nd, "fno": "4 layers, 32 channels, 64 cosine modes", "train_iters": iters, "batch": 32},
        "snapshots": {"train": int(Xtr.shape[0]), "test": int(Xte.shape[0])},
        "error_relative_to_W": rel_w, "orders_4_7_share_of_W": share,
        "per_snapshot_error_relative_to_W": {"median": float(np.median(per_snap)), "max": float(np.max(per_snap))},
        "loss": {"first10": float(np.mean(losses[:10])), "last10": float(np.mean(losses[-10:]))},
        "seconds": {"collect": t_collect, "train": t_train},
        "inference_ms": {"one_field": times[1], "five_fields": times[5]},
        "plain_m7_step_ms": step_ms,
        "note": "offline: the surrogate is not used inside the time loop"}), flush=True)


def run_profile_step(args, w):
    """One step of a tank between cudaProfilerStart / cudaProfilerStop, after
    `--warmup` untimed steps, for `ncu --profile-from-start off`: the capture
    then holds exactly the kernels of one step graph and its accept."""
    import torch
    import hosnwt
    tank = hosnwt.Tank(w["inp"], w["n1"], w["n2"], w["n3"], w["mHOS"], w["p1"], w["p2"],
                       probes=w["probes"], wave_dir=w["wave_dir"])
    info = tank.info()
    h = info["delt"]
    for _ in range(args.warmup):
        tank.step(h)
        tank.accept(h)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    tank.step(h)
    tank.accept(h)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"profile_step": w["name"], "kernels_per_step": info["kernels_per_step"],
                      "fmas_per_step": info["fmas_per_step"], "n1": info["n1"], "n2": info["n2"],
                      "nd1": info["nd1"], "nd2": info["nd2"]}), flush=True)
    tank.close()


def run_profile_roofline(args, w):
    """The roofline transform of run_cuda (FOURIER_2_SPACE_BIG of the n1 x n2
    extended modes; a batch of four in a 2-D tank) once inside a
    cudaProfilerStart / Stop range, for `ncu --profile-from-start off`.
    time_transform runs the transform three times uncaptured before its
    graph replay: the capture holds those three and the replay."""
    import torch
    import hosnwt
    tank = hosnwt.Tank(w["inp"], w["n1"], w["n2"], w["n3"], w["mHOS"], w["p1"], w["p2"],
                       probes=w["probes"], wave_dir=w["wave_dir"])
    info = tank.info()
    n1, n2, nd1, nd2 = info["n1"], info["n2"], info["nd1"], info["nd2"]
    batch = 1 if n2 > 1 else 4
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    tank.time_transform("big", -1, "cos", "cos", (n1, n2), (nd1, nd2), batch=batch, nrep=1)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"profile_roofline": w["name"], "n1": n1, "n2": n2, "nd1": nd1, "nd2": nd2,
                      "batch": batch}), flush=True)
    tank.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="cuda", choices=("cuda", "reference"))
    ap.add_argument("--workload", default="steep_3d",
                    choices=SINGLE_TANK + ("ensemble", "tc_gemm", "surrogate"))
    ap.add_argument("--sim-seconds", type=float, default=1.0, help="ensemble: simulated seconds per tank")
    ap.add_argument("--profile-step", action="store_true",
                    help="run one step inside a cudaProfilerStart/Stop range (for ncu) and exit")
    ap.add_argument("--profile-roofline", action="store_true",
                    help="run the roofline transform once inside a cudaProfilerStart/Stop range and exit")
    ap.add_argument("--profile-n2", type=int, default=0,
                    help="with --profile-roofline: a narrower tank of the same x length (n2 modes, same p2), "
                         "so that a full ncu capture of the x pass holds a few GB on the device")
    args = ap.parse_args()
    if args.workload == "tc_gemm":
        run_profile_gemm(args) if args.profile_step else run_tc_gemm(args)
        return
    if args.workload == "surrogate":
        run_surrogate(args)
        return
    if args.workload == "ensemble":
        run_ensemble(args)
        return
    with tempfile.TemporaryDirectory() as tmp:
        w = _single_tank(args.workload, tmp)
        if args.profile_n2 > 0:
            w = dict(w, n2=args.profile_n2)
        if args.profile_roofline:
            run_profile_roofline(args, w)
        elif args.profile_step:
            run_profile_step(args, w)
        elif args.impl == "reference":
            run_reference(args, w)
        else:
            run_cuda(args, w)


if __name__ == "__main__":
    main()
