"""Synthetic tank configurations with the shapes of the benchmark cases.

No public data set is involved: each case writes its own input (and, for
the irregular cases, a .cfg/.dat wave file with seeded random phases) with
the tank, wavemaker, spectrum and numerical sizes stated below.

  regular_2d    2-D regular wave: 50 m tank, h = 5 m, flap hinged 2.0 m above
                the bottom, T = 1.0 s, H = 0.05 m, 3 s linear ramp,
                n1 = 257, n3 = 33, M = 3, p1 = 3, tol 1e-7, probes 5/10/20 m
  irregular_2d  2-D JONSWAP Hs = 0.10 m, Tp = 1.4 s, gamma = 3.3, 512
                components (harmonics 128..639 of 1/256 Hz, 0.5-2.5 Hz),
                phases U[0, 2 pi) from numpy PCG64(seed); n1 = 1025, n3 = 65,
                M = 5, p1 = 5, tol 1e-7, probes 5/10/15/20/30 m
  directional_3d  50 x 30 m tank, snake flap, JONSWAP Hs = 0.08 m, Tp = 1.2 s,
                cos^2s spreading (s = 10) drawn per frequency bin;
                n1 = 513, n2 = 257, n3 = 33, M = 5, p1 = p2 = 4
  steep_3d      the same tank with JONSWAP Hs = 0.15 m, Tp = 1.3 s, gamma = 5,
                s = 15; n1 = 1025, n2 = 513, n3 = 33, M = 7, p1 = p2 = 7
Every case uses an absorbing beach over the last 10 m (xabsf = 0.8).
"""
from __future__ import annotations

import math
import os

import numpy as np

G = 9.81


def base_input(**kw):
    d = dict(xlen=50.0, ylen=30.0, h=5.0, icase=2, islosh=3, aslosh=0.02, amp_mono=0.025,
             nu_mono=1.0, theta_mono=0.0, ph_mono=0.0, ibat=2, xd_mono=18.0, file_name="",
             i_cut=0, nuc_low=0.3, nuc_high=3.0, Hs=0.05, Tp=1.0, gamma=3.3, iseed=513,
             i_wmk=1, igeom=2, d_hinge=2.0, iramp=1, Tramp=3.0, iabsnb=1, xabsf=0.8,
             coeffabsf=1.0, iprobes=1, pro_file="prob.inp", T_stop=30.0, toler=1e-7, f_out=10.0,
             idim=1, i3d=0, imodes=0, iwmk=0, i_sw=0)
    d.update(kw)
    return d


def jonswap_density(f, Hs, Tp, gamma):
    """JONSWAP S(f) with sigma 0.07 / 0.09, the shape of
    initial_condition.f90:261-265, before the Hs rescaling."""
    sigma = np.where(f < 1.0 / Tp, 0.07, 0.09)
    return (1.0 / (2 * np.pi) ** 4 * G ** 2 / f ** 5 * np.exp(-1.25 * (f * Tp) ** -4)
            * gamma ** np.exp(-(f - 1.0 / Tp) ** 2 / (2.0 * (sigma / Tp) ** 2)))


def write_wave_files(directory, name, harmo, clock, rnum, amp, angle_deg, phase, depth, Ly,
                     hinge, cut_lo, cut_hi, ramp=3.0):
    """.cfg/.dat wave files in the layout file2wave reads
    (wave_def.f90:181-278): cfg lines rnum, clock, depth, ramp, typ_ramp,
    cutoff_low, cutoff_high, Ly, typ_wmk, hinge; dat lines
    harmo, freq, ampli, angle, phase."""
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, name + ".cfg"), "w") as f:
        for v in (f"{rnum:3d}", clock, depth, ramp, "lin", cut_lo, cut_hi, Ly, "hinged", hinge):
            f.write(f" {v} \n")
    freq = harmo * clock / 2.0 ** rnum
    with open(os.path.join(directory, name + ".dat"), "w") as f:
        for hh, fr, a, an, ph in zip(harmo, freq, amp, angle_deg, phase):
            f.write(f"{int(hh)} , {fr:.15e} , {a:.15e} , {an:.15e} , {ph:.15e} ,\n")


def irregular_2d(directory, seed=513, n1=1025, n3=65, mHOS=5, p1=5, T_stop=256.0):
    """The 2-D irregular benchmark tank (n1 = 1025, M = 5)."""
    clock, rnum = 32.0, 13
    harmo = np.arange(128, 640)
    f = harmo * clock / 2 ** rnum
    df = clock / 2 ** rnum
    S = jonswap_density(f, 0.10, 1.4, 3.3)
    S *= (0.10 / (4.0 * math.sqrt(np.sum(S * df)))) ** 2
    amp = np.sqrt(2.0 * S * df)
    phase = np.random.Generator(np.random.PCG64(seed)).uniform(0.0, 2 * np.pi, harmo.size)
    name = "J010_14"
    write_wave_files(directory, name, harmo, clock, rnum, amp, np.zeros(harmo.size), phase,
                     5.0, 30.0, 2.0, 0.5, 3.0)
    inp = base_input(icase=3, file_name=name, T_stop=T_stop, toler=1e-7, f_out=10.0, Hs=0.10, Tp=1.4)
    probes = [(x, 0.0) for x in (5.0, 10.0, 15.0, 20.0, 30.0)]
    return dict(inp=inp, n1=n1, n2=1, n3=n3, mHOS=mHOS, p1=p1, p2=1, probes=probes, wave_dir=directory,
                Hs=0.10, name="irregular_2d")


def regular_2d(n1=257, n3=33, mHOS=3, p1=3, T_stop=30.0):
    inp = base_input(icase=2, amp_mono=0.025, nu_mono=1.0, T_stop=T_stop, toler=1e-7, f_out=10.0)
    return dict(inp=inp, n1=n1, n2=1, n3=n3, mHOS=mHOS, p1=p1, p2=1,
                probes=[(5.0, 0.0), (10.0, 0.0), (20.0, 0.0)], wave_dir=".", Hs=0.05, name="regular_2d")


def directional_3d(directory, seed=2025, n1=513, n2=257, n3=33, mHOS=5, p1=4, p2=4, T_stop=120.0):
    """3-D directional JONSWAP: one direction per frequency bin drawn from a
    cos^2s(theta/2) spreading (s = 10) by inverse CDF."""
    clock, rnum = 32.0, 12
    harmo = np.arange(int(0.4 * 2 ** rnum / clock), int(2.5 * 2 ** rnum / clock) + 1)
    f = harmo * clock / 2 ** rnum
    df = clock / 2 ** rnum
    S = jonswap_density(f, 0.08, 1.2, 3.3)
    S *= (0.08 / (4.0 * math.sqrt(np.sum(S * df)))) ** 2
    amp = np.sqrt(2.0 * S * df)
    rng = np.random.Generator(np.random.PCG64(seed))
    th = np.linspace(-np.pi, np.pi, 4001)
    cdf = np.cumsum(np.cos(th / 2.0) ** 20)
    cdf /= cdf[-1]
    angle = np.degrees(np.interp(rng.uniform(size=harmo.size), cdf, th))
    phase = rng.uniform(0.0, 2 * np.pi, harmo.size)
    name = "D008_12"
    write_wave_files(directory, name, harmo, clock, rnum, amp, angle, phase, 5.0, 30.0, 2.0, 0.4, 2.5)
    inp = base_input(icase=3, file_name=name, T_stop=T_stop, toler=1e-7, f_out=10.0, Hs=0.08, Tp=1.2)
    probes = [(5.0, 15.0), (10.0, 15.0), (20.0, 15.0), (20.0, 7.5), (30.0, 15.0)]
    return dict(inp=inp, n1=n1, n2=n2, n3=n3, mHOS=mHOS, p1=p1, p2=p2, probes=probes, wave_dir=directory,
                Hs=0.08, name="directional_3d")


def steep_3d(directory, seed=200, n1=1025, n2=513, n3=33, mHOS=7, p1=7, p2=7, T_stop=100.0):
    """The steep 3-D tank of the surrogate study, run on the plain FP64 path:
    50 x 30 m, h = 5 m, snake flap, JONSWAP Hs = 0.15 m, Tp = 1.3 s,
    gamma = 5, cos^2s spreading with s = 15 drawn per frequency bin (0.4 to
    2.5 Hz, bins of 1/128 Hz), phases U[0, 2 pi) from PCG64(seed);
    n1 = 1025, n2 = 513, n3 = 33, M = 7, p1 = p2 = 7 (dealiased grid
    4100 x 2052)."""
    clock, rnum = 32.0, 12
    harmo = np.arange(int(0.4 * 2 ** rnum / clock), int(2.5 * 2 ** rnum / clock) + 1)
    f = harmo * clock / 2 ** rnum
    df = clock / 2 ** rnum
    S = jonswap_density(f, 0.15, 1.3, 5.0)
    S *= (0.15 / (4.0 * math.sqrt(np.sum(S * df)))) ** 2
    amp = np.sqrt(2.0 * S * df)
    rng = np.random.Generator(np.random.PCG64(seed))
    th = np.linspace(-np.pi, np.pi, 4001)
    cdf = np.cumsum(np.cos(th / 2.0) ** 30)
    cdf /= cdf[-1]
    angle = np.degrees(np.interp(rng.uniform(size=harmo.size), cdf, th))
    phase = rng.uniform(0.0, 2 * np.pi, harmo.size)
    name = "S015_13"
    write_wave_files(directory, name, harmo, clock, rnum, amp, angle, phase, 5.0, 30.0, 2.0, 0.4, 2.5)
    inp = base_input(icase=3, file_name=name, T_stop=T_stop, toler=1e-7, f_out=10.0, Hs=0.15, Tp=1.3,
                     gamma=5.0)
    probes = [(5.0, 15.0), (10.0, 15.0), (20.0, 15.0), (20.0, 7.5), (30.0, 15.0)]
    return dict(inp=inp, n1=n1, n2=n2, n3=n3, mHOS=mHOS, p1=p1, p2=p2, probes=probes, wave_dir=directory,
                Hs=0.15, name="steep_3d")


def ensemble(n_tanks=64, seed=7, T_stop=60.0, n3=33):
    """64 independent 2-D JONSWAP tanks of uneven size and order: n1 from
    {129, 257, 513, 1025, 2049}, M from {3, 5, 7} with p1 = M, Hs from
    U[0.04, 0.12] m, Tp from U[1.0, 2.0] s, gamma = 3.3, phases from the
    reference's SRAND/RAND with seed 1000 + k; all draws from PCG64(seed)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n_tanks):
        n1 = int(rng.choice([129, 257, 513, 1025, 2049]))
        M = int(rng.choice([3, 5, 7]))
        Hs = float(rng.uniform(0.04, 0.12))
        Tp = float(rng.uniform(1.0, 2.0))
        inp = base_input(icase=4, Hs=Hs, Tp=Tp, gamma=3.3, iseed=1000 + k, T_stop=T_stop, toler=1e-7,
                         f_out=10.0)
        out.append(dict(inp=inp, n1=n1, n2=1, n3=n3, mHOS=M, p1=M, p2=1, probes=[(10.0, 0.0)],
                        wave_dir=".", Hs=Hs, name=f"tank{k}"))
    return out
