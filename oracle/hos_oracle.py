"""CPU oracle for the HOS-NWT hot path -- TEST INFRASTRUCTURE ONLY.

This module is a plain numpy/scipy restatement of the reference HOS-NWT
solver (LHEEA, Fortran 90).  It exists only so that tests, the smoke check
and the CPU-baseline leg of the benchmark can check the CUDA product against
an independent implementation.  Nothing in the product imports it.

Parity status
-------------
The reference cannot be compiled here (it needs gfortran + FFTW3), so this
oracle is pinned by:
  * FFTW's published r2r definitions (REDFT00/RODFT00/REDFT01/REDFT10/
    RODFT01/RODFT10): scipy.fft dct/dst types 1-3 with norm=None use the same
    unnormalised conventions; tests check both against explicit sums;
  * libgfortran's SRAND/RAND (the reference's random phases for icase=4),
    called directly through ctypes from the libgfortran that scipy bundles;
  * analytic known answers the reference's own physics must reproduce: the
    linear sloshing standing wave (icase=1) and the linear wavemaker
    transfer function (TF_adim_new) far-field amplitude, plus volume
    conservation.
Bit-level parity with an FFTW build of the reference is *unpinned*: no FFTW
golden dump exists in the reference tree and none can be produced here.

Conventions: arrays are indexed [i1-1, i2-1] (x first), matching the
Fortran (i1, i2) indices of the reference.  Everything is float64.
"""
from __future__ import annotations

import ctypes
import glob
import math
import os

import numpy as np
from scipy import fft as sfft

# type.f90:44-50 constants
PI = 3.141592653589793238462643383279502888419
G = 9.81
TWOPI = 6.283185307179586476925286766559005768394
TINY = float(np.finfo(np.float64).eps)  # epsilon(1.0_rp)


# ----------------------------------------------------------------------------
# Input file (input.f90:62-201)
# ----------------------------------------------------------------------------
_INPUT_ORDER = [
    None, ("xlen", float), ("ylen", float), ("h", float),
    None, ("icase", int),
    None, ("islosh", int), ("aslosh", float),
    None, ("amp_mono", float), ("nu_mono", float), ("theta_mono", float),
    ("ph_mono", float), ("ibat", int), ("xd_mono", float),
    None, ("file_name", str), ("i_cut", int), ("nuc_low", float), ("nuc_high", float),
    None, ("Hs", float), ("Tp", float), ("gamma", float), ("iseed", int),
    None, ("i_wmk", int), ("igeom", int), ("d_hinge", float), ("iramp", int), ("Tramp", float),
    None, ("iabsnb", int), ("xabsf", float), ("coeffabsf", float),
    None, ("iprobes", int), ("pro_file", str),
    None, ("T_stop", float), ("toler", float), ("f_out", float),
    None, ("idim", int), ("i3d", int), ("imodes", int), ("iwmk", int), ("i_sw", int),
]


def _parse_value(txt, typ):
    if typ is str:
        return txt.strip()
    t = txt.strip().replace("d", "e").replace("D", "e")
    if typ is int:
        return int(float(t)) if t else 0
    return float(t)


def read_input(path):
    """read_input (input.f90:62-201): 52-character description, then value."""
    with open(path) as f:
        lines = f.read().splitlines()
    out = {}
    for line, item in zip(lines, _INPUT_ORDER):
        if item is None:
            continue
        name, typ = item
        out[name] = _parse_value(line[52:], typ)
    return out


def default_input(**kw):
    """A complete input dictionary (values of Benchmark/Regular style tanks)."""
    d = dict(xlen=50.0, ylen=30.0, h=5.0, icase=2, islosh=3, aslosh=0.02,
             amp_mono=0.025, nu_mono=1.0, theta_mono=0.0, ph_mono=0.0, ibat=2,
             xd_mono=18.0, file_name="", i_cut=0, nuc_low=0.3, nuc_high=3.0,
             Hs=0.05, Tp=1.0, gamma=3.3, iseed=513, i_wmk=1, igeom=2,
             d_hinge=2.0, iramp=1, Tramp=3.0, iabsnb=1, xabsf=0.8,
             coeffabsf=1.0, iprobes=1, pro_file="prob.inp", T_stop=30.0,
             toler=1e-7, f_out=10.0, idim=1, i3d=0, imodes=0, iwmk=0, i_sw=0)
    d.update(kw)
    return d


# ----------------------------------------------------------------------------
# libgfortran SRAND/RAND (initial_condition.f90:246,253)
# ----------------------------------------------------------------------------
def gfortran_rand_sequence(seed, n):
    """n successive REAL(4) values of RAND() after SRAND(seed), from the real
    libgfortran (the one scipy bundles)."""
    import scipy
    base = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
    libs = sorted(glob.glob(os.path.join(base, "libgfortran*")))
    if not libs:
        raise RuntimeError("libgfortran not found")
    lib = ctypes.CDLL(libs[0])
    lib._gfortran_srand.argtypes = [ctypes.POINTER(ctypes.c_int)]
    lib._gfortran_rand.argtypes = [ctypes.POINTER(ctypes.c_int)]
    lib._gfortran_rand.restype = ctypes.c_float
    s = ctypes.c_int(int(seed))
    lib._gfortran_srand(ctypes.byref(s))
    z = ctypes.c_int(0)
    return np.array([lib._gfortran_rand(ctypes.byref(z)) for _ in range(n)],
                    dtype=np.float32)


# ----------------------------------------------------------------------------
# Linear wave helpers (linear_wave.f90)
# ----------------------------------------------------------------------------
def _xthx(x):
    return x * math.tanh(x)


def dichoto(func, f0, a, b, prec):
    """dichoto (linear_wave.f90:427-466), same bisection and exit rule."""
    fa = func(a) - f0
    if fa * (func(b) - f0) >= 0.0:
        if abs(func(a) - f0) < TINY:
            return a
        if abs(func(b) - f0) < TINY:
            return b
    x1, x2 = a, b
    x3 = 0.0
    while abs(x1 - x2) > prec * abs(x2):
        x3 = (x1 + x2) / 2.0
        f3 = func(x3) - f0
        if abs(f3) < TINY:
            return x3
        if fa * f3 < 0.0:
            x2 = x3
        else:
            x1 = x3
    return x3


def wave_number_adim_r(f, prec):
    """linear_wave.f90:137-151."""
    w2 = (TWOPI * f) ** 2
    if w2 < math.log(np.finfo(np.float64).max) - 1.0:
        return dichoto(_xthx, w2, 0.0, 1.0e6, prec)
    return w2


def ocean_txt2cfg_dat(path, i_cut, nuc_low, nuc_high, icase):
    """ocean_txt2cfg_dat (read_ocean_txt.f90:33-228) for the ECN wave basin
    (icase 31) and towing tank (32): the fronts of an Edinburgh Designs .txt
    file as the lines of the .cfg and .dat files it writes (the .dat values
    pass through G20.7, i.e. 7 significant digits)."""
    with open(path, encoding="latin-1") as f:
        lines = f.read().splitlines()
    rnum = ramp = rcomp = n_front = n_start = None
    for i, t in enumerate(lines):
        if "rnumber  =" in t:
            rnum = int(t.split("=")[1].split()[0])
        if "ramp     =" in t:
            ramp = int(t.split("=")[1].split()[0])
        if "rnumber compression" in t:
            rcomp = int(t.split("=")[-1].split()[0])
        if "Wave has " in t:
            n_front = int(t.split("Wave has ")[1].split()[0])
            n_start = i + 2
    vals = np.array([[float(v) for v in lines[n_start + j].split()[:5]] for j in range(n_front)])
    harmo = vals[:, 0].astype(np.int64)
    ampli, angle, phase = vals[:, 2].copy(), vals[:, 3].copy(), vals[:, 4].copy()
    if rcomp is not None:
        harmo = harmo * rcomp
    clock = 32.0
    freq = harmo * (clock / 2 ** rnum)
    if icase == 31:
        for i in range(n_front):
            k = wave_number_r(freq[i], 5.0, 1.0e-12)
            phase[i] = phase[i] + k * 29.74 / 2.0 * math.sin(angle[i])
    angle = 180.0 * angle / PI
    f_lo, f_hi = (nuc_low, nuc_high) if i_cut == 1 else (0.0, 100.0)
    if icase == 31:
        cfg = [f"{rnum:2d}", f"{clock:5.2f}", f"{5.0:5.2f}", f"{ramp:4d}", "lin", f"{f_lo:5.2f}",
               f"{f_hi:6.2f}", f"{30.0:5.2f}", "hinged", f"{2.147:6.3f}"]
    else:
        cfg = [f"{rnum:2d}", f"{clock:5.2f}", f"{2.88:5.2f}", f"{ramp:4d}", "lin", f"{f_lo:5.2f}",
               f"{f_hi:6.2f}", f"{5.0:5.2f}", "hinged", f"{0.0:6.3f}"]
    ampli[ampli < 1.0e-98] = 0.0
    g7 = lambda v: f"{float(v):.6E}"
    dat = [f"{int(harmo[i]):5d} {g7(freq[i])} {g7(ampli[i])} {g7(angle[i])} {g7(phase[i])}"
           for i in range(n_front) if f_lo <= freq[i] <= f_hi]
    return cfg, dat


def wave_number_r(f, h, prec):
    """linear_wave.f90:120-134 (dimensional)."""
    w2h = (TWOPI * f) ** 2 / G * h
    if w2h < math.log(np.finfo(np.float64).max) - 1.0:
        return dichoto(_xthx, (TWOPI * f) ** 2 * h / G, 0.0, 10000000.0, prec) / h
    return (TWOPI * f) ** 2 / G


def TF_adim_new(typ, k, hinge):
    """TF_adim_new (linear_wave.f90:277-334), hinged/piston branches."""
    typ = typ.strip()
    if typ in ("hinged", "monofl"):
        d = hinge
        if k < 50 and k * d < 50:
            resu = -1j * k * (1.0 - d) * (2.0 * k + math.sinh(2.0 * k)) / (4.0 * math.sinh(k))
            resu = resu / (k * (1.0 - d) * math.sinh(k) + math.cosh(k * d) - math.cosh(k))
        elif k >= 50 and k * d < 50:
            resu = -1j * k * (1.0 - d) / (2.0 * k * (1.0 - d) - 2.0 + 4.0 * math.cosh(k * d) * math.exp(-k))
        else:
            if k * (1.0 - d) >= 20:
                resu = -0.5j
            else:
                resu = -1j * k * (1.0 - d) / (2.0 * k * (1.0 - d) - 2.0 + 2.0 * math.exp(k * (d - 1.0)))
    elif typ == "piston":
        if k < 50.0:
            resu = complex(0.0, -(2.0 * k + math.sinh(2.0 * k)) / (4.0 * math.sinh(k) * math.sinh(k)))
        else:
            resu = complex(0.0, -0.5)
    else:
        resu = complex(1.0, 0.0)
    return complex(resu)


# ----------------------------------------------------------------------------
# r2r transforms with FFTW conventions (fourier_FFTW.f90:89-653)
# ----------------------------------------------------------------------------
# Threads of the scipy transforms (1: single-threaded, like the Fortran
# reference).  The benchmark's CPU arm raises it to the host's core count.
_WORKERS = 1


def set_workers(n):
    """Threads used by every scipy.fft call of the oracle."""
    global _WORKERS
    _WORKERS = max(1, int(n))


def _r2r(a, axis, kind):
    """Unnormalised FFTW r2r along `axis`.  kind: REDFT00, RODFT00, REDFT01,
    REDFT10, RODFT01, RODFT10.  scipy's norm=None types match FFTW exactly."""
    w = _WORKERS
    if kind == "REDFT00":
        return sfft.dct(a, type=1, axis=axis, workers=w)
    if kind == "RODFT00":
        return sfft.dst(a, type=1, axis=axis, workers=w)
    if kind == "REDFT10":
        return sfft.dct(a, type=2, axis=axis, workers=w)
    if kind == "REDFT01":
        return sfft.dct(a, type=3, axis=axis, workers=w)
    if kind == "RODFT10":
        return sfft.dst(a, type=2, axis=axis, workers=w)
    if kind == "RODFT01":
        return sfft.dst(a, type=3, axis=axis, workers=w)
    raise ValueError(kind)


def _ends_interior(n, end, interior):
    v = np.full(n, interior, dtype=np.float64)
    v[0] = end
    v[-1] = end
    return v


class Fourier:
    """Fourier_ini + DCT_FFTW/IDCT_FFTW/_big/_add (fourier_FFTW.f90:89-653)."""

    def __init__(self, n1, n2, nd1, nd2, n3_add):
        self.n1, self.n2, self.nd1, self.nd2, self.n3_add = n1, n2, nd1, nd2, n3_add
        # fourier_FFTW.f90:175-229 normalisation tables (separable)
        self.s2f = self._s2f(n1, n2)
        self.f2s = self._f2s(n1, n2)
        self.s2f_big = self._s2f(nd1, nd2)
        self.f2s_big = self._f2s(nd1, nd2)
        s = np.full((n3_add, n2), 1.0 / n3_add)
        f = np.full((n3_add, n2), 0.5)
        if n2 != 1:
            s = s / max(1, 2 * (n2 - 1))
            s[:, 1:n2 - 1] *= 2.0
            f[:, 1:n2 - 1] *= 0.5
        self.s2f_add, self.f2s_add = s, f

    def _s2f(self, a, b):
        s = np.full((a, b), 1.0 / max(1, 2 * (a - 1)))
        s[1:a - 1, :] *= 2.0
        if self.n2 != 1:
            s = s / max(1, 2 * (b - 1))
            s[:, 1:b - 1] *= 2.0
        return s

    def _f2s(self, a, b):
        f = np.ones((a, b))
        f[1:a - 1, :] *= 0.5
        if self.n2 != 1:
            f[:, 1:b - 1] *= 0.5
        return f

    def _execute(self, inp, csx, csy, yn):
        """execute / execute_big (fourier_FFTW.f90:271-302, 616-653)."""
        inp = np.array(inp, dtype=np.float64, copy=True)
        nx = inp.shape[0]
        if self.n2 != 1 and csy == "sin":
            inp[:, 0] = 0.0
            inp[:, yn - 1] = 0.0
        out = np.zeros_like(inp)
        # x-direction
        if csx == "cos":
            tmp = _r2r(inp, 0, "REDFT00")
        elif csx == "sin":
            tmp = np.zeros_like(inp)
            tmp[1:nx - 1, :] = _r2r(inp[1:nx - 1, :], 0, "RODFT00")
        else:
            raise ValueError(csx)
        # y-direction (2D plans only)
        if self.n2 != 1:
            if csy == "cos":
                out = _r2r(tmp, 1, "REDFT00")
            elif csy == "sin":
                out[:, 1:yn - 1] = _r2r(tmp[:, 1:yn - 1], 1, "RODFT00")
            else:
                raise ValueError(csy)
        else:
            out = tmp
        if csx == "sin":
            out[0, :] = 0.0
            out[nx - 1, :] = 0.0
        if self.n2 != 1 and csy == "sin":
            out[:, 0] = 0.0
            out[:, yn - 1] = 0.0
        return out

    # small grid
    def S2F(self, f, csx="cos", csy="cos"):
        return self._execute(f, csx, csy, self.n2) * self.s2f

    def F2S(self, f, csx="cos", csy="cos"):
        return self._execute(f * self.f2s, csx, csy, self.n2)

    # big (dealiased) grid
    def S2F_big(self, f, csx="cos", csy="cos"):
        return self._execute(f, csx, csy, self.nd2) * self.s2f_big

    def F2S_big(self, f, csx="cos", csy="cos"):
        return self._execute(f * self.f2s_big, csx, csy, self.nd2)

    # wavemaker grid (fourier_FFTW.f90:432-548)
    def _execute_add(self, inp, csz, csy, fb):
        inp = np.array(inp, dtype=np.float64, copy=True)
        n2 = self.n2
        if n2 != 1 and csy == "sin":
            inp[:, 0] = 0.0
            inp[:, n2 - 1] = 0.0
        if fb == 1:
            kz = "REDFT01" if csz == "cos" else "RODFT01"
        else:
            kz = "REDFT10" if csz == "cos" else "RODFT10"
        tmp = _r2r(inp, 0, kz)
        if n2 != 1:
            if csy == "cos":
                out = _r2r(tmp, 1, "REDFT00")
            else:
                out = np.zeros_like(tmp)
                out[:, 1:n2 - 1] = _r2r(tmp[:, 1:n2 - 1], 1, "RODFT00")
                out[:, 0] = 0.0
                out[:, n2 - 1] = 0.0
        else:
            out = tmp
        return out

    def F2S_y(self, f, csy="cos"):
        """FOURIER_2_SPACE_y (fourier_FFTW.f90:340-428) along axis 1; the
        identity when n2 = 1."""
        f = np.array(f, dtype=np.float64, copy=True)
        n2 = self.n2
        if n2 == 1:
            return f
        fy = np.ones(n2)
        fy[1:n2 - 1] = 0.5
        inp = f * fy[None, :]
        if csy == "cos":
            return _r2r(inp, 1, "REDFT00")
        out = np.zeros_like(inp)
        out[:, 1:n2 - 1] = _r2r(inp[:, 1:n2 - 1], 1, "RODFT00")
        return out

    def S2F_add(self, f, csz="cos", csy="cos"):
        return self._execute_add(f, csz, csy, 1) * self.s2f_add

    def F2S_add(self, f, csz="cos", csy="cos"):
        return self._execute_add(f * self.f2s_add, csz, csy, -1)


# ----------------------------------------------------------------------------
# The tank
# ----------------------------------------------------------------------------
class Tank:
    """HOS-NWT state, tables and hot path (plain FP64, numpy)."""

    def __init__(self, inp, n1, n2, n3, mHOS, p1, p2=1, probes=None,
                 wave_files_dir=".", count_transforms=False):
        self.inp = dict(inp)
        self.n1, self.n2, self.n3, self.M = int(n1), int(n2), int(n3), int(mHOS)
        self.p1, self.p2 = int(p1), int(p2)
        # common_vars.f90:40-48
        self.nd1 = ((self.p1 + 1) * self.n1) // 2
        self.nd2 = ((self.p2 + 1) * self.n2) // 2
        self.l_add = 2
        self.n3_add = self.l_add * (self.n3 - 1)
        self.fourier = Fourier(self.n1, self.n2, self.nd1, self.nd2, self.n3_add)
        self.ntrans = 0
        self._count = count_transforms
        self.wave_files_dir = wave_files_dir
        self.probes_xy = probes
        self._check()
        self._nondim()
        self._dt_choice()
        self._mesh()
        self._wave_cfg()
        self._absorb()
        self._tables()
        self._initialize()

    # ------------------------------------------------------------------ checks
    def _check(self):
        # check_range (initial_condition.f90:584-605)
        ok = (1, 2, 3, 4, 5, 7, 8, 9, 11, 14, 15, 17, 19, 23, 29)
        for v, name in ((self.M, "M"), (self.p1, "p1"), (self.p2, "p2")):
            if v not in ok:
                raise ValueError(f"forbidden value of {name}: {v}")
        if self.p1 > self.M or self.p2 > self.M:
            raise ValueError("p1/p2 higher than M")
        if self.inp["i_wmk"] not in (1, 2, 3) and self.inp["icase"] != 1:
            raise NotImplementedError("wavemaker orders i_wmk = 1, 2, 3 only")

    # ------------------------------------------------------------------ setup
    def _nondim(self):
        """HOS-NWT.f90:99-119."""
        p = self.inp
        self.h = p["h"]
        self.Tscale = 1.0 / math.sqrt(G / self.h)
        h = self.h
        self.xlen = p["xlen"] / h
        self.ylen = p["ylen"] / h
        self.amp_mono = p["amp_mono"] / h
        self.xd_mono = p["xd_mono"] / self.h
        self.xlen_add = 2.0 * float(self.l_add)
        self.d_hinge = p["d_hinge"] / h
        self.aslosh = p["aslosh"] / h
        self.Tramp = p["Tramp"] / self.Tscale
        if p["iramp"] == 0:  # input.f90:170-172
            self.Tramp = 0.0
        self.T_stop = p["T_stop"] / self.Tscale
        self.f_out = p["f_out"] * self.Tscale
        self.nu_mono = p["nu_mono"] * self.Tscale
        self.w_mono = self.nu_mono * TWOPI
        self.T_mono = 1.0 / self.nu_mono
        theta = p["theta_mono"] if self.n2 != 1 else 0.0
        self.theta_mono = theta * PI / 180.0
        self.ph_mono = p["ph_mono"]
        self.islosh = p["islosh"] + 1  # input.f90:165
        self.icase, self.igeom, self.iramp = p["icase"], p["igeom"], p["iramp"]
        self.iabsnb, self.toler = p["iabsnb"], p["toler"]

    def _dt_choice(self):
        """HOS-NWT.f90:130-217."""
        n1, n2, n3, l_add = self.n1, self.n2, self.n3, self.l_add
        xlen, ylen = self.xlen, self.ylen
        dtc = [0.0, 0.0, 0.0]
        dtr = [0.0, 0.0, 0.0]
        k_m = PI / xlen
        dtc[0] = math.sqrt(k_m * xlen ** 2 / math.tanh(k_m)) / float(n1 - 1)
        dtr[0] = math.sqrt(8 / PI ** 2) * xlen / float(n1 - 1)
        if n2 != 1:
            k_m = PI / ylen
            dtc[1] = math.sqrt(k_m * ylen ** 2 / math.tanh(k_m)) / float(n2 - 1)
            dtr[1] = math.sqrt(8 / PI ** 2) * ylen / float(n2 - 1)
        else:
            dtc[1] = dtc[0] + 1.0
            dtr[1] = dtr[0] + 1.0
        if self.igeom != 3:
            k_m = PI / (2.0 * float(l_add))
            dtc[2] = math.sqrt(k_m * (2.0 * float(l_add)) ** 2 / math.tanh(k_m)) / float(float(l_add) * (n3 - 1))
            dtr[2] = math.sqrt(8 / PI ** 2) * (2.0 * float(l_add)) / float(l_add * (n3 - 1))
        else:
            dtc[2] = dtc[0] + 1.0
            dtr[2] = dtr[0] + 1.0
        if self.igeom == 3 or self.icase == 1:
            dt_stab = dtr[0] if n2 == 1 else min(dtr[0], dtr[1])
        elif n2 == 1:
            dt_stab = min(dtr[0], dtr[2])
        else:
            dt_stab = min(dtr)
        self.dt_stab = dt_stab
        self.delt_out = 1.0 / self.f_out
        self.delt = min(0.95 * dt_stab, self.delt_out)
        if abs(self.delt - self.delt_out) < TINY:
            raise ValueError("DECREASE f_out")

    def _mesh(self):
        """HOS-NWT.f90:220-244."""
        n1, n2, n3 = self.n1, self.n2, self.n3
        self.delx = self.xlen / (n1 - 1)
        self.delz = 1.0 / (n3 - 1)
        self.dely = self.ylen / (n2 - 1) if n2 != 1 else 0.0
        self.cy = np.arange(n2) * self.dely
        self.cx = np.arange(n1) * self.delx
        self.cx_add = self.delz * np.arange(n3)
        self.cz = self.cx_add - 1.0

    # ---------------------------------------------------------- wave synthesis
    def _wave_init(self, typ_wmk, hinge, freq):
        """wave_init (wave_def.f90:282-329)."""
        k = np.zeros(len(freq))
        TF = np.zeros(len(freq), dtype=np.complex128)
        for i, f in enumerate(freq):
            kt = wave_number_adim_r(f, 1.0e-15)
            k[i] = kt
            TF[i] = TF_adim_new(typ_wmk, kt, hinge) if abs(kt) > TINY else 1.0
        small = freq < 1.0e-8
        k[small] = 0.0
        TF[small] = 1.0
        return k, TF

    def _wave_cfg(self):
        """initialize_wav_cfg (initial_condition.f90:128-310) + wmk_ini."""
        p, h = self.inp, self.h
        typ = "hinged" if self.igeom == 2 else "piston"
        if self.icase == 1:
            self.wave = None
            self.freq_w = np.zeros(0)
            self.pos_ini = np.zeros((self.n2, 0), dtype=np.complex128)
            self.pos_gzed = np.array([self._gzed(z) for z in self.cz])
            return
        if self.icase == 2:
            rnum, clock = 1, 2.0 * self.nu_mono
            harmo = np.array([1])
            if p["ibat"] not in (2, 3):
                raise NotImplementedError("snake (ibat=2) or Dalrymple (ibat=3) wavemaking only")
            if p["ibat"] == 3:
                harmo, freq, ampli, angle, phase = self._dalrymple(
                    clock, rnum, 1, self.amp_mono, self.theta_mono, self.ph_mono)
            else:
                freq = np.array([1 * clock / 2 ** rnum])
                ampli = np.array([self.amp_mono])
                angle = np.array([self.theta_mono])
                phase = np.array([self.ph_mono])
            depth, hinge = h, self.d_hinge
        elif self.icase in (3, 31, 32):
            base = os.path.join(self.wave_files_dir, p["file_name"].strip())
            if self.icase == 3:
                with open(base + ".cfg") as f:
                    cl = [ln.strip() for ln in f.read().splitlines()]
                with open(base + ".dat") as f:
                    dat_lines = f.read().splitlines()
            else:
                cl, dat_lines = ocean_txt2cfg_dat(base + ".txt", p["i_cut"], p["nuc_low"], p["nuc_high"],
                                                  self.icase)
            rnum = int(cl[0].split()[0])
            clock_d = float(cl[1].split()[0].replace("d", "e"))
            depth = float(cl[2].split()[0].replace("d", "e"))
            cut_lo = float(cl[5].split()[0].replace("d", "e"))
            cut_hi = float(cl[6].split()[0].replace("d", "e"))
            typ = cl[8].split()[0]
            hinge_d = float(cl[9].split()[0].replace("d", "e"))
            Ts = math.sqrt(depth / G)
            clock = clock_d * Ts
            cut_lo_n, cut_hi_n = cut_lo * Ts, cut_hi * Ts
            hinge = hinge_d / depth
            rows = [ln.replace(",", " ").split() for ln in dat_lines if ln.strip()]
            harmo_a = np.array([int(r[0]) for r in rows])
            freq_a = np.array([float(r[1]) for r in rows])
            amp_a = np.array([float(r[2]) for r in rows])
            ang_a = np.array([float(r[3]) for r in rows])
            ph_a = np.array([float(r[4]) for r in rows])
            n_start, n_stop = 1, 0
            for i in range(len(rows)):  # wave_def.f90:240-248
                if freq_a[i] <= cut_hi_n / Ts:
                    n_stop = i + 1
                if freq_a[i] < cut_lo_n / Ts:
                    n_start += 1
            if n_stop - n_start + 1 <= 0:
                raise ValueError("n_good == 0")
            sl = slice(n_start - 1, n_stop)
            harmo = harmo_a[sl]
            freq = freq_a[sl] * Ts
            ampli = amp_a[sl] / depth
            angle = ang_a[sl] * PI / 180.0
            phase = ph_a[sl]
            if p["ibat"] == 3 and self.n2 != 1:
                # initial_condition.f90:192-199: the Dalrymple waves of every
                # component, concatenated (add_wave, wave_def.f90:333-384)
                parts = [self._dalrymple(clock, rnum, int(hh), a, an, ph)
                         for hh, a, an, ph in zip(harmo, ampli, angle, phase)]
                harmo = np.concatenate([q[0] for q in parts])
                freq = np.concatenate([q[1] for q in parts])
                ampli = np.concatenate([q[2] for q in parts])
                angle = np.concatenate([q[3] for q in parts])
                phase = np.concatenate([q[4] for q in parts])
        elif self.icase == 4:
            Tp, Hs, gam = p["Tp"], p["Hs"], p["gamma"]
            clock = 32.0
            rnum = int(math.ceil(math.log10(self.T_stop * self.Tscale * clock) / math.log10(2.0)))
            depth = h
            n_pts = int(round(2 * 2 ** rnum / clock + 1))
            f_base = float(clock) / 2.0 ** rnum
            rnd = gfortran_rand_sequence(p["iseed"], n_pts)
            harmo = np.arange(n_pts)
            freq = np.zeros(n_pts)
            ampli = np.zeros(n_pts)
            phase = np.zeros(n_pts)
            Hs_int = 0.0
            for i1 in range(1, n_pts + 1):
                fr = i1 * f_base
                freq[i1 - 1] = fr
                phase[i1 - 1] = TWOPI * float(rnd[i1 - 1])
                sigma = float(np.float32(0.07)) if fr < 1.0 / Tp else float(np.float32(0.09))
                a = (1.0 / (TWOPI ** 4) * G ** 2 / fr ** 5 * math.exp(-5.0 / 4.0 * (fr * Tp) ** (-4))
                     * gam ** (math.exp((-(fr - 1.0 / Tp) ** 2) / (2.0 * (sigma / Tp) ** 2))) * f_base)
                Hs_int += a
                ampli[i1 - 1] = math.sqrt(2.0 * a)
            Hs_int = 4.0 * math.sqrt(Hs_int)
            ampli = ampli * Hs / Hs_int
            freq = freq * self.Tscale
            ampli = ampli / h
            angle = np.zeros(n_pts)
            clock = clock * self.Tscale
            hinge = self.d_hinge
        else:
            raise NotImplementedError(f"icase={self.icase}")
        k, TF = self._wave_init(typ, hinge, freq)
        self.wave = dict(harmo=harmo, freq=freq, ampli=ampli, angle=angle, phase=phase,
                         k=k, TF=TF, rnum=rnum, clock=clock, depth=depth)
        self._wmk_ini()

    @staticmethod
    def _phase(z):
        """phase (wave_def.f90:491-523) as written: its first test returns 0
        for every |z| > tiny, so only |z| <= tiny reaches the angle formula."""
        if abs(z) > TINY:
            return 0.0
        with np.errstate(invalid="ignore", divide="ignore"):
            zt = z / abs(z)
            pt = math.asin(zt.imag) if abs(zt.imag) <= 1.0 else float("nan")
        if zt.real >= 0.0:
            return pt if zt.imag >= 0.0 else TWOPI + pt
        return PI - pt

    def _dalrymple(self, clock, rnum, harmo, ampli, angle, phas):
        """dalrymple (wave_def.f90:111-177): the oblique wave of one
        frequency as 2 (N+1) components over the tank's y-modes, focused at
        x = xd_mono."""
        Ly, X_d = self.ylen, self.xd_mono
        freq = harmo * clock / 2 ** rnum
        k = wave_number_adim_r(freq, 1.0e-12)
        N = int(math.floor(k * Ly / PI))
        mu = np.arange(N + 1) * PI / Ly
        theta = np.arcsin(mu / k)
        beta = k * math.sin(angle)
        delta = np.zeros(N + 1)
        delta[0] = 1.0
        if abs(angle) < TINY:
            I_n = delta.astype(np.complex128)
        else:
            I_n = np.zeros(N + 1, dtype=np.complex128)
            tmp = -np.exp(-1j * beta * Ly)
            for n in range(N + 1):
                tmp = -tmp
                if abs(mu[n] - abs(beta)) < TINY:
                    I_n[n] = 1.0
                else:
                    I_n[n] = 2 * 1j * beta * (tmp - 1) / (beta ** 2 - mu[n] ** 2) / ((1 + delta[n]) * Ly)
        k_n = 1j * np.sqrt(k ** 2 - mu ** 2 + 0j)
        a_on = ampli * np.exp(1j * phas) * I_n * np.exp((k_n - 1j * k * math.cos(angle)) * X_d)
        ph = np.array([self._phase(z) for z in a_on])
        amp = np.abs(a_on / 2.0)
        n_f = 2 * (N + 1)
        return (np.full(n_f, harmo), np.full(n_f, freq), np.concatenate([amp, amp]),
                np.concatenate([theta, -theta]), np.concatenate([ph, ph]))

    def _gzed(self, z):
        """gzed (wavemaking.f90:184-213)."""
        dh = self.d_hinge
        delta = min(dh, (1.0 - dh) / 10.0)
        if self.igeom == 1:
            return 1.0
        if z >= (dh - 1.0 + delta):
            return (z + 1.0 - dh) / (1.0 - dh)
        if z <= (dh - 1.0 - delta):
            return 0.0
        U = z - (dh - 1.0)
        return delta / (2.0 * (1.0 - dh)) * (5.0 / 16.0 + (U / delta) + 15.0 / 16.0 * (
            (U / delta) ** 2 - 1.0 / 3.0 * (U / delta) ** 4 + 1.0 / 15.0 * (U / delta) ** 6))

    def _dgzeddz(self, z):
        """dgzeddz (wavemaking.f90:222-250)."""
        dh = self.d_hinge
        delta = min(dh, (1.0 - dh) / 10.0)
        if self.igeom == 1:
            return 0.0
        if z >= (dh - 1.0 + delta):
            return 1.0 / (1.0 - dh)
        if z <= (dh - 1.0 - delta):
            return 0.0
        U = z - (dh - 1.0)
        return 1.0 / (1.0 - dh) * (1.0 / 2.0 + 15.0 / 16.0 * ((U / delta) - 2.0 / 3.0 * (U / delta) ** 3
                                                               + 1.0 / 5.0 * (U / delta) ** 5))

    def _wmk_ini(self):
        """wmk_ini (wavemaking.f90:37-175), full-width wavemaker (iwidth=1)."""
        w = self.wave
        n_max = max(1, int(math.floor(w["clock"] * math.sqrt(G / w["depth"]))))
        n_max = 2 ** w["rnum"] // n_max
        groups = []
        for harm in range(0, 4 * n_max + 1):
            idx = np.nonzero(w["harmo"] == harm)[0]
            if len(idx):
                groups.append(idx)
        pos_ini = np.zeros((self.n2, len(groups)), dtype=np.complex128)
        dposdy_ini = np.zeros((self.n2, len(groups)), dtype=np.complex128)
        freq = np.zeros(len(groups))
        for g_i, idx in enumerate(groups):
            freq[g_i] = w["freq"][idx[0]]
            for j1 in range(self.n2):
                acc = 0j
                for i in idx:
                    ang = w["angle"][i]
                    acc = acc + 1.0 * (w["TF"][i] * math.cos(ang) * w["ampli"][i] * np.exp(
                        1j * (-w["k"][i] * math.sin(ang) * self.cy[j1] + w["phase"][i])))
                pos_ini[j1, g_i] = acc
                # dposdy_ini, full-width wavemaker (rampy = 1, drampy = 0)
                dacc = 0j
                for i in idx:
                    ang = w["angle"][i]
                    pos_tmp = w["TF"][i] * math.cos(ang) * w["ampli"][i] * np.exp(
                        1j * (-w["k"][i] * math.sin(ang) * self.cy[j1] + w["phase"][i]))
                    dacc = dacc + (0.0 - 1j * w["k"][i] * math.sin(ang) * 1.0) * pos_tmp
                dposdy_ini[j1, g_i] = dacc
        self.pos_ini = pos_ini
        self.dposdy_ini = dposdy_ini
        self.freq_w = freq
        self.pos_gzed = np.array([self._gzed(z) for z in self.cz])
        self.dpos_gzed = np.array([self._dgzeddz(z) for z in self.cz])

    def _absorb(self):
        """absorb (initial_condition.f90:724-794), iwidth=1, no back beach."""
        n1, n2 = self.n1, self.n2
        self.nu = np.zeros((n1, n2))
        # dnux as written in absorb: coeffabsf * 2 * x3 (without 1 / x2)
        self.dnux = np.zeros((n1, n2))
        self.dnuy = np.zeros((n1, n2))
        if self.iabsnb == 0:
            return
        xabsf, coeff = self.inp["xabsf"], self.inp["coeffabsf"]
        x0 = self.xlen * xabsf
        if abs(xabsf - 1.0) > TINY:
            x2 = self.xlen - x0
            for i1 in range(n1):
                if self.cx[i1] >= x0:
                    x3 = (self.cx[i1] - x0) / x2
                    self.nu[i1, :] = coeff * x3 * x3
                    self.dnux[i1, :] = coeff * 2 * x3

    def _tables(self):
        """Spectral tables (HOS-NWT.f90:267-406)."""
        n1, n2, M = self.n1, self.n2, self.M
        pixlen = PI / self.xlen
        piylen = PI / self.ylen if n2 != 1 else 0.0
        self.ky = np.arange(n2) * piylen
        ky2 = self.ky * self.ky
        self.kx = np.arange(n1) * pixlen
        kx2 = self.kx * self.kx
        self.k = np.sqrt(kx2[:, None] + ky2[None, :])
        self.omega = np.sqrt(self.k * np.tanh(self.k))
        thk = np.tanh(self.k)
        kth = np.zeros((n1, n2, M))
        for j in range(1, M + 1):
            kth[:, :, j - 1] = self.k ** j * thk if j % 2 == 1 else self.k ** j
        self.kth = kth
        nd1, nd2 = self.nd1, self.nd2
        kxe = np.arange(nd1) * pixlen
        kye = np.arange(nd2) * piylen
        ke = np.sqrt(kxe[:, None] ** 2 + kye[None, :] ** 2)
        thke = np.tanh(ke)
        kth_ext = np.zeros((nd1, nd2, M))
        for j in range(1, M + 1):
            kth_ext[:, :, j - 1] = ke ** j * thke if j % 2 == 1 else ke ** j
        self.kth_ext = kth_ext
        # wavemaker modes
        n3_add = self.n3_add
        pixlen_add = PI / self.xlen_add
        self.kx_add = (2 * np.arange(1, n3_add + 1) - 1) * pixlen_add
        self.k_add = np.sqrt(self.kx_add[:, None] ** 2 + ky2[None, :])
        k_add_2 = 2.0 * self.k_add
        self.k_add_thk_add = self.k_add * np.tanh(self.k_add * self.xlen)
        # csh_add_x etc. (HOS-NWT.f90:361-404), with the 700 overflow guard
        XMAX = 700.0
        kx_ = k_add_2 * self.xlen
        expon3 = np.where(kx_ <= XMAX, np.exp(-np.minimum(kx_, XMAX)), 0.0)
        expon3p1 = expon3 + 1.0
        cx = self.cx[:, None, None]
        ka = self.k_add.T[None, :, :]       # (1, n2, n3_add)
        ka2 = k_add_2.T[None, :, :]
        x1 = ka * cx
        e1 = np.where(x1 <= XMAX, np.exp(-np.minimum(x1, XMAX)) / expon3p1.T[None, :, :], 0.0)
        x2 = ka2 * (self.xlen - cx)
        e2 = np.where(x2 <= XMAX, np.exp(-np.minimum(x2, XMAX)), 0.0)
        e12 = np.where(x1 + x2 <= XMAX, e1 * e2, 0.0)
        csh = e1 + e12
        sh = e1 - e12
        self.csh_add_x = csh                               # (n1, n2, n3_add)
        self.k_add_sh_add_x = sh * ka
        self.kycsh_add_x = csh * self.ky[None, :, None]
        self.kx_add_csh_add_x = csh * self.kx_add[None, None, :]
        # probes (initialize_probes_matrices, initial_condition.f90:486-501)
        if self.probes_xy is not None:
            P = np.asarray(self.probes_xy, dtype=np.float64).reshape(-1, 2) / self.h
            self.probe_pos = P
            self.mat_coscos = (np.cos(self.kx[:, None, None] * P[None, None, :, 0])
                               * np.cos(self.ky[None, :, None] * P[None, None, :, 1]))

    # --------------------------------------------------------- wavemaker law
        if self.inp["i_wmk"] >= 2:
            # free-surface modes on the wavemaker (HOS-NWT.f90:343-355)
            arg = self.k[:, :, None] * self.cx_add[None, None, :]
            csh0 = np.cosh(self.k)[:, :, None]
            cshx = np.cosh(arg) / csh0
            self.kx2cshx_add = cshx * kx2[:, None, None]
            self.kycshx_add = cshx * self.ky[None, :, None]
            self.kshx_add = self.k[:, :, None] * np.sinh(arg) / csh0

    def ramp(self, time):
        """ramp (resol_wmkr.f90:1268-1397)."""
        iramp, Tramp, T_stop = self.iramp, self.Tramp, self.T_stop
        if iramp == 11:
            T_swtt = 3.0 / math.sqrt(5.0 / 9.81)
            return (time / T_swtt, 1.0 / T_swtt, 0.0) if time <= T_swtt else (1.0, 0.0, 0.0)
        if iramp == 33:
            T_swtt = -math.log(0.1) / (10.0 * self.T_mono)
            a = 1.0 - math.exp(-T_swtt * time)
            return a, (1.0 - a) * T_swtt, (1.0 - a) * T_swtt * T_swtt
        if time <= Tramp:
            if iramp == 0:
                return 1.0, 0.0, 0.0
            if iramp == 1:
                return time / Tramp, 1.0 / Tramp, 0.0
            if iramp == 2:
                tmp = time / Tramp
                return tmp * tmp, 2.0 * tmp / Tramp, 2.0 / (Tramp * Tramp)
            if iramp == 21:
                T2, tim2, timsup = Tramp ** 2, time ** 2, time / Tramp - 1.0
                if time <= Tramp / 2.0:
                    return 2.0 * tim2 / T2, 4.0 * time / T2, 4.0 / T2
                return 1.0 - 2.0 * timsup ** 2, -4.0 * timsup / Tramp, -4.0 / T2
            if iramp == 4:
                tmp = time / Tramp
                tmp2 = tmp * tmp
                return tmp2 * tmp2, 4.0 * tmp2 * tmp / Tramp, 12.0 * tmp2 / (Tramp * Tramp)
            if iramp == 41:
                T2, tim2 = Tramp ** 2, time ** 2
                rap, rap2 = 8.0 * time / Tramp, tim2 / T2
                rap22 = 3.0 * rap2
                return ((rap22 - rap + 6.0) * rap2, (4.0 * rap22 - 3.0 * rap + 12.0) * time / T2,
                        (12.0 * rap22 - 6.0 * rap + 12.0) / T2)
            raise ValueError("Unknown ramp")
        if time >= T_stop + Tramp:
            return 0.0, 0.0, 0.0
        if time >= T_stop:
            ti = T_stop + Tramp - time
            if iramp == 1:
                return ti / Tramp, -1.0 / Tramp, 0.0
            if iramp == 2:
                tmp = ti / Tramp
                return tmp * tmp, -2.0 * tmp / Tramp, 2.0 / (Tramp * Tramp)
            if iramp == 21:
                T2, tim2, timsup = Tramp ** 2, ti ** 2, ti / Tramp - 1.0
                if ti <= Tramp / 2.0:
                    return 2.0 * tim2 / T2, -4.0 * ti / T2, 4.0 / T2
                return 1.0 - 2.0 * timsup ** 2, 4.0 * timsup / Tramp, -4.0 / T2
            if iramp == 4:
                tmp = ti / Tramp
                tmp2 = tmp * tmp
                return tmp2 * tmp2, -4.0 * tmp2 * tmp / Tramp, 12.0 * tmp2 / (Tramp * Tramp)
            if iramp == 41:
                T2, tim2 = Tramp ** 2, ti ** 2
                rap, rap2 = 8.0 * ti / Tramp, tim2 / T2
                rap22 = 3.0 * rap2
                return ((rap22 - rap + 6.0) * rap2, -(4.0 * rap22 - 3.0 * rap + 12.0) * ti / T2,
                        (12.0 * rap22 - 6.0 * rap + 12.0) / T2)
            return self._alpha  # unknown ramp: reference leaves alpha unchanged
        return 1.0, 0.0, 0.0

    def pos_1st(self, time):
        """pos_1st (wavemaking.f90:259-304): paddle position and time
        derivatives on the n3 x n2 wavemaker grid."""
        w = TWOPI * self.freq_w                    # (nf,)
        eiwt = np.exp(1j * w * time)
        resu = self.pos_ini * eiwt[None, :]        # (n2, nf)
        p0 = resu.sum(axis=1)
        p1 = (resu * (1j * w)[None, :]).sum(axis=1)
        p2 = (resu * ((1j * w) ** 2)[None, :]).sum(axis=1)
        g = self.pos_gzed[:, None]
        return (g * p0.real[None, :], g * p1.real[None, :], g * p2.real[None, :])

    # --------------------------------------------------------- match surface
    @staticmethod
    def match_coeffs(f, df, d2f):
        """c_poly_add_2 of match_surface_wmk (resol_wmkr.f90:1669-1722) for
        l_add = 2 (x_med = 1), alpha_add = 6, beta_add = 1/3."""
        x = 1.0
        a = 6.0
        b = 1.0 / 3.0
        E = math.exp(-a * b)
        inv_det = 1.0 / (-320 * x ** 13 * E * b ** 4 + 128 * x ** 13 * E * b ** 3
                         + 288 * x ** 13 * E * b ** 5 - 112 * x ** 13 * E * b ** 6
                         + 16 * x ** 13 * E * b ** 7)
        c1 = inv_det * (2 * (3 * x * b ** 4 * df + 2 * x ** 2 * b ** 4 * df * a + f * a ** 2 * x ** 2 * b ** 4
              + 3 * f * a * x * b ** 4 + x ** 2 * b ** 4 * d2f + 3 * f * b ** 4 - 12 * x * b ** 3 * df
              - 8 * x ** 2 * b ** 3 * df * a - 4 * f * a ** 2 * x ** 2 * b ** 3 - 12 * f * a * x * b ** 3
              - 4 * x ** 2 * b ** 3 * d2f - 12 * f * b ** 3 + 4 * x ** 2 * b ** 2 * d2f + 8 * x ** 2 * b ** 2 * df * a
              + 8 * f * b ** 2 + 8 * f * a * x * b ** 2 + 4 * f * a ** 2 * x ** 2 * b ** 2 + 8 * x * b ** 2 * df
              + 8 * f * b + 8 * x * b * df + 8 * f * a * x * b + 8 * f) * (-1 + b) * x ** 6 * E)
        c2 = inv_det * (-2 * (24 * f - 20 * f * a ** 2 * x ** 2 * b ** 3 + 24 * f * a * x * b
              + 12 * x ** 2 * b ** 2 * d2f - 6 * f * a ** 2 * x ** 2 * b ** 5 + 3 * f * x * b ** 6 * a
              + f * x ** 2 * b ** 6 * a ** 2 - 60 * f * a * x * b ** 3 + 12 * f * a ** 2 * x ** 2 * b ** 2
              + 15 * f * a ** 2 * x ** 2 * b ** 4 + 45 * f * a * x * b ** 4 - 18 * f * a * x * b ** 5
              + 2 * x ** 2 * b ** 6 * df * a - 12 * x ** 2 * b ** 5 * df * a + 30 * x ** 2 * b ** 4 * df * a
              - 40 * x ** 2 * b ** 3 * df * a + 24 * x ** 2 * b ** 2 * df * a + 24 * f * b ** 2 - 60 * f * b ** 3
              + 24 * f * b + 45 * f * b ** 4 - 18 * f * b ** 5 + 3 * f * b ** 6 + 24 * f * a * x * b ** 2 + 3 * x * b ** 6 * df
              - 18 * x * b ** 5 * df + 45 * x * b ** 4 * df - 60 * x * b ** 3 * df + 24 * x * b ** 2 * df
              + x ** 2 * b ** 6 * d2f - 6 * x ** 2 * b ** 5 * d2f + 15 * x ** 2 * b ** 4 * d2f - 20 * x ** 2 * b ** 3 * d2f
              + 24 * x * b * df) * (-1 + b) * x ** 8 * E)
        c3 = inv_det * (2 * (24 * f - 28 * f * a ** 2 * x ** 2 * b ** 3 + 24 * f * a * x * b
              + 12 * x ** 2 * b ** 2 * d2f - 12 * f * a ** 2 * x ** 2 * b ** 5 + 10 * f * x * b ** 6 * a
              + 2 * f * x ** 2 * b ** 6 * a ** 2 - 116 * f * a * x * b ** 3 + 12 * f * a ** 2 * x ** 2 * b ** 2
              + 27 * f * a ** 2 * x ** 2 * b ** 4 + 129 * f * a * x * b ** 4 - 60 * f * a * x * b ** 5
              + 4 * x ** 2 * b ** 6 * df * a - 24 * x ** 2 * b ** 5 * df * a
              + 54 * x ** 2 * b ** 4 * df * a - 56 * x ** 2 * b ** 3 * df * a + 24 * x ** 2 * b ** 2 * df * a
              + 24 * f * b ** 2 - 116 * f * b ** 3 + 24 * f * b + 129 * f * b ** 4 - 60 * f * b ** 5 + 10 * f * b ** 6
              + 24 * f * a * x * b ** 2 + 10 * x * b ** 6 * df - 60 * x * b ** 5 * df + 129 * x * b ** 4 * df
              - 116 * x * b ** 3 * df + 24 * x * b ** 2 * df + 2 * x ** 2 * b ** 6 * d2f - 12 * x ** 2 * b ** 5 * d2f
              + 27 * x ** 2 * b ** 4 * d2f - 28 * x ** 2 * b ** 3 * d2f + 24 * x * b * df) * (-1 + b)
              * x ** 10 * E)
        c4 = inv_det * (-2 * (8 * f - 12 * f * a ** 2 * x ** 2 * b ** 3 + 8 * f * a * x * b
              + 4 * x ** 2 * b ** 2 * d2f - 6 * f * a ** 2 * x ** 2 * b ** 5 + 7 * f * x * b ** 6 * a
              + f * x ** 2 * b ** 6 * a ** 2 - 68 * f * a * x * b ** 3 + 4 * f * a ** 2 * x ** 2 * b ** 2
              + 13 * f * a ** 2 * x ** 2 * b ** 4 + 87 * f * a * x * b ** 4 - 42 * f * a * x * b ** 5
              + 2 * x ** 2 * b ** 6 * df * a - 12 * x ** 2 * b ** 5 * df * a + 26 * x ** 2 * b ** 4 * df * a
              - 24 * x ** 2 * b ** 3 * df * a + 8 * x ** 2 * b ** 2 * df * a + 8 * f * b ** 2 - 132 * f * b ** 3
              + 8 * f * b + 183 * f * b ** 4 - 90 * f * b ** 5 + 15 * f * b ** 6 + 8 * f * a * x * b ** 2 + 7 * x * b ** 6 * df
              - 42 * x * b ** 5 * df + 87 * x * b ** 4 * df - 68 * x * b ** 3 * df + 8 * x * b ** 2 * df
              + x ** 2 * b ** 6 * d2f - 6 * x ** 2 * b ** 5 * d2f + 13 * x ** 2 * b ** 4 * d2f - 12 * x ** 2 * b ** 3 * d2f
              + 8 * x * b * df) * (-1 + b) * x ** 12 * E)
        return c1, c2, c3, c4

    def match_surface_wmk(self, data):
        """match_surface_wmk (resol_wmkr.f90:1655-1741): overwrite rows
        n3+1..n3_add of data (n3_add x n2) with the damped odd polynomial."""
        n3, n3_add, l_add, delz = self.n3, self.n3_add, self.l_add, self.delz
        x_med = float(l_add) - 1.0
        out = data.copy()
        a = 6.0
        for i2 in range(self.n2):
            d = data[:, i2]
            df = (d[n3 - 3] - 4.0 * d[n3 - 2] + 3.0 * d[n3 - 1]) / (2.0 * delz)
            f = d[n3 - 1]
            d2f = (-d[n3 - 4] + 4.0 * d[n3 - 3] - 5.0 * d[n3 - 2] + 2.0 * d[n3 - 1]) / (delz ** 2)
            c1, c2, c3, c4 = self.match_coeffs(f, df, d2f)
            for i3 in range(n3 + 1, n3_add + 1):
                xx = float(i3 - 1) / float(n3 - 1) - float(l_add)
                xx2 = xx * xx
                out[i3 - 1, i2] = (((c1 * xx2 + c2) * xx2 + c3) * xx2 + c4) * xx * math.exp(-a * (xx + x_med))
        return out

    # --------------------------------------------------------- dealiasing
    def _dealias_active(self, order):
        p1, p2 = self.p1, self.p2
        return ((p1 != 1 and (order - 1) % (p1 - 1) == 0)
                or (p2 != 1 and (order - 1) % (p2 - 1) == 0))

    def dealias(self, order, a, tx="cos", ty="cos"):
        """dealias (dealiasing.f90:39-92)."""
        F, n1, n2 = self.fourier, self.n1, self.n2
        act = self._dealias_active(order)
        if not act:
            return a
        self._tick(2)
        m = F.S2F_big(a, tx, ty)
        if self.p1 != 1 and (order - 1) % (self.p1 - 1) == 0:
            m[n1:, :] = 0.0
        if n2 != 1 and self.p2 != 1 and (order - 1) % (self.p2 - 1) == 0:
            m[:, n2:] = 0.0
        return F.F2S_big(m, tx, ty)

    def filter_ext(self, a, tx="cos", ty="cos"):
        """filter_ext (dealiasing.f90:96-134): big grid -> n1 x n2 grid."""
        self._tick(2)
        m = self.fourier.S2F_big(a, tx, ty)
        return self.fourier.F2S(m[:self.n1, :self.n2], tx, ty)

    def extend(self, a):
        """extend (variables.f90:243-267)."""
        out = np.zeros((self.nd1, self.nd2))
        out[:self.n1, :self.n2] = a
        return out

    def _tick(self, n=1):
        if self._count:
            self.ntrans += n

    # --------------------------------------------------------- initialize
    def _initialize(self):
        """initialize (initial_condition.f90:314-482), i_wmk = 1, 2."""
        n1, n2, n3, n3_add = self.n1, self.n2, self.n3, self.n3_add
        self.time = 0.0
        self.time_cur = 0.0
        self.eta = np.zeros((n1, n2))
        if self.icase == 1:
            k1 = self.kx[self.islosh - 1]
            self.eta = self.aslosh * np.cos(k1 * self.cx)[:, None] * np.ones((1, n2))
        self.phis = np.zeros((n1, n2))
        z1 = np.zeros((n1, n2))
        za = np.zeros((n3_add, n2))
        self.a1st, self.eta1st, self.a2nd, self.eta2nd = z1.copy(), z1.copy(), z1.copy(), z1.copy()
        self.a1st_add, self.a2nd_add, self.a3rd_add = za.copy(), za.copy(), za.copy()
        self.a_add_ramp = za.copy()
        self.deta = z1.copy()
        self._alpha = (0.0, 0.0, 0.0)
        self._pos = (np.zeros((n3, n2)),) * 3
        self.phi_add = z1.copy()
        if self.icase == 1:
            return
        self._alpha = self.ramp(self.time)
        self._pos = self.pos_1st(self.time)
        alpha, alphat, alphatt = self._alpha
        pos, dpos, d2pos = self._pos
        a = np.zeros((n3_add, n2))
        a[:n3, :] = -alpha * dpos - alphat * pos
        a = self.match_surface_wmk(a)
        a = self.fourier.S2F_add(a, "cos", "cos")
        self.a1st_add = a / self.k_add_thk_add
        da1st, deta1st, da_add, _, phiadd1 = self.solveHOS_SWEET_1(
            self.a1st, self.eta1st, self.a1st_add, self.time)
        self.a_add_ramp = self.a1st_add.copy()
        self.da1st_add = da_add
        if self.inp["i_wmk"] >= 2:
            da2nd, _, da_add_2, _ = self.solveHOS_SWEET_2(self.a2nd, self.eta2nd, self.eta1st, self.a2nd_add,
                                                          self.time)
            if self.inp["i_wmk"] == 3:
                da_add_3 = self.solveHOS_SWEET_3(self.a2nd, da2nd, self.a1st_add, da_add, self.a2nd_add,
                                                 da_add_2, self.time)
                da_add = da_add + da_add_2 + da_add_3
            else:
                da_add = da_add + da_add_2
        out = self.phiadd_SL(self.a1st_add + self.a2nd_add + self.a3rd_add, da_add, self.eta)
        self.phi_add = out[0]

    # --------------------------------------------------------- SWEET 1
    def solveHOS_SWEET_1(self, a1st, eta1st, a_add_1, time):
        """solveHOS_SWEET_1 (resol_wmkr.f90:109-210); with i_wmk = 2 also the
        first-order set of d1st_for_2nd for solveHOS_SWEET_2.
        Returns da1st (modes), deta1st (space), da_add_1, da_add_ramp and
        (phi_add_1, phit_add_1, phiz_add_1)."""
        n1, n2, n3 = self.n1, self.n2, self.n3
        F = self.fourier
        self._alpha = self.ramp(time)
        self._pos = self.pos_1st(time)
        alpha, alphat, alphatt = self._alpha
        pos, dpos, d2pos = self._pos
        d1 = np.zeros((self.n3_add, n2))
        dr = np.zeros((self.n3_add, n2))
        d1[:n3, :] = -alpha * d2pos - 2.0 * alphat * dpos - alphatt * pos
        dr[:n3, :] = -alphat * dpos - alphatt * pos
        dr = self.match_surface_wmk(dr)
        d1 = self.match_surface_wmk(d1)
        d1 = F.S2F_add(d1, "cos", "cos") / self.k_add_thk_add
        dr = F.S2F_add(dr, "cos", "cos") / self.k_add_thk_add
        # phiadd_1st_SWEET (resol_wmkr.f90:446-574): reconstruction at z=0
        cosk = np.cos(self.kx_add)
        sink = np.sin(self.kx_add)
        cy_mat = np.cos(self.ky[:, None] * self.cy[None, :])   # (j2, i2)
        # A(i1, j2) = sum_i3 a(i3, j2) cos(kx_add(i3)) tab(i1, j2, i3)
        A = np.einsum("ij,kji->kj", a_add_1 * cosk[:, None], self.csh_add_x)
        phi2 = A @ cy_mat
        At = np.einsum("ij,kji->kj", d1 * cosk[:, None], self.csh_add_x)
        phi2t = At @ cy_mat
        Az = np.einsum("ij,kji->kj", a_add_1 * sink[:, None], self.kx_add_csh_add_x)
        phi2z = -(Az @ cy_mat)
        # phidphiz (resol_wmkr.f90:583-636)
        phiz1st = F.F2S(a1st * self.kth[:, :, 0], "cos", "cos") + phi2z
        self._tick(3)
        da1 = F.S2F(-eta1st - phi2t - self.iabsnb * self.nu * phiz1st, "cos", "cos")
        if self.inp["i_wmk"] >= 2:
            self._d1st = self._d1st_for_2nd(a1st, da1, a_add_1, d1, phiz1st)
        return da1, phiz1st, d1, dr, (phi2, phi2t, phi2z)

    def _contract_fs(self, coef, tab, trig="cos"):
        """sum_{i3, j2} coef(i3, j2) tab(i1, j2, i3) trig(ky(j2) y(i2)): the
        z = 0 reconstructions of phiadd_1st_SWEET / phiadd_2nd."""
        A = np.einsum("ij,kji->kj", coef, tab)
        m = np.cos if trig == "cos" else np.sin
        return A @ m(self.ky[:, None] * self.cy[None, :])

    def _d1st_for_2nd(self, a1st, da1st, a_add, da_add, phiz1st):
        """phiadd_1st_SWEET's full output set (resol_wmkr.f90:446-574) and
        d1st_for_2nd (resol_wmkr.f90:645-793): first-order quantities on the
        free surface and on the wavemaker that the second order needs."""
        F = self.fourier
        n3 = self.n3
        ca = np.cos(self.kx_add)[:, None]
        sa = np.sin(self.kx_add)[:, None]
        kxa = self.kx_add[:, None]
        ka2 = self.k_add * self.k_add
        ky = self.ky
        C = self._contract_fs
        q = {}
        q["phi2x"] = -C(a_add * ca, self.k_add_sh_add_x)
        q["phi2y"] = -C(a_add * ca, self.kycsh_add_x, "sin")
        q["phi2zz"] = -C(a_add * ca * kxa, self.kx_add_csh_add_x)
        q["phi2xt"] = -C(da_add * ca, self.k_add_sh_add_x)
        q["phi2yt"] = -C(da_add * ca, self.kycsh_add_x, "sin")
        q["phi2zt"] = -C(da_add * sa, self.kx_add_csh_add_x)
        q["phi2xx"] = C(a_add * ca * ka2, self.csh_add_x)
        q["phi2xz"] = C(a_add * sa * kxa, self.k_add_sh_add_x)
        q["phi2yz"] = C(a_add * sa * ky[None, :], self.csh_add_x, "sin")
        # on the wavemaker (the add grid's first n3 nodes)
        w_xx = F.F2S_add(a_add * ka2, "cos", "cos")[:n3]
        w_xxt = F.F2S_add(da_add * ka2, "cos", "cos")[:n3]
        w_y = F.F2S_add(-a_add * ky[None, :], "cos", "sin")[:n3]
        w_yt = F.F2S_add(-da_add * ky[None, :], "cos", "sin")[:n3]
        w_z = F.F2S_add(-a_add * kxa, "sin", "cos")[:n3]
        w_zt = F.F2S_add(-da_add * kxa, "sin", "cos")[:n3]
        # d1st_for_2nd: free-surface modes on the wavemaker, y to space
        def onwmk(a, tab, sign):
            return sign * np.einsum("ij,ijk->kj", a, tab)   # (n3, n2)
        d = {}
        d["phixx_add"] = F.F2S_y(onwmk(a1st, self.kx2cshx_add, -1.0), "cos") + w_xx
        d["phixxt_add"] = F.F2S_y(onwmk(da1st, self.kx2cshx_add, -1.0), "cos") + w_xxt
        d["phiy_add"] = F.F2S_y(onwmk(a1st, self.kycshx_add, -1.0), "sin") + w_y
        d["phiyt_add"] = F.F2S_y(onwmk(da1st, self.kycshx_add, -1.0), "sin") + w_yt
        d["phiz_add"] = F.F2S_y(onwmk(a1st, self.kshx_add, 1.0), "cos") + w_z
        d["phizt_add"] = F.F2S_y(onwmk(da1st, self.kshx_add, 1.0), "cos") + w_zt
        kx = self.kx[:, None]
        kyv = ky[None, :]
        kth1 = self.kth[:, :, 0]
        d["phix1st"] = F.F2S(-a1st * kx, "sin", "cos") + q["phi2x"]
        d["phiy1st"] = F.F2S(-a1st * kyv, "cos", "sin") + q["phi2y"]
        etax = F.F2S(da1st * kx, "sin", "cos")
        etay = F.F2S(da1st * kyv, "cos", "sin")
        d["phizt1st"] = F.F2S(da1st * kth1, "cos", "cos") + q["phi2zt"]
        d["phixx1st"] = F.F2S(-a1st * kx * kx, "cos", "cos") + q["phi2xx"]
        d["phizz1st"] = F.F2S(a1st * self.k * self.k, "cos", "cos") + q["phi2zz"]
        phixz = F.F2S(-a1st * kx * kth1, "sin", "cos") + q["phi2xz"]
        phiyz = F.F2S(-a1st * kyv * kth1, "cos", "sin") + q["phi2yz"]
        d["etax1st"] = etax - q["phi2xt"] - self.iabsnb * (self.dnux * phiz1st + self.nu * phixz)
        d["etay1st"] = etay - q["phi2yt"] - self.iabsnb * (self.dnuy * phiz1st + self.nu * phiyz)
        d["phiz1st"] = phiz1st
        return d

    def _dpos_1st(self, time):
        """dposdy_1st and dposdz_1st (wavemaking.f90:313-406): y and z
        derivatives of the paddle position and their time derivatives."""
        w = TWOPI * self.freq_w
        eiwt = np.exp(1j * w * time)
        ry = self.dposdy_ini * eiwt[None, :]         # (n2, nf)
        rz = self.pos_ini * eiwt[None, :]
        g = self.pos_gzed[:, None]
        dg = self.dpos_gzed[:, None]
        dy = g * ry.sum(axis=1).real[None, :]
        dyt = g * (ry * (1j * w)[None, :]).sum(axis=1).real[None, :]
        dz = dg * rz.sum(axis=1).real[None, :]
        dzt = dg * (rz * (1j * w)[None, :]).sum(axis=1).real[None, :]
        return dy, dyt, dz, dzt

    def solveHOS_SWEET_3(self, a2nd, da2nd, a_add_1, da_add_1, a_add_2, da_add_2, time):
        """solveHOS_SWEET_3 (resol_wmkr.f90:338-437) with wmk_3rdorder
        (resol_wmkr.f90:942-1115), no free-wave correction (ifree = 0):
        the third-order wavemaker condition from the first- and second-order
        potentials at the paddle.  Returns da_add_3.  (phiadd_3rd's fields
        are not read by the right-hand side.)"""
        F = self.fourier
        n3 = self.n3
        ka, kthk = self.k_add, self.k_add_thk_add
        ky = self.ky[None, :]
        kxa = self.kx_add[:, None]
        xxx = F.F2S_add(-a_add_1 * ka * ka * kthk, "cos", "cos")[:n3]
        xxxt = F.F2S_add(-da_add_1 * ka * ka * kthk, "cos", "cos")[:n3]
        xy = F.F2S_add(a_add_1 * ky * kthk, "cos", "sin")[:n3]
        xyt = F.F2S_add(da_add_1 * ky * kthk, "cos", "sin")[:n3]
        xz = F.F2S_add(a_add_1 * kxa * kthk, "sin", "cos")[:n3]
        xzt = F.F2S_add(da_add_1 * kxa * kthk, "sin", "cos")[:n3]

        def onwmk(a, tab, sign):
            return sign * np.einsum("ij,ijk->kj", a, tab)
        xx2 = F.F2S_y(onwmk(a2nd, self.kx2cshx_add, -1.0), "cos") + F.F2S_add(a_add_2 * ka * ka, "cos", "cos")[:n3]
        xxt2 = F.F2S_y(onwmk(da2nd, self.kx2cshx_add, -1.0), "cos") + F.F2S_add(da_add_2 * ka * ka, "cos", "cos")[:n3]
        y2 = F.F2S_y(onwmk(a2nd, self.kycshx_add, -1.0), "sin") + F.F2S_add(-a_add_2 * ky, "cos", "sin")[:n3]
        yt2 = F.F2S_y(onwmk(da2nd, self.kycshx_add, -1.0), "sin") + F.F2S_add(-da_add_2 * ky, "cos", "sin")[:n3]
        z2 = F.F2S_y(onwmk(a2nd, self.kshx_add, 1.0), "cos") + F.F2S_add(-a_add_2 * kxa, "sin", "cos")[:n3]
        zt2 = F.F2S_y(onwmk(da2nd, self.kshx_add, 1.0), "cos") + F.F2S_add(-da_add_2 * kxa, "sin", "cos")[:n3]
        alpha, alphat, _ = self._alpha
        pos, dpos, _ = self._pos
        dy, dyt, dz, dzt = self._dpos_1st(time)
        a_alpha = -alpha * (-dpos * xx2 - pos * xxt2 + dyt * y2 + dy * yt2 + dzt * z2 + dz * zt2)
        a_alphat = -alphat * (-pos * xx2 + dy * y2 + dz * z2)
        a_alpha2 = -alpha ** 2 * (-(pos ** 2) / 2.0 * xxxt - dpos * pos * xxx + dpos * dy * xy + pos * dy * xyt
                                  + pos * dyt * xy + dpos * dz * xz + pos * dz * xzt + pos * dzt * xz)
        a_aat = -alpha * alphat * (-pos ** 2 * xxx + 2.0 * pos * dy * xy + 2.0 * pos * dz * xz)
        dd = np.zeros((self.n3_add, self.n2))
        dd[:n3] = a_alpha + a_alphat + a_alpha2 + a_aat
        dd = self.match_surface_wmk(dd)
        return F.S2F_add(dd, "cos", "cos") / kthk

    def solveHOS_SWEET_2(self, a2nd, eta2nd, eta1st, a_add_2, time):
        """solveHOS_SWEET_2 (resol_wmkr.f90:219-329) with phiadd_2nd
        (resol_wmkr.f90:802-864), no free-wave correction (ifree = 0).
        Needs the first-order set of the same stage (solveHOS_SWEET_1).
        Returns da2nd (modes), deta2nd (space), da_add_2 and the second-order
        additional fields (phi, phix, phiy, phiz, phit) at z = 0."""
        F = self.fourier
        n3 = self.n3
        d = self._d1st
        alpha, alphat, alphatt = self._alpha
        pos, dpos, d2pos = self._pos
        dy, dyt, dz, dzt = self._dpos_1st(time)
        noramp = -pos * d["phixx_add"] + dy * d["phiy_add"] + dz * d["phiz_add"]
        dd = np.zeros((self.n3_add, self.n2))
        dd[:n3] = -alpha * (-pos * d["phixxt_add"] - dpos * d["phixx_add"] + dy * d["phiyt_add"]
                            + dyt * d["phiy_add"] + dz * d["phizt_add"] + dzt * d["phiz_add"]) \
            - alphat * noramp
        dd = self.match_surface_wmk(dd)
        da_add_2 = F.S2F_add(dd, "cos", "cos") / self.k_add_thk_add
        ca = np.cos(self.kx_add)[:, None]
        sa = np.sin(self.kx_add)[:, None]
        C = self._contract_fs
        p2 = C(a_add_2 * ca, self.csh_add_x)
        p2t = C(da_add_2 * ca, self.csh_add_x)
        p2z = -C(a_add_2 * sa, self.kx_add_csh_add_x)
        p2x = -C(a_add_2 * ca, self.k_add_sh_add_x)
        p2y = -C(a_add_2 * ca, self.kycsh_add_x, "sin")
        phiz2nd = F.F2S(a2nd * self.kth[:, :, 0], "cos", "cos") + p2z
        deta2 = phiz2nd - d["phix1st"] * d["etax1st"] - d["phiy1st"] * d["etay1st"] + eta1st * d["phizz1st"]
        da2 = (-eta2nd - p2t - 0.5 * (d["phix1st"] ** 2 + d["phiy1st"] ** 2 + d["phiz1st"] ** 2)
               - eta1st * d["phizt1st"] - self.iabsnb * self.nu * deta2)
        da2 = F.S2F(da2, "cos", "cos")
        return da2, deta2, da_add_2, (p2, p2x, p2y, p2z, p2t)

    # --------------------------------------------------------- phiadd_SL
    def phiadd_SL(self, a_add, da_add, eta):
        """phiadd_SL (resol_wmkr.f90:1124-1187): phi_add and derivatives on
        z = eta, as the y-sum per (i1, i3) then the i3 contraction."""
        kx_add = self.kx_add
        cy_mat = np.cos(self.ky[:, None] * self.cy[None, :])   # (j2, i2)
        sy_mat = np.sin(self.ky[:, None] * self.cy[None, :])
        # B[q](i1, i2, i3) = sum_j2 a(i3,j2) tab(i1,j2,i3) trig(j2,i2): the
        # elementwise product first, then the j2 sum as one matrix product
        n1, n2, n3a = self.csh_add_x.shape[0], cy_mat.shape[0], a_add.shape[0]

        def ysum(a, tab, trig):
            p = a.T[None, :, :] * tab                      # (i1, j2, i3)
            if n2 > 2:
                # ky(j2) y(i2) = pi j2 i2 / (n2 - 1): the sums are the
                # REDFT00 (cos) / RODFT00 on the interior (sin) along j2
                if trig is cy_mat:
                    sgn = np.where(np.arange(n2) % 2 == 0, 1.0, -1.0)[None, :, None]
                    return 0.5 * (_r2r(p, 1, "REDFT00") + p[:, :1, :] + sgn * p[:, -1:, :])
                out = np.zeros_like(p)
                out[:, 1:-1, :] = 0.5 * _r2r(p[:, 1:-1, :], 1, "RODFT00")
                return out
            q = p.transpose(0, 2, 1).reshape(n1 * n3a, n2)
            return (q @ trig).reshape(n1, n3a, trig.shape[1]).transpose(0, 2, 1)

        B_phi = ysum(a_add, self.csh_add_x, cy_mat)
        B_t = ysum(da_add, self.csh_add_x, cy_mat)
        B_x = ysum(a_add, self.k_add_sh_add_x, cy_mat)
        B_y = ysum(a_add, self.kycsh_add_x, sy_mat)
        B_z = ysum(a_add, self.kx_add_csh_add_x, cy_mat)
        arg = kx_add[None, None, :] * (eta[:, :, None] + 1.0)
        c = np.cos(arg)
        s = np.sin(arg)
        phi = (c * B_phi).sum(axis=2)
        phit = (c * B_t).sum(axis=2)
        phix = -(c * B_x).sum(axis=2)
        phiy = -(c * B_y).sum(axis=2)
        phiz = -(s * B_z).sum(axis=2)
        return phi, phix, phiy, phiz, phit

    # --------------------------------------------------------- RHS
    def solveHOS2(self, state, delta_t, time):
        """solveHOS2 (resol_HOS.f90:270-656) for the RK path (no `c`).

        state: dict with G1, G2, a_add_1, a_add_2, a_add_3, a_add_ramp,
        a1st, eta1st, a2nd, eta2nd.  Returns the same keys as derivatives."""
        F = self.fourier
        n1, n2, M = self.n1, self.n2, self.M
        G1, G2 = state["G1"], state["G2"]
        om = self.omega
        # GtoF (variablechange.f90:88-130)
        c = np.cos(-om * delta_t)
        s = np.sin(-om * delta_t)
        etam = G1 * c - G2 * s
        phim = G2 * c + G1 * s
        omd = om.copy()
        omd[0, 0] = 1.0
        phim = phim / omd
        phim[0, 0] = (G2 * c + G1 * s)[0, 0]
        # volume correction with the previous stage's alpha/pos1st
        self._tick(1)
        NL1 = F.F2S(etam)
        alpha = self._alpha[0]
        pos_top = self._pos[0][self.n3 - 1, 0]
        if self.igeom == 2:
            etam[0, 0] = 0.5 * alpha * (1 - self.d_hinge) * pos_top / self.xlen + NL1[0, 0] * alpha * pos_top / self.xlen
        elif self.igeom == 1:
            etam[0, 0] = alpha * pos_top / self.xlen + NL1[0, 0] * alpha * pos_top / self.xlen
        else:
            etam[0, 0] = 0.0
        self._tick(2)
        etark = F.F2S(etam)
        phisrk = F.F2S(phim)
        ext = self._phisxy_etaxy(phisrk, etark)
        hos = self._HOSphis_modes(phisrk, ext)
        etax, etay, phisx, phisy = ext["etax"], ext["etay"], ext["phisx"], ext["phisy"]
        detext = -phisx * etax - phisy * etay
        dphext = -phisx * phisx - phisy * phisy
        detext = self.dealias(2, detext)
        dphext = self.dealias(2, dphext)
        detext = detext + hos["geta2phiz"]
        dphext = dphext + hos["geta2phiz2"] + hos["phiz2"]
        detark = self.filter_ext(detext)
        dphisrk = self.filter_ext(dphext)
        out = {}
        # wavemaker (resol_HOS.f90:403-499)
        if self.icase != 1 and self.igeom in (1, 2):
            da1, deta1, d_add1, d_ramp, _ = self.solveHOS_SWEET_1(
                state["a1st"], state["eta1st"], state["a_add_1"], time)
            a_tot = state["a_add_1"] + state["a_add_2"] + state["a_add_3"]
            da_tot = d_add1
            if self.inp["i_wmk"] >= 2:
                da2, deta2, d_add2, _ = self.solveHOS_SWEET_2(
                    state["a2nd"], state["eta2nd"], state["eta1st"], state["a_add_2"], time)
                da_tot = d_add1 + d_add2
                out.update(a2nd=da2, eta2nd=deta2, a_add_2=d_add2)
                if self.inp["i_wmk"] == 3:
                    d_add3 = self.solveHOS_SWEET_3(state["a2nd"], da2, state["a_add_1"], d_add1,
                                                   state["a_add_2"], d_add2, time)
                    da_tot = d_add1 + d_add2 + d_add3
                    out.update(a_add_3=d_add3)
            phi_add, phix_add, phiy_add, phiz_add, phit_add = self.phiadd_SL(a_tot, da_tot, etark)
            out.update(a1st=da1, eta1st=deta1, a_add_1=d_add1, a_add_ramp=d_ramp)
        else:
            z = np.zeros((n1, n2))
            phi_add = phix_add = phiy_add = phiz_add = phit_add = z
            za = np.zeros((self.n3_add, n2))
            out.update(a1st=z.copy(), eta1st=z.copy(), a_add_1=za.copy(), a_add_ramp=za.copy())
        za = np.zeros((self.n3_add, n2))
        out.setdefault("a_add_2", za.copy())
        out.setdefault("a2nd", np.zeros((n1, n2)))
        out.setdefault("eta2nd", np.zeros((n1, n2)))
        out.setdefault("a_add_3", za.copy())
        self.phi_add = phi_add
        # grad eta . grad phi_add (resol_HOS.f90:534-555)
        self._tick(9)
        px = F.S2F(phix_add)
        py = F.S2F(phiy_add)
        pz = F.S2F(phiz_add)
        pxe, pye, pze = F.F2S_big(self.extend(px)), F.F2S_big(self.extend(py)), F.F2S_big(self.extend(pz))
        phiz_add = F.F2S(pz)
        gg_ext = etax * pxe + etay * pye
        gpg_ext = phisx * pxe + phisy * pye + 0.5 * (pxe * pxe + pye * pye + pze * pze)
        gg = self.filter_ext(gg_ext)
        gpg = self.filter_ext(gpg_ext)
        if M == 1:
            dphin = hos["phiz"] + phiz_add
            detark = dphin - hos["W1"]
            dphisrk = -phit_add - self.nu * dphin
        else:
            dphin = detark + hos["phiz"] + phiz_add - gg
            detark = dphin - hos["W1"]
            dphisrk = 0.5 * dphisrk - phit_add - self.nu * dphin - gpg
        # new variable G (resol_HOS.f90:623-644)
        self._tick(2)
        NL1 = F.S2F(detark)
        NL2 = F.S2F(dphisrk)
        d0 = NL2[0, 0]
        NL2 = NL2 * om
        ce = np.cos(om * delta_t)
        se = np.sin(om * delta_t)
        dG1 = NL1 * ce - NL2 * se
        dG2 = NL2 * ce + NL1 * se
        dG2[0, 0] = d0
        out["G1"], out["G2"] = dG1, dG2
        self.etax, self.etay = etax, etay
        return out

    def _phisxy_etaxy(self, phisrk, etark):
        """phisxy_etaxy (resol_HOS.f90:924-1078)."""
        F, M = self.fourier, self.M
        self._tick(1)
        a = F.S2F(etark)
        ext = {}
        etapm = [None] * M
        self._tick(1)
        etapm[0] = F.F2S_big(self.extend(a))
        for j in range(1, M):
            e = etapm[j - 1] / (j + 1) * etapm[0]
            etapm[j] = self.dealias(j + 1, e)
        ext["etapm"] = etapm
        self._tick(2)
        ext["etax"] = F.F2S_big(self.extend(-self.kx[:, None] * a), "sin", "cos")
        ext["etay"] = F.F2S_big(self.extend(-self.ky[None, :] * a), "cos", "sin")
        ext["gradeta2"] = self.dealias(2, ext["etax"] ** 2 + ext["etay"] ** 2)
        self._tick(3)
        a = F.S2F(phisrk)
        ext["phisx"] = F.F2S_big(self.extend(-self.kx[:, None] * a), "sin", "cos")
        ext["phisy"] = F.F2S_big(self.extend(-self.ky[None, :] * a), "cos", "sin")
        return ext

    def _HOSphis_modes(self, phisrk, ext):
        """HOSphis_modes (resol_HOS.f90:665-915)."""
        F, M = self.fourier, self.M
        etapm, gradeta2 = ext["etapm"], ext["gradeta2"]
        self._tick(1)
        aHOS = [None] * (M + 1)
        aHOS[1] = self.extend(F.S2F(phisrk))
        phizm = [None] * (M + 1)
        for iHOS in range(1, M + 1):
            phimext = np.zeros((self.nd1, self.nd2))
            acc = np.zeros((self.nd1, self.nd2))
            for j in range(iHOS, 1, -1):
                jm1 = j - 1
                j2 = iHOS - jm1
                self._tick(1)
                phizi = F.F2S_big(aHOS[j2] * self.kth_ext[:, :, j - 1])
                phimext = phimext - phizi * etapm[j - 1]
                acc = acc + phizi * etapm[jm1 - 1]
            self._tick(1)
            phizi = F.F2S_big(aHOS[iHOS] * self.kth_ext[:, :, 0])
            phimext = phimext - phizi * etapm[0]
            acc = acc + phizi
            if iHOS > 1:
                acc = self.dealias(iHOS, acc)
            phizm[iHOS] = acc
            if iHOS < M:
                phimext = self.dealias(iHOS + 1, phimext)
                self._tick(1)
                aHOS[iHOS + 1] = F.S2F_big(phimext)
        # kept for the per-order snapshot check of the GPU hook hosnwt_hos_terms
        self.last_phizm = [None] + [p.copy() for p in phizm[1:]]
        self.last_eta_big = etapm[0].copy()
        res = {}
        if M >= 2:
            phizMm1 = np.zeros((self.nd1, self.nd2))
            for j in range(1, M - 1):
                phizMm1 = phizMm1 + phizm[j]
            phizMm1 = phizMm1 + phizm[M - 1]
            res["phiz"] = self.filter_ext(phizMm1) + self.filter_ext(phizm[M])
            res["phizMm1"] = phizMm1
        else:
            res["phiz"] = self.filter_ext(phizm[1])
            res["phizMm1"] = np.zeros((self.nd1, self.nd2))
        res["W1"] = self.filter_ext(phizm[1])
        geta2phiz = np.zeros((self.nd1, self.nd2))
        for j in range(1, M - 2):
            geta2phiz = geta2phiz + self.dealias(j + 2, gradeta2 * phizm[j])
        if M >= 3:
            geta2phiz = geta2phiz + self.dealias(M, gradeta2 * phizm[max(M - 2, 1)])
        res["geta2phiz"] = geta2phiz
        t1 = np.zeros((self.nd1, self.nd2))
        geta2phiz2 = np.zeros((self.nd1, self.nd2))
        for j in range(1, (M - 2) // 2 + 1):
            t2 = self.dealias(2 * j, phizm[j] * phizm[j])
            t1 = t1 + t2
            t2 = self.dealias(2 * j + 2, gradeta2 * t2)
            geta2phiz2 = geta2phiz2 + t2
        for j in range(2, M - 2):
            for q in range(1, min(M - 2 - j, j - 1) + 1):
                t2 = self.dealias(j + q, 2.0 * phizm[j] * phizm[q])
                t1 = t1 + t2
                t2 = self.dealias(j + q + 2, gradeta2 * t2)
                geta2phiz2 = geta2phiz2 + t2
        if M >= 2:
            t2 = self.dealias(2 * (M // 2), phizm[M // 2] * phizm[M // 2])
            t1 = t1 + t2
        for j in range(2, M):
            for q in range(max(0, min(M - 2 - j, j - 1)) + 1, min(M - j, j - 1) + 1):
                t2 = self.dealias(j + q, 2.0 * phizm[j] * phizm[q])
                t1 = t1 + t2
        res["phiz2"] = t1
        res["geta2phiz2"] = geta2phiz2
        return res

    # --------------------------------------------------------- RK step
    STATE_KEYS = ("G1", "G2", "a_add_1", "a_add_2", "a_add_ramp", "a_add_3",
                  "a1st", "eta1st", "a2nd", "eta2nd")
    # fill_butcher_array (runge_kutta.f90:40-72)
    RK_A = np.array([[0, 0, 0, 0, 0], [0.5, 0, 0, 0, 0], [0, 0.5, 0, 0, 0],
                     [0, 0, 1.0, 0, 0], [-1.0, 2.0, 0, 0, 0]])
    RK_b = np.array([1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 0.0])
    RK_c = np.array([0.0, 0.5, 0.5, 1.0, 1.0])
    RK_e = np.array([1.0 / 6.0, 2.0 / 3.0, 0.0, 0.0, 1.0 / 6.0])
    RK_p = 4

    def runge4_adapt2(self, t_o, eta, phis, a_add_1, a_add_2, a_add_ramp, a_add_3,
                      eta1st, eta2nd, a1st, a2nd, h_loc):
        """runge4_adapt2 (runge_kutta.f90:81-360).  Returns (new arrays, err,
        deta, stage-5 derivatives)."""
        F, om = self.fourier, self.omega
        G1 = F.S2F(eta)
        G2 = F.S2F(phis)
        phisrk0 = G2[0, 0]
        G2 = G2 * om
        y0 = dict(G1=G1, G2=G2, a_add_1=a_add_1, a_add_2=a_add_2, a_add_ramp=a_add_ramp,
                  a_add_3=a_add_3, a1st=a1st, eta1st=eta1st, a2nd=a2nd, eta2nd=eta2nd)
        ks = []
        self.time = t_o
        k = self.solveHOS2(y0, h_loc * self.RK_c[0], self.time)
        k["G2"][0, 0] = 0.0
        ks.append(k)
        for s in range(1, 5):
            ys = {}
            for key in self.STATE_KEYS:
                acc = np.zeros_like(y0[key])
                for ns in range(s):
                    acc = acc + ks[ns][key] * self.RK_A[s, ns]
                ys[key] = y0[key] + h_loc * acc
            self.time = t_o + h_loc * self.RK_c[s]
            k = self.solveHOS2(ys, h_loc * self.RK_c[s], self.time)
            k["G2"][0, 0] = 0.0
            ks.append(k)
        new = {}
        dsum = {}
        for key in self.STATE_KEYS:
            acc = np.zeros_like(y0[key])
            for j in range(5):
                acc = acc + ks[j][key] * self.RK_b[j]
            dsum[key] = acc
            new[key] = y0[key] + h_loc * acc
        err = 0.0
        for key in ("G1", "G2", "a_add_1", "a_add_2", "a_add_3"):
            e = np.zeros_like(y0[key])
            for j in range(5):
                e = e + ks[j][key] * self.RK_e[j]
            e = (e - dsum[key]) * h_loc
            e = np.abs(e) / (np.max(np.abs(new[key])) + TINY)
            err = max(err, float(np.max(e)))
        # GtoF of the new state and of the last stage slope (runge_kutta.f90:281-296)
        c = np.cos(-om * h_loc)
        s = np.sin(-om * h_loc)
        etam = new["G1"] * c - new["G2"] * s
        phim = new["G2"] * c + new["G1"] * s
        detam = ks[4]["G1"] * c - ks[4]["G2"] * s
        mask = np.ones(om.shape, dtype=bool)
        mask[0, 0] = False
        ph = phim.copy()
        ph[0, 0] = phisrk0
        ph[mask] = phim[mask] / om[mask]
        detam[mask] = detam[mask] + ph[mask] * om[mask] ** 2
        modesFS = F.F2S(etam)
        alpha = self._alpha[0]
        pos_top = self._pos[0][self.n3 - 1, 0]
        if self.igeom == 2:
            etam[0, 0] = 0.5 * alpha * (1 - self.d_hinge) * pos_top / self.xlen + modesFS[0, 0] * alpha * pos_top / self.xlen
        elif self.igeom == 1:
            etam[0, 0] = alpha * pos_top / self.xlen + modesFS[0, 0] * alpha * pos_top / self.xlen
        else:
            etam[0, 0] = 0.0
        self.modesFS = etam.copy()
        eta_n = F.F2S(etam)
        phis_n = F.F2S(ph)
        deta = F.F2S(detam)
        res = dict(eta=eta_n, phis=phis_n, a_add_1=new["a_add_1"], a_add_2=new["a_add_2"],
                   a_add_ramp=new["a_add_ramp"], a_add_3=new["a_add_3"],
                   eta1st=new["eta1st"], eta2nd=new["eta2nd"], a1st=new["a1st"], a2nd=new["a2nd"])
        return res, err, deta, ks

    # --------------------------------------------------------- time loop
    def state_tuple(self):
        return (self.eta, self.phis, self.a1st_add, self.a2nd_add, self.a_add_ramp, self.a3rd_add,
                self.eta1st, self.eta2nd, self.a1st, self.a2nd)

    def advance_to(self, time_next, h_rk, max_steps=None):
        """Inner adaptive loop of HOS-NWT.f90:498-571 up to time_next.
        Returns (h_rk, n_accepted, n_rejected)."""
        n_rk = n_err = 0
        endramp = getattr(self, "_endramp", 0)
        steps = 0
        while self.time_cur < time_next:
            h_loc = h_rk
            if time_next - self.time_cur < h_rk:
                h_loc = time_next - self.time_cur
            res, error, deta, _ = self.runge4_adapt2(self.time_cur, *self.state_tuple(), h_loc)
            if error > self.toler and h_rk > 0.001 * 0.95 * self.dt_stab:
                # REAL(4) constants in the reference (HOS-NWT.f90:525)
                dt_correc = float(np.float32(0.9)) * (error / self.toler) ** (-(float(np.float32(1.0) / np.float32(self.RK_p))))
                n_err += 1
                if abs(self.Tramp - (self.time_cur + h_loc)) <= TINY and self.Tramp > self.time_cur:
                    endramp = 0
            else:
                self.eta, self.phis = res["eta"], res["phis"]
                self.a1st_add, self.a2nd_add = res["a_add_1"], res["a_add_2"]
                self.a_add_ramp, self.a3rd_add = res["a_add_ramp"], res["a_add_3"]
                self.a1st, self.a2nd = res["a1st"], res["a2nd"]
                self.eta1st, self.eta2nd = res["eta1st"], res["eta2nd"]
                self.deta = deta
                if (self.iramp == 1 and self.Tramp - (self.time_cur + h_loc) <= TINY
                        and self.Tramp > self.time_cur and endramp != 1):
                    self.a1st_add = self.a1st_add - self.a_add_ramp
                    endramp = 1
                self.time_cur = self.time_cur + h_loc
                if abs(error) < TINY:
                    dt_correc = 2.0
                else:
                    dt_correc = 0.9 * (error / self.toler) ** (-(1.0 / float(self.RK_p)))
                n_rk += 1
            h_rk = h_rk * dt_correc
            h_rk = min(h_rk, 0.95 * self.dt_stab, self.delt_out)
            h_rk = max(h_rk, 0.0001 * 0.95 * self.dt_stab, 0.0001 * self.delt_out)
            steps += 1
            if max_steps is not None and steps >= max_steps:
                break
        self._endramp = endramp
        return h_rk, n_rk, n_err

    def probes(self):
        """Probe elevations (output.f90:265-282), nondimensional."""
        FT = self.fourier.S2F(self.eta)
        return np.einsum("ij,ijp->p", FT, self.mat_coscos)

    def volume(self):
        """volume (vol_energy.f90:36-62)."""
        e = self.eta
        if self.n2 == 1:
            s = 0.5 * (e[:, 0] + e[:, 0])
        else:
            s = 0.5 * (e[:, 0] + e[:, -1]) + e[:, 1:-1].sum(axis=1)
        v = (0.5 * (s[0] + s[-1]) + s[1:-1].sum()) * self.delx
        v = v / self.xlen
        if self.n2 != 1:
            v = v / self.ylen * self.dely
        return v

    def energy(self):
        """energy (vol_energy.f90:69-119) with phis + phi_add and deta."""
        def integ(f):
            if self.n2 == 1:
                sy = 0.5 * (f[:, 0] + f[:, 0])
            else:
                sy = 0.5 * (f[:, 0] + f[:, -1]) + f[:, 1:-1].sum(axis=1)
            v = (0.5 * (sy[0] + sy[-1]) + sy[1:-1].sum()) * self.delx
            return v
        ep = integ(self.eta * self.eta) / 2.0
        ek = integ((self.phis + self.phi_add) * self.deta) / 2.0
        if self.n2 != 1:
            ep *= self.dely
            ek *= self.dely
        return ep, ek

    def run(self, T_end=None, on_output=None):
        """Whole time loop (HOS-NWT.f90:446-581); returns probe records."""
        T_stop = self.T_stop if T_end is None else T_end / self.Tscale
        recs = []
        h_rk = self.delt
        while self.time_cur < T_stop + self.delt_out:
            if self.probes_xy is not None:
                recs.append((self.time_cur, self.probes().copy()))
            if on_output is not None:
                on_output(self)
            if abs(self.time_cur - T_stop) <= TINY:
                break
            time_next = self.time_cur + self.delt_out
            if time_next > T_stop + self.delt_out:
                time_next = T_stop + self.delt_out
            h_rk = self.delt
            h_rk, _, _ = self.advance_to(time_next, h_rk)
            self.delt = h_rk
            self.check_slope()
        return recs

    def check_slope(self):
        """check_slope (initial_condition.f90:687-716) with the cut filter of
        filtering_x/filtering_base (filtering.f90:37-86, 334-360)."""
        F = self.fourier
        etax = getattr(self, "etax", None)
        if etax is None:
            return False
        hit = False
        if np.max(np.abs(etax)) > 8.0:
            nf = abs(int(self.n1 * 0.7))
            for name in ("phis", "eta"):
                m = F.S2F(getattr(self, name))
                m[nf:, :] = 0.0
                setattr(self, name, F.F2S(m))
            hit = True
        if np.max(np.abs(self.etay)) > 8.0 and self.n2 != 1:
            nf = abs(int(self.n2 * 0.7))
            for name in ("phis", "eta"):
                m = F.S2F(getattr(self, name))
                m[:, nf:] = 0.0
                setattr(self, name, F.F2S(m))
            hit = True
        return hit
