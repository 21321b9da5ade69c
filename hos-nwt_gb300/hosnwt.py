"""Python binding of libhosnwt.so (ctypes), mirroring the reference's
interfaces: read_input (input.f90:62), runge4_adapt2 (runge_kutta.f90:81),
solveHOS2 (resol_HOS.f90:270), SPACE_2_FOURIER / FOURIER_2_SPACE
(fourier_FFTW.f90:35-63) and the time loop of HOS-NWT.f90.

Arrays are numpy float64 of shape (n1, n2) (free surface) or (n3_add, n2)
(wavemaker modes); they are passed to the library in Fortran order, i1
fastest, like the reference's arrays.  The library runs on the current CUDA
device; there is no CPU fallback: importing works without a GPU, creating a
tank does not.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhosnwt.so")

HOSNWT_OK = 0
ERRORS = {1: "ARG", 2: "CUDA", 3: "NAN", 4: "TIMEOUT", 5: "DT_UNDERFLOW", 6: "IO", 7: "UNSUPPORTED"}

C_FUNCTIONS = ("hosnwt_read_input", "hosnwt_create", "hosnwt_destroy", "hosnwt_last_error",
               "hosnwt_get_info", "hosnwt_runge4_adapt2", "hosnwt_step", "hosnwt_accept",
               "hosnwt_advance", "hosnwt_run", "hosnwt_get_state", "hosnwt_set_state",
               "hosnwt_probes", "hosnwt_solveHOS2", "hosnwt_transform", "hosnwt_advance_many",
               "hosnwt_time_transform", "hosnwt_fp64_peak", "hosnwt_get_rk_state",
               "hosnwt_transform_noalloc", "hosnwt_diagnostics", "hosnwt_check_slope")


class HosInput(ctypes.Structure):
    _fields_ = [
        ("xlen", ctypes.c_double), ("ylen", ctypes.c_double), ("h", ctypes.c_double),
        ("icase", ctypes.c_int), ("islosh", ctypes.c_int), ("aslosh", ctypes.c_double),
        ("amp_mono", ctypes.c_double), ("nu_mono", ctypes.c_double),
        ("theta_mono", ctypes.c_double), ("ph_mono", ctypes.c_double),
        ("ibat", ctypes.c_int), ("xd_mono", ctypes.c_double),
        ("file_name", ctypes.c_char * 256), ("i_cut", ctypes.c_int),
        ("nuc_low", ctypes.c_double), ("nuc_high", ctypes.c_double),
        ("Hs", ctypes.c_double), ("Tp", ctypes.c_double), ("gamma", ctypes.c_double),
        ("iseed", ctypes.c_int), ("i_wmk", ctypes.c_int), ("igeom", ctypes.c_int),
        ("d_hinge", ctypes.c_double), ("iramp", ctypes.c_int), ("Tramp", ctypes.c_double),
        ("iabsnb", ctypes.c_int), ("xabsf", ctypes.c_double), ("coeffabsf", ctypes.c_double),
        ("iprobes", ctypes.c_int), ("pro_file", ctypes.c_char * 256),
        ("T_stop", ctypes.c_double), ("toler", ctypes.c_double), ("f_out", ctypes.c_double),
        ("idim", ctypes.c_int), ("i3d", ctypes.c_int), ("imodes", ctypes.c_int),
        ("iwmk", ctypes.c_int), ("i_sw", ctypes.c_int),
    ]


class HosNumerics(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("n1", "n2", "n3", "mHOS", "p1", "p2")]


class HosInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("n1", "n2", "n3", "n3_add", "nd1", "nd2", "mHOS", "p1", "p2")] + \
        [(n, ctypes.c_double) for n in ("Tscale", "xlen", "ylen", "dt_stab", "delt", "delt_out",
                                        "T_stop", "toler", "time_cur")] + \
        [("nprobes", ctypes.c_int), ("n_rhs", ctypes.c_longlong), ("kernels_per_step", ctypes.c_int),
         ("device_ms", ctypes.c_double), ("fmas_per_step", ctypes.c_double), ("step_control", ctypes.c_int)]


_lib = None


def load_library(path=LIB_PATH):
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with hos-nwt_gb300/build.py")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    dp = P(ctypes.c_double)
    vp = ctypes.c_void_p
    lib.hosnwt_read_input.argtypes = [ctypes.c_char_p, P(HosInput)]
    lib.hosnwt_create.argtypes = [P(HosInput), P(HosNumerics), ctypes.c_char_p, dp, ctypes.c_int, P(vp)]
    lib.hosnwt_destroy.argtypes = [vp]
    lib.hosnwt_destroy.restype = None
    lib.hosnwt_last_error.argtypes = [vp]
    lib.hosnwt_last_error.restype = ctypes.c_char_p
    lib.hosnwt_get_info.argtypes = [vp, P(HosInfo)]
    lib.hosnwt_runge4_adapt2.argtypes = [vp, ctypes.c_double] + [dp] * 10 + [ctypes.c_double, dp]
    lib.hosnwt_step.argtypes = [vp, ctypes.c_double, dp]
    lib.hosnwt_accept.argtypes = [vp, ctypes.c_double]
    lib.hosnwt_advance.argtypes = [vp, ctypes.c_double, dp, P(ctypes.c_int), P(ctypes.c_int)]
    lib.hosnwt_run.argtypes = [vp, ctypes.c_char_p]
    lib.hosnwt_get_state.argtypes = [vp, dp, dp, dp]
    lib.hosnwt_set_state.argtypes = [vp, dp, dp]
    lib.hosnwt_probes.argtypes = [vp, dp]
    lib.hosnwt_solveHOS2.argtypes = [vp, P(dp), P(dp), ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double]
    lib.hosnwt_transform.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp]
    lib.hosnwt_hos_terms.argtypes = [vp, dp, dp]
    lib.hosnwt_advance_many.argtypes = [P(vp), ctypes.c_int, dp, dp]
    lib.hosnwt_time_transform.argtypes = [vp] + [ctypes.c_int] * 10 + [dp]
    lib.hosnwt_fp64_peak.argtypes = [dp]
    lib.hosnwt_get_rk_state.argtypes = [vp] + [dp] * 10
    lib.hosnwt_diagnostics.argtypes = [vp, dp]
    lib.hosnwt_check_slope.argtypes = [vp, P(ctypes.c_int)]
    lib.hosnwt_transform_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    vp8 = ctypes.c_void_p
    ll = ctypes.c_longlong
    ci = ctypes.c_int
    lib.hosnwt_tc_gemm_bf16.argtypes = [vp8, ll, vp8, ll, vp8, ll, ci, ci, ci, ci, vp8, ci, vp8, vp8, vp8]
    _lib = lib
    return lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_input(d):
    """hosnwt_input from a dict with the input_HOS-NWT.dat field names."""
    s = HosInput()
    for name, typ in HosInput._fields_:
        if name not in d:
            continue
        v = d[name]
        if typ in (ctypes.c_int,):
            setattr(s, name, int(v))
        elif typ is ctypes.c_double:
            setattr(s, name, float(v))
        else:
            setattr(s, name, str(v).encode())
    return s


def fp64_peak_gflops():
    """FP64 FMA throughput of the current device (GFLOP/s)."""
    v = ctypes.c_double()
    if load_library().hosnwt_fp64_peak(ctypes.byref(v)) != HOSNWT_OK:
        raise HosError("hosnwt_fp64_peak failed")
    return v.value


def read_input(path):
    """read_input (input.f90:62-201) through the library's parser."""
    lib = load_library()
    s = HosInput()
    rc = lib.hosnwt_read_input(path.encode(), ctypes.byref(s))
    if rc != HOSNWT_OK:
        raise RuntimeError(f"hosnwt_read_input failed ({ERRORS.get(rc, rc)})")
    out = {}
    for name, typ in HosInput._fields_:
        v = getattr(s, name)
        out[name] = v.decode() if isinstance(v, bytes) else v
    return out


NOALLOC_MAX_N = 16385  # HOSNWT_NOALLOC_MAX_N of include/hosnwt.h


def transform_noalloc(direction, cs, n, nlines, in_ptr, out_ptr, stream=0):
    """hosnwt_transform_noalloc on device pointers (integers): the transform
    for callers that cannot allocate device memory; see include/hosnwt.h."""
    rc = load_library().hosnwt_transform_noalloc(int(direction), CS[cs] if isinstance(cs, str) else int(cs),
                                                 int(n), int(nlines), ctypes.c_void_p(in_ptr),
                                                 ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream))
    if rc != HOSNWT_OK:
        raise HosError(f"hosnwt_transform_noalloc failed ({ERRORS.get(rc, rc)})")


def advance_many(tanks, time_next, h_rk):
    """Advance independent tanks together (hosnwt_advance_many): each tank
    keeps its own adaptive step; their launches overlap on the GPU.
    time_next, h_rk: sequences (nondimensional); returns the new h_rk."""
    n = len(tanks)
    arr = (ctypes.c_void_p * n)(*[t._h.value for t in tanks])
    tn = np.ascontiguousarray(np.asarray(time_next, dtype=np.float64))
    hr = np.ascontiguousarray(np.asarray(h_rk, dtype=np.float64)).copy()
    rc = load_library().hosnwt_advance_many(arr, n, _dptr(tn), _dptr(hr))
    if rc != HOSNWT_OK:
        raise HosError(f"hosnwt_advance_many failed ({ERRORS.get(rc, rc)})")
    return hr


GRID = {"n": 0, "big": 1, "add": 2}
CS = {"cos": 0, "sin": 1}


class HosError(RuntimeError):
    pass


class Tank:
    """One wave tank on the current CUDA device."""

    def __init__(self, inp, n1, n2, n3, mHOS, p1, p2=1, probes=None, wave_dir="."):
        self.lib = load_library()
        self.n1, self.n2, self.n3, self.M = int(n1), int(n2), int(n3), int(mHOS)
        self.n3_add = 2 * (self.n3 - 1)
        self._in = make_input(inp)
        self._num = HosNumerics(self.n1, self.n2, self.n3, self.M, int(p1), int(p2))
        pr = None
        self.nprobes = 0
        if probes is not None:
            pr = np.ascontiguousarray(np.asarray(probes, dtype=np.float64).reshape(-1, 2))
            self.nprobes = pr.shape[0]
        self._probes = pr
        h = ctypes.c_void_p()
        rc = self.lib.hosnwt_create(ctypes.byref(self._in), ctypes.byref(self._num),
                                    wave_dir.encode(), _dptr(pr) if pr is not None else None,
                                    self.nprobes, ctypes.byref(h))
        self._h = h
        if rc != HOSNWT_OK:
            msg = self.lib.hosnwt_last_error(h).decode() if h.value else ""
            self.close()
            raise HosError(f"hosnwt_create failed ({ERRORS.get(rc, rc)}): {msg}")

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.lib.hosnwt_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != HOSNWT_OK:
            raise HosError(f"{what} failed ({ERRORS.get(rc, rc)}): "
                           f"{self.lib.hosnwt_last_error(self._h).decode()}")

    # ------------------------------------------------------------------ info
    def info(self):
        s = HosInfo()
        self._check(self.lib.hosnwt_get_info(self._h, ctypes.byref(s)), "get_info")
        return {n: getattr(s, n) for n, _ in HosInfo._fields_}

    # ------------------------------------------------------------ hot path
    def runge4_adapt2(self, t_o, eta, phis, a_add_1, a_add_2, a_add_ramp, a_add_3,
                      eta1st, eta2nd, a1st, a2nd, h_loc):
        """runge4_adapt2: returns (new arrays tuple in the same order, err)."""
        arrs = [np.array(a, dtype=np.float64, order="F", copy=True)
                for a in (eta, phis, a_add_1, a_add_2, a_add_ramp, a_add_3, eta1st, eta2nd, a1st, a2nd)]
        err = ctypes.c_double()
        rc = self.lib.hosnwt_runge4_adapt2(self._h, float(t_o), *[_dptr(a) for a in arrs],
                                           float(h_loc), ctypes.byref(err))
        self._check(rc, "runge4_adapt2")
        return tuple(arrs), err.value

    def solveHOS2(self, y, delta_t, time, alpha_prev, pos_top_prev):
        """y: 10 arrays (G1, G2, a_add_1, a_add_2, a_add_ramp, a_add_3, a1st,
        eta1st, a2nd, eta2nd); returns the 10 slopes."""
        ys = [np.array(a, dtype=np.float64, order="F", copy=True) for a in y]
        ks = [np.zeros_like(a, order="F") for a in ys]
        yp = (ctypes.POINTER(ctypes.c_double) * 10)(*[_dptr(a) for a in ys])
        kp = (ctypes.POINTER(ctypes.c_double) * 10)(*[_dptr(a) for a in ks])
        rc = self.lib.hosnwt_solveHOS2(self._h, yp, kp, float(delta_t), float(time),
                                       float(alpha_prev), float(pos_top_prev))
        self._check(rc, "solveHOS2")
        return ks

    def hos_terms(self):
        """eta on the dealiased grid and the M vertical-velocity terms
        phizm(:,:,1..M) of the last right-hand side evaluated on this tank
        (hosnwt_hos_terms): arrays (nd1, nd2) and (M, nd1, nd2)."""
        inf = self.info()
        nd1, nd2 = inf["nd1"], inf["nd2"]
        eta = np.zeros((nd1, nd2), order="F")
        phizm = np.zeros(self.M * nd1 * nd2)
        self._check(self.lib.hosnwt_hos_terms(self._h, _dptr(eta), _dptr(phizm)), "hos_terms")
        return eta, np.stack([phizm[m * nd1 * nd2:(m + 1) * nd1 * nd2].reshape((nd1, nd2), order="F")
                              for m in range(self.M)])

    def transform(self, grid, direction, csx, csy, a):
        """SPACE_2_FOURIER (direction=+1) / FOURIER_2_SPACE (-1) on the
        'n', 'big' or 'add' grid."""
        x = np.array(a, dtype=np.float64, order="F", copy=True)
        out = np.zeros_like(x, order="F")
        rc = self.lib.hosnwt_transform(self._h, GRID[grid], int(direction), CS[csx], CS[csy],
                                       _dptr(x), _dptr(out))
        self._check(rc, "transform")
        return out

    def time_transform(self, grid, direction, csx, csy, nin, nout, batch=1, nrep=20):
        ms = ctypes.c_double()
        rc = self.lib.hosnwt_time_transform(self._h, GRID[grid], int(direction), CS[csx], CS[csy],
                                            int(nin[0]), int(nin[1]), int(nout[0]), int(nout[1]),
                                            int(batch), int(nrep), ctypes.byref(ms))
        self._check(rc, "time_transform")
        return ms.value

    def step(self, h_loc):
        err = ctypes.c_double()
        self._check(self.lib.hosnwt_step(self._h, float(h_loc), ctypes.byref(err)), "step")
        return err.value

    def accept(self, h_loc):
        self._check(self.lib.hosnwt_accept(self._h, float(h_loc)), "accept")

    def advance(self, time_next, h_rk):
        h = ctypes.c_double(h_rk)
        na, nr = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.hosnwt_advance(self._h, float(time_next), ctypes.byref(h),
                                            ctypes.byref(na), ctypes.byref(nr)), "advance")
        return h.value, na.value, nr.value

    def run(self, results_dir=None):
        self._check(self.lib.hosnwt_run(self._h, results_dir.encode() if results_dir else None), "run")

    def get_state(self):
        eta = np.zeros((self.n1, self.n2), order="F")
        phis = np.zeros((self.n1, self.n2), order="F")
        deta = np.zeros((self.n1, self.n2), order="F")
        self._check(self.lib.hosnwt_get_state(self._h, _dptr(eta), _dptr(phis), _dptr(deta)), "get_state")
        return eta, phis, deta

    def get_rk_state(self, out=None):
        """The 10 arrays of runge4_adapt2 (eta, phis, a_add_1, a_add_2,
        a_add_ramp, a_add_3, eta1st, eta2nd, a1st, a2nd); `out` may supply
        preallocated Fortran-ordered arrays (e.g. pinned host memory)."""
        n1, n2, na = self.n1, self.n2, self.n3_add
        shapes = [(n1, n2)] * 2 + [(na, n2)] * 4 + [(n1, n2)] * 4
        arrs = out if out is not None else [np.zeros(s, order="F") for s in shapes]
        rc = self.lib.hosnwt_get_rk_state(self._h, *[_dptr(a) for a in arrs])
        self._check(rc, "get_rk_state")
        return arrs

    def runge4_adapt2_inplace(self, t_o, arrs, h_loc):
        """runge4_adapt2 on caller-owned Fortran-ordered arrays (no copies)."""
        err = ctypes.c_double()
        rc = self.lib.hosnwt_runge4_adapt2(self._h, float(t_o), *[_dptr(a) for a in arrs],
                                           float(h_loc), ctypes.byref(err))
        self._check(rc, "runge4_adapt2")
        return err.value

    def set_state(self, eta, phis):
        e = np.array(eta, dtype=np.float64, order="F", copy=True)
        p = np.array(phis, dtype=np.float64, order="F", copy=True)
        self._check(self.lib.hosnwt_set_state(self._h, _dptr(e), _dptr(p)), "set_state")

    def diagnostics(self):
        """(volume, potential energy, kinetic energy, max|eta_x|, max|eta_y|)."""
        out = np.zeros(5)
        self._check(self.lib.hosnwt_diagnostics(self._h, _dptr(out)), "diagnostics")
        return out

    def check_slope(self):
        f = ctypes.c_int()
        self._check(self.lib.hosnwt_check_slope(self._h, ctypes.byref(f)), "check_slope")
        return f.value

    def probes(self):
        out = np.zeros(max(self.nprobes, 1))
        self._check(self.lib.hosnwt_probes(self._h, _dptr(out)), "probes")
        return out[:self.nprobes]

    def simulate(self, T_end=None):
        """The time loop of HOS-NWT.f90:446-581 with probe records at each
        output time; returns [(time, probes)] (nondimensional)."""
        inf = self.info()
        T_stop = inf["T_stop"] if T_end is None else T_end / inf["Tscale"]
        delt, delt_out = inf["delt"], inf["delt_out"]
        tiny = float(np.finfo(np.float64).eps)
        recs = []
        while self.info()["time_cur"] < T_stop + delt_out:
            t = self.info()["time_cur"]
            recs.append((t, self.probes().copy()))
            if abs(t - T_stop) <= tiny:
                break
            time_next = min(t + delt_out, T_stop + delt_out)
            delt, _, _ = self.advance(time_next, delt)
            self.check_slope()
        return recs


def tc_gemm(A, B, bias=None, act=0, Dadd=None, out=None, out_bf16=False, err=None, stream=0):
    """hosnwt_tc_gemm_bf16 on CUDA tensors: act(A B^T + bias + Dadd) with A
    (M x K) and B (N x K) BF16 row-major (row strides A.stride(0),
    B.stride(0)), FP32 accumulation; returns D (M x N, FP32 or BF16).  `err`
    is an optional int32 CUDA tensor of one element that the kernel sets to
    1 if one of its waits timed out."""
    import torch
    M, K = A.shape
    N = B.shape[0]
    if out is None:
        out = torch.empty((M, N), dtype=torch.bfloat16 if out_bf16 else torch.float32, device=A.device)
    if err is None:
        err = torch.zeros(1, dtype=torch.int32, device=A.device)
    # the row stride of a one-row matrix is arbitrary in PyTorch (a transposed
    # column reports 1); the kernel never steps over it, so pass the row length
    lda = A.stride(0) if M > 1 else K
    ldb = B.stride(0) if N > 1 else K
    ldd = out.stride(0) if M > 1 else N
    rc = load_library().hosnwt_tc_gemm_bf16(
        A.data_ptr(), lda, B.data_ptr(), ldb, out.data_ptr(), ldd,
        1 if out.dtype == torch.bfloat16 else 0, M, N, K, bias.data_ptr() if bias is not None else None,
        int(act), Dadd.data_ptr() if Dadd is not None else None, err.data_ptr(), stream)
    if rc != HOSNWT_OK:
        raise HosError(f"hosnwt_tc_gemm_bf16 failed ({ERRORS.get(rc, rc)})")
    return out
