"""Fourier-neural-operator surrogate for the high HOS orders of a 2-D tank.

What it learns: the orders 4..M part of the vertical velocity,
W_hi = sum_{m=4..M} phizm(:, m), on the dealiased grid, from eta and
phizm(:, 1..3) of the same right-hand side (HOSphis_modes,
resol_HOS.f90:665-915).  Snapshots come from the plain FP64 GPU solver
through hosnwt_hos_terms.

Arithmetic: BF16 weights and activations entering every contraction, FP32
accumulation, FP32 master weights in the optimiser.  Every contraction of
the forward and the backward pass (lift, projection, pointwise channel
mixes, the truncated cosine transforms and the per-mode channel mixes) runs
on the library's tcgen05 kernel (hosnwt_tc_gemm_bf16); PyTorch is the
training harness (autograd, GELU, Adam).  There is no fallback: without the
CUDA library the calls raise.

The spectral layers use the tank's own basis, cos(pi j k / D) on the
dealiased grid (D = nd1 - 1), truncated to the lowest `modes` modes; the
per-mode 32 x 32 channel mixes are one block-diagonal contraction.

This surrogate is trained and checked offline, on held-out snapshots; it is
not used inside the time loop.
"""
from __future__ import annotations

import math
import time

import numpy as np

import hosnwt


def _torch():
    import torch
    return torch


_ERR = {}


def _err_flag(device):
    torch = _torch()
    key = str(device)
    if key not in _ERR:
        _ERR[key] = torch.zeros(1, dtype=torch.int32, device=device)
    return _ERR[key]


def gemm_bf16(A, B):
    """D = A B^T on tcgen05: A (R, K), B (N, K) cast to BF16; D FP32 (R, N).
    K is zero-padded to a multiple of 8 (the TMA row-stride rule)."""
    torch = _torch()
    A = A.to(torch.bfloat16)
    B = B.to(torch.bfloat16)
    K = A.shape[1]
    if K % 8:
        pad = 8 - K % 8
        A = torch.nn.functional.pad(A, (0, pad))
        B = torch.nn.functional.pad(B, (0, pad))
    A = A.contiguous()
    B = B.contiguous()
    if A.data_ptr() % 16:
        A = A.clone()
    if B.data_ptr() % 16:
        B = B.clone()
    return hosnwt.tc_gemm(A, B, err=_err_flag(A.device), stream=torch.cuda.current_stream().cuda_stream)


def check_kernel_flags():
    """Raise if a wait inside the tensor-core kernel timed out."""
    for t in _ERR.values():
        v = int(t.item())
        if v == 2:
            raise hosnwt.HosError("tc_gemm: the MMAs never reported completion; their tensor memory was "
                                  "left allocated, so the CUDA context must not be used further")
        if v != 0:
            raise hosnwt.HosError("tc_gemm: a bounded wait timed out")


class _TcMatmul:
    """y = x W^T with its gradients, every product on tcgen05."""

    _fn = None

    @classmethod
    def fn(cls):
        if cls._fn is None:
            torch = _torch()

            class F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, x, w):
                    xb = x.to(torch.bfloat16)
                    wb = w.to(torch.bfloat16)
                    ctx.save_for_backward(xb, wb)
                    return gemm_bf16(xb, wb)

                @staticmethod
                def backward(ctx, gy):
                    xb, wb = ctx.saved_tensors
                    gyb = gy.to(torch.bfloat16)
                    gx = gw = None
                    if ctx.needs_input_grad[0]:
                        gx = gemm_bf16(gyb, wb.t())              # (R, N) x (N, K)
                    if ctx.needs_input_grad[1]:
                        gw = gemm_bf16(gyb.t(), xb.t())          # (N, R) x (R, K)
                    return gx, gw

            cls._fn = F
        return cls._fn


def tc_matmul(x, w):
    """x (R, K) times w (N, K) transposed: (R, N), differentiable."""
    return _TcMatmul.fn().apply(x, w)


def cos_bases(nd, modes, device):
    """Truncated cosine transform pair on nd points (D = nd - 1), scaled as
    the tank's SPACE_2_FOURIER / FOURIER_2_SPACE: forward (modes, nd) gives
    the amplitudes a_k of x = sum_k a_k cos(pi j k / D), inverse (nd, modes)
    sums them back, so inverse(forward x) keeps the lowest `modes` modes of
    x exactly."""
    torch = _torch()
    D = nd - 1
    j = np.arange(nd)
    k = np.arange(modes)
    c = np.cos(np.pi * np.outer(k, j) / D)
    wj = np.ones(nd)
    wj[0] = wj[-1] = 0.5
    ek = np.full(modes, 2.0)
    ek[0] = 1.0
    fwd = c * wj[None, :] * ek[:, None] / D
    inv = c.T
    return (torch.tensor(fwd, dtype=torch.float32, device=device),
            torch.tensor(inv, dtype=torch.float32, device=device))


def build_fno(nd, c_in=4, width=32, modes=64, layers=4, seed=0, device="cuda"):
    """The 4-layer FNO (32 channels, `modes` cosine modes) as a torch module."""
    torch = _torch()
    nn = torch.nn

    class Linear(nn.Module):
        def __init__(self, cin, cout):
            super().__init__()
            self.w = nn.Parameter(torch.randn(cout, cin) / math.sqrt(cin))
            self.b = nn.Parameter(torch.zeros(cout))

        def forward(self, x):  # (..., cin)
            sh = x.shape
            y = tc_matmul(x.reshape(-1, sh[-1]), self.w) + self.b
            return y.reshape(*sh[:-1], -1)

    class Spectral(nn.Module):
        def __init__(self, fwd, inv):
            super().__init__()
            self.register_buffer("fwd", fwd)
            self.register_buffer("inv", inv)
            self.R = nn.Parameter(torch.randn(modes, width, width) / math.sqrt(width))

        def forward(self, x):  # (Bt, nd, C)
            Bt = x.shape[0]
            xt = x.permute(0, 2, 1).reshape(Bt * width, nd)
            xh = tc_matmul(xt, self.fwd)                                   # (Bt C, modes)
            xh = xh.reshape(Bt, width, modes).permute(0, 2, 1).reshape(Bt, modes * width)
            yh = tc_matmul(xh, torch.block_diag(*self.R.unbind(0)))         # per-mode channel mixes
            yh = yh.reshape(Bt, modes, width).permute(0, 2, 1).reshape(Bt * width, modes)
            y = tc_matmul(yh, self.inv)                                    # (Bt C, nd)
            return y.reshape(Bt, width, nd).permute(0, 2, 1)

    class FNO(nn.Module):
        def __init__(self):
            super().__init__()
            fwd, inv = cos_bases(nd, modes, "cpu")
            self.lift = Linear(c_in, width)
            self.spec = nn.ModuleList([Spectral(fwd, inv) for _ in range(layers)])
            self.point = nn.ModuleList([Linear(width, width) for _ in range(layers)])
            self.proj1 = Linear(width, width)
            self.proj2 = Linear(width, 1)

        def forward(self, x):  # (Bt, nd, c_in) -> (Bt, nd)
            h = self.lift(x)
            for s, p in zip(self.spec, self.point):
                h = torch.nn.functional.gelu(s(h) + p(h))
            return self.proj2(torch.nn.functional.gelu(self.proj1(h)))[..., 0]

    torch.manual_seed(seed)
    return FNO().to(device)


def features(eta_big, phizm):
    """Inputs (nd, 4): eta and phizm(:, 1..3); target (nd,): sum of
    phizm(:, 4..M), all on the dealiased grid of a 2-D tank."""
    x = np.stack([eta_big[:, 0], phizm[0][:, 0], phizm[1][:, 0], phizm[2][:, 0]], axis=-1)
    y = phizm[3:, :, 0].sum(axis=0)
    return x, y


def collect(tank, t_start, t_end, dt_sample, h_rk):
    """Snapshots of a plain run: advance with the reference's step control to
    each sample time, then evaluate one step from there without accepting it
    and read the terms of its last right-hand side.  Returns (X, Y, W)
    arrays (n, nd, 4), (n, nd), (n, nd) with W the whole vertical velocity
    sum_{m=1..M} phizm, and the last step size.  (The probe step leaves its
    last stage's ramp and paddle values behind, which the next right-hand
    side's volume correction of the mean mode reads, as after a rejected
    step; the sampled run is a valid run, not bit-identical to an unsampled
    one.)"""
    Ts = tank.info()["Tscale"]
    X, Y, W = [], [], []
    t = t_start
    while t <= t_end + 1e-9:
        h_rk, _, _ = tank.advance(t / Ts, h_rk)
        tank.step(h_rk)
        eta, pz = tank.hos_terms()
        x, y = features(eta, pz)
        X.append(x)
        Y.append(y)
        W.append(pz[:, :, 0].sum(axis=0))
        t += dt_sample
    return np.array(X), np.array(Y), np.array(W), h_rk


def train(model, X, Y, iters=600, batch=32, lr=3e-3, seed=0):
    """Adam on the normalised MSE; returns (losses, seconds, scales)."""
    torch = _torch()
    dev = next(model.parameters()).device
    xs = X.reshape(-1, X.shape[-1]).std(axis=0) + 1e-30
    ys = Y.std() + 1e-30
    Xt = torch.tensor(X / xs, dtype=torch.float32, device=dev)
    Yt = torch.tensor(Y / ys, dtype=torch.float32, device=dev)
    opt = torch.optim.Adam(model.parameters(), lr=lr)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, iters)
    g = torch.Generator(device="cpu").manual_seed(seed)
    losses = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(iters):
        idx = torch.randint(0, Xt.shape[0], (min(batch, Xt.shape[0]),), generator=g).to(dev)
        pred = model(Xt[idx])
        loss = torch.mean((pred - Yt[idx]) ** 2)
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        sched.step()
        losses.append(float(loss.detach()))
    torch.cuda.synchronize()
    check_kernel_flags()
    return losses, time.perf_counter() - t0, (xs, ys)


def predict(model, X, scales):
    torch = _torch()
    xs, ys = scales
    dev = next(model.parameters()).device
    with torch.no_grad():
        Xt = torch.tensor(X / xs, dtype=torch.float32, device=dev)
        out = model(Xt).double().cpu().numpy() * ys
    check_kernel_flags()
    return out
