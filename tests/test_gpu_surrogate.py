"""The surrogate's pieces on the GPU: the tensor-core product with its
gradients (against a PyTorch FP32 reference of the same BF16 inputs), the
snapshot hook hosnwt_hos_terms (against the oracle's phizm of the same
right-hand side) and a short FNO training run.

Tolerances: products of BF16 values are exact in FP32, so only the FP32
summation order differs: |got - ref| <= 1e-5 * max sum |a||b|.  The snapshot
hook returns the FP64 terms of the right-hand side: 1e-10 relative, as the
right-hand-side parity tests."""
import numpy as np
import pytest

import cases
from oracle.hos_oracle import Tank as OTank

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _bf(t):
    return t.bfloat16().float()


def test_tc_matmul_forward_backward(lib):
    import surrogate
    g = torch.Generator(device="cuda").manual_seed(11)
    # (300, 1, 36): the weight gradient multiplies a transposed one-column
    # gradient, a one-row view whose row stride PyTorch reports as 1
    for R, N, K in [(300, 24, 36), (1, 32, 40), (300, 1, 36), (2052, 32, 32), (64, 2048, 2048)]:
        x = torch.randn(R, K, device="cuda", generator=g, requires_grad=True)
        w = torch.randn(N, K, device="cuda", generator=g, requires_grad=True)
        y = surrogate.tc_matmul(x, w)
        gy = torch.randn(R, N, device="cuda", generator=g)
        y.backward(gy)
        torch.cuda.synchronize()
        surrogate.check_kernel_flags()
        xb, wb, gyb = _bf(x.detach()), _bf(w.detach()), _bf(gy)
        tol = lambda a, b: 1e-5 * (a.abs() @ b.abs()).max().item()
        assert (y - xb @ wb.T).abs().max().item() <= tol(xb, wb.T), (R, N, K)
        assert (x.grad - gyb @ wb).abs().max().item() <= tol(gyb, wb), (R, N, K)
        assert (w.grad - gyb.T @ xb).abs().max().item() <= tol(gyb.T, xb), (R, N, K)


@pytest.mark.parametrize("name", ["reg1d_m5", "reg3d"])
def test_hos_terms_match_oracle(lib, name):
    import hosnwt
    case = cases.ALL[name]
    g = hosnwt.Tank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"])
    o = OTank(case["inp"], case["n1"], case["n2"], case["n3"], case["mHOS"], case["p1"], case["p2"])
    rng = np.random.default_rng(3)
    n1, n2, n3a = o.n1, o.n2, o.n3_add
    decay = np.exp(-0.15 * np.arange(n1))[:, None] * np.exp(-0.3 * np.arange(n2))[None, :]
    y = {k: np.zeros((n3a if k.startswith("a_add") else n1, n2)) for k in o.STATE_KEYS}
    y["G1"] = 1e-2 * rng.standard_normal((n1, n2)) * decay
    y["G2"] = 1e-2 * rng.standard_normal((n1, n2)) * decay * o.omega
    y["G2"][0, 0] = 0.0
    t, dt = 1.3, 0.02
    # the previous stage's ramp and paddle top, read by the volume correction
    alpha_prev, pos_top = o._alpha[0], o._pos[0][o.n3 - 1, 0]
    o.solveHOS2({k: v.copy() for k, v in y.items()}, dt, t)
    g.solveHOS2([y[k] for k in o.STATE_KEYS], dt, t, alpha_prev, pos_top)
    eta, pz = g.hos_terms()
    scale = max(np.max(np.abs(o.last_eta_big)), 1e-300)
    assert np.max(np.abs(eta - o.last_eta_big)) <= 1e-10 * scale
    for m in range(case["mHOS"]):
        r = o.last_phizm[m + 1]
        sc = max(np.max(np.abs(r)), 1e-300)
        assert np.max(np.abs(pz[m] - r)) <= 1e-10 * sc, (m + 1, np.max(np.abs(pz[m] - r)) / sc)
    g.close()


def test_fno_training_reduces_loss(lib):
    import surrogate
    nd, n = 130, 64
    rng = np.random.default_rng(0)
    j = np.arange(nd)
    X = np.zeros((n, nd, 4))
    for i in range(n):
        a = rng.standard_normal((4, 6)) / (1 + np.arange(6))
        for c in range(4):
            X[i, :, c] = sum(a[c, k] * np.cos(np.pi * k * j / (nd - 1)) for k in range(6))
    Y = X[:, :, 0] * X[:, :, 1] + 0.5 * X[:, :, 2] ** 2
    model = surrogate.build_fno(nd, modes=16)
    losses, _, sc = surrogate.train(model, X, Y, iters=150, batch=16, lr=3e-3)
    assert np.mean(losses[-10:]) < 0.05 * np.mean(losses[:10])
    pred = surrogate.predict(model, X[:8], sc)
    assert np.linalg.norm(pred - Y[:8]) / np.linalg.norm(Y[:8]) < 0.25
