"""Host-side pieces of the surrogate (CPU): the truncated cosine bases and the
snapshot features."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import surrogate


def test_cos_bases_keep_low_modes():
    nd, modes = 65, 16
    fwd, inv = surrogate.cos_bases(nd, modes, "cpu")
    D = nd - 1
    j = np.arange(nd)
    # a field made of the lowest modes only is reproduced exactly
    a = np.random.default_rng(0).standard_normal(modes)
    x = sum(a[k] * np.cos(np.pi * k * j / D) for k in range(modes))
    xh = fwd.double().numpy() @ x
    assert np.allclose(xh, a, atol=1e-6)
    assert np.allclose(inv.double().numpy() @ xh, x, atol=1e-5)
    # a mode above the truncation is removed
    y = np.cos(np.pi * (modes + 3) * j / D)
    assert np.max(np.abs(fwd.double().numpy() @ y)) < 1e-6


def test_features_split_orders():
    nd, M = 20, 7
    rng = np.random.default_rng(1)
    eta = rng.standard_normal((nd, 1))
    pz = rng.standard_normal((M, nd, 1))
    x, y = surrogate.features(eta, pz)
    assert x.shape == (nd, 4) and y.shape == (nd,)
    assert np.allclose(x[:, 0], eta[:, 0]) and np.allclose(x[:, 3], pz[2, :, 0])
    assert np.allclose(y, pz[3:, :, 0].sum(axis=0))
