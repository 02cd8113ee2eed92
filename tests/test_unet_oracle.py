"""The U-Net oracle checked on its own (CPU): its backward pass against central
finite differences of its forward pass in float64, the BF16 rounding helper,
and the warm-start features / targets against their definitions."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import unet_oracle as U


def _loss(flat, x, t):
    net = U.UNet(flat, bf16_mode=False)
    return U.mse(net.forward(x), t)[0]


def test_param_count():
    # 3-level U-Net at 16/32/64 channels: about a quarter of a million parameters
    assert U.param_count() == 243473


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(7)
    flat = U.init_params(3).astype(np.float64)
    flat += 0.05 * rng.standard_normal(flat.size)  # non-zero biases too
    x = rng.standard_normal((2, 4, 4, 8, 2))
    t = rng.standard_normal((2, 4, 4, 8))
    net = U.UNet(flat, bf16_mode=False)
    loss, dout = U.mse(net.forward(x), t)
    g = net.backward(dout)
    offs = np.cumsum([0] + [27 * ci * co + co for _, ci, co, _ in U.LAYERS])
    picks = []
    for li in range(len(U.LAYERS)):  # weights and a bias of every layer
        picks += list(rng.integers(offs[li], offs[li + 1] - U.LAYERS[li][2], 3))
        picks.append(offs[li + 1] - 1)
    h = 1e-6
    for i in picks:
        e = np.zeros_like(flat)
        e[i] = h
        fd = (_loss(flat + e, x, t) - _loss(flat - e, x, t)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 65504.0, 1e-30], np.float32)
    b = U.bf16(a)
    # bf16 keeps 8 significant bits; 1 + 2^-8 is a tie and rounds to even (1.0)
    assert b[0] == 1.0 and b[1] == 1.0
    assert b[2] == np.float32(1.0078125)
    assert abs(b[3] - a[3]) <= abs(a[3]) * 2 ** -8
    assert np.all(b.view(np.uint32) & 0xFFFF == 0)


def test_features_and_target_definitions():
    rng = np.random.default_rng(11)
    n = 8
    p = rng.standard_normal((n + 2,) * 3)
    p[0], p[-1] = p[1], p[-2]
    p[:, 0], p[:, -1] = p[:, 1], p[:, -2]
    p[:, :, 0], p[:, :, -1] = p[:, :, 1], p[:, :, -2]
    rhs = rng.standard_normal((n + 2,) * 3)
    h = 1.0 / n
    x, s = U.features(p, rhs, h, h, h)
    assert x.shape == (n // 2,) * 3 + (2,)
    assert np.sqrt(np.mean(x[..., 0] ** 2)) == pytest.approx(1.0, rel=1e-6)
    assert np.sqrt(np.mean(x[..., 1] ** 2)) == pytest.approx(1.0, rel=1e-6)
    # a p that solves the Neumann problem has zero residual features
    b = rhs[1:-1, 1:-1, 1:-1] - rhs[1:-1, 1:-1, 1:-1].mean()
    lap = U.laplacian(p, h, h, h)
    assert np.allclose(U.restrict(b - lap) / s, x[..., 0], atol=1e-5)
    t = U.target(p, p + 1.0, s, h, h, h)
    assert np.allclose(t, U.kappa((n, n, n), h, h, h) / s)
    assert U.kappa((n, n, n), h, h, h) == pytest.approx(3 * np.pi ** 2)


def test_adam_step():
    w = np.array([1.0, -2.0])
    g = np.array([0.5, -0.25])
    w1, m, v = U.adam(w, g, np.zeros(2), np.zeros(2), 1, lr=0.1)
    # first bias-corrected step moves every weight by lr against its gradient's sign
    assert np.allclose(w1, w - 0.1 * np.sign(g), atol=1e-6)
