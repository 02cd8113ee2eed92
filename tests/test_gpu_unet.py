"""The U-Net's GPU kernels (tensor-core convolutions, backward pass, Adam)
against the numpy oracle with the same BF16 rounding points, and the
tcgen05 convolutions against the mma.sync ones on volumes where every level
runs on tcgen05 (x-rows tiling into 128-cell blocks).

Tolerances: outputs and gradients are compared as relative L2 norms per
layer. The GPU sums in FP32 in another order than the oracle, so a stored
BF16 activation can differ by one BF16 unit (2^-8 relative) where a value sits
near a rounding boundary; 2e-2 on outputs and 5e-2 on gradients leaves room
for that and nothing else (a wrong tap, channel or transpose gives O(1))."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def _case(seed, shape=(2, 8, 8, 16)):
    rng = np.random.default_rng(seed)
    flat = U.init_params(seed)
    offs = np.cumsum([0] + [27 * ci * co + co for _, ci, co, _ in U.LAYERS])
    for li, (_, ci, co, _) in enumerate(U.LAYERS):  # non-zero biases
        flat[offs[li + 1] - co:offs[li + 1]] = 0.1 * rng.standard_normal(co)
    x = rng.standard_normal(shape + (2,)).astype(np.float32)
    t = rng.standard_normal(shape).astype(np.float32)
    return flat, x, t


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_param_layout_round_trip(nusif_lib):
    from nusif import UNet
    with UNet(seed=5) as net:
        assert net.n_params == U.param_count()
        p = net.params()
        # He-normal weights, zero biases, per the flat layout
        w = U.unpack(p.astype(np.float64))
        for name, ci, co, _ in U.LAYERS:
            assert np.all(w[name][1] == 0.0)
            assert np.std(w[name][0]) == pytest.approx(np.sqrt(2.0 / (27 * ci)), rel=0.25)
        flat, _, _ = _case(1)
        net.set_params(flat)
        np.testing.assert_array_equal(net.params(), flat)


@pytest.mark.parametrize("shape", [(2, 8, 8, 16), (1, 12, 8, 4)])
def test_forward_matches_oracle(nusif_lib, shape):
    from nusif import UNet
    flat, x, _ = _case(2, shape)
    ref = U.UNet(flat).forward(x)
    with UNet() as net:
        net.set_params(flat)
        out = net.forward(_dev(x)).cpu().numpy()
    assert _rel(out, ref) < 2e-2
    # and the BF16 network stays close to the float64 one
    assert _rel(out, U.UNet(flat, bf16_mode=False).forward(x)) < 5e-2


def test_gradients_match_oracle(nusif_lib):
    from nusif import UNet
    flat, x, t = _case(3)
    onet = U.UNet(flat)
    out = onet.forward(x)
    loss, dout = U.mse(out, t)
    gref = onet.backward(dout)
    with UNet() as net:
        net.set_params(flat)
        gl = net.train_step(_dev(x), _dev(t), update=False)
        g = net.grads()
        np.testing.assert_array_equal(net.params(), flat)  # no update
    assert gl == pytest.approx(loss, rel=2e-2)
    offs = np.cumsum([0] + [27 * ci * co + co for _, ci, co, _ in U.LAYERS])
    for li, (name, ci, co, _) in enumerate(U.LAYERS):
        w0, w1 = offs[li], offs[li + 1] - co
        assert _rel(g[w0:w1], gref[w0:w1]) < 5e-2, name
        assert _rel(g[w1:offs[li + 1]], gref[w1:offs[li + 1]]) < 5e-2, name + " bias"


def test_adam_step_matches_formula(nusif_lib):
    from nusif import UNet
    flat, x, t = _case(4)
    lr = 1e-3
    with UNet() as net:
        net.set_params(flat)
        net.train_step(_dev(x), _dev(t), lr=lr, update=False)
        g = net.grads().astype(np.float64)
        net.set_params(flat)
        net.train_step(_dev(x), _dev(t), lr=lr, update=True)
        g2 = net.grads().astype(np.float64)
        new = net.params()
    np.testing.assert_allclose(g2, g, rtol=0, atol=1e-6 * np.abs(g).max())  # deterministic
    want, _, _ = U.adam(flat.astype(np.float64), g, np.zeros_like(g), np.zeros_like(g), 1, lr=lr)
    np.testing.assert_allclose(new, want, rtol=0, atol=2e-6)


def test_training_reduces_loss(nusif_lib):
    """A learnable map (a fixed smoothing of channel 0 plus channel 1): 150 Adam
    steps on one batch cut the loss by more than 5x."""
    from nusif import UNet
    rng = np.random.default_rng(9)
    x = rng.standard_normal((4, 16, 16, 16, 2)).astype(np.float32)
    s = x[..., 0].copy()
    for ax in (1, 2, 3):
        s = (np.roll(s, 1, ax) + 2 * s + np.roll(s, -1, ax)) / 4
    t = (2.0 * s + 0.5 * x[..., 1]).astype(np.float32)
    with UNet(seed=1) as net:
        xd, td = _dev(x), _dev(t)
        first = net.train_step(xd, td, lr=1e-3, update=True)
        for _ in range(148):
            net.train_step(xd, td, lr=1e-3, update=True, want_loss=False)
        last = net.train_step(xd, td, lr=1e-3, update=True)
    assert last < first / 5, (first, last)


@pytest.mark.parametrize("shape", [(1, 16, 16, 32), (2, 16, 32, 16)])
def test_tcgen05_forward_matches_oracle(nusif_lib, shape):
    """Levels 0 and 1 of these volumes run on tcgen05 (level 2 where it tiles)."""
    from nusif import UNet
    flat, x, _ = _case(6, shape)
    ref = U.UNet(flat).forward(x)
    with UNet() as net:
        net.set_params(flat)
        out = net.forward(_dev(x)).cpu().numpy()
    assert _rel(out, ref) < 2e-2


@pytest.mark.parametrize("shape", [(1, 64, 64, 64), (2, 32, 32, 64)])
def test_tcgen05_matches_mma_sync(nusif_lib, shape):
    """Every level on tcgen05 against every level on mma.sync: the forward
    output and all gradients (both paths share the BF16 rounding points and
    differ only in FP32 summation order)."""
    from nusif import UNet
    flat, x, t = _case(7, shape)
    res = {}
    for tc in (True, False):
        with UNet() as net:
            net.set_params(flat)
            net.set_tensor_core(tc)
            out = net.forward(_dev(x)).cpu().numpy()
            loss = net.train_step(_dev(x), _dev(t), update=False)
            res[tc] = (out, loss, net.grads())
    assert _rel(res[True][0], res[False][0]) < 1e-2
    assert res[True][1] == pytest.approx(res[False][1], rel=1e-2)
    offs = np.cumsum([0] + [27 * ci * co + co for _, ci, co, _ in U.LAYERS])
    for li, (name, ci, co, _) in enumerate(U.LAYERS):
        a, b = res[True][2][offs[li]:offs[li + 1]], res[False][2][offs[li]:offs[li + 1]]
        assert _rel(a, b) < 3e-2, name
