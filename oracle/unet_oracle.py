"""CPU oracle of the learned pressure warm start -- TEST INFRASTRUCTURE ONLY.

A numpy restatement of the 3-level 3D U-Net that the library trains and runs
on the GPU (cfd-bench_gb300/csrc/unet.cu), with its forward pass, its backward
pass, one Adam step, and the features / targets made from a pressure solve.
The reference has no learned component, so this oracle is project-written
("parity unpinned" against the reference by construction); its backward pass
is checked against finite differences (tests/test_unet_oracle.py) and the GPU
kernels are checked against it.

Network (volumes are channels-last [B][Z][Y][X][C]; every conv is 3x3x3,
zero padding, weights W[tap][cout][cin] with tap = 9(dz+1) + 3(dy+1) + (dx+1)):

    e0a  2->16 relu   e0b 16->16 relu           (level 0, the feature grid)
    pool (2x2x2 mean)
    e1a 16->32 relu   e1b 32->32 relu           (level 1)
    pool
    e2a 32->64 relu                             (level 2)
    up (nearest x2), concat [up(e2a), e1b] = 96
    d1a 96->32 relu   d1b 32->32 relu           (level 1)
    up, concat [up(d1b), e0b] = 48
    d0a 48->16 relu   d0b 16->16 relu           (level 0)
    out 16->1 (linear, FP32)

Precision model (``bf16=True``, what the GPU computes): features, weights and
every stored activation are rounded to BF16 (round to nearest even); sums are
exact here and FP32 on the GPU; the output and every gradient are FP32, except
that a layer's output gradient times its ReLU mask is rounded to BF16 before
it meets the tensor cores. ``bf16=False`` keeps everything in float64 (for the
finite-difference check).
"""
from __future__ import annotations

import numpy as np

LAYERS = [  # name, cin, cout, relu
    ("e0a", 2, 16, True), ("e0b", 16, 16, True),
    ("e1a", 16, 32, True), ("e1b", 32, 32, True),
    ("e2a", 32, 64, True),
    ("d1a", 96, 32, True), ("d1b", 32, 32, True),
    ("d0a", 48, 16, True), ("d0b", 16, 16, True),
    ("out", 16, 1, False),
]
TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def param_count() -> int:
    return sum(27 * ci * co + co for _, ci, co, _ in LAYERS)


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(flat):
    """Flat parameter vector (layer order; per layer W[27][cout][cin] then b[cout])."""
    out, o = {}, 0
    for name, ci, co, _ in LAYERS:
        w = flat[o:o + 27 * co * ci].reshape(27, co, ci)
        o += 27 * co * ci
        b = flat[o:o + co]
        o += co
        out[name] = (w, b)
    assert o == flat.size
    return out


def pack(params):
    return np.concatenate([np.concatenate([params[n][0].ravel(), params[n][1].ravel()])
                           for n, _, _, _ in LAYERS])


def init_params(seed: int) -> np.ndarray:
    """He-normal weights (std sqrt(2 / (27 cin))), zero biases, from numpy's PCG64."""
    rng = np.random.default_rng(seed)
    parts = []
    for _, ci, co, _ in LAYERS:
        parts.append(rng.standard_normal(27 * co * ci) * np.sqrt(2.0 / (27 * ci)))
        parts.append(np.zeros(co))
    return np.concatenate(parts).astype(np.float32)


def _shift(x, dz, dy, dx):
    """y[b,z,y,x] = x[b,z+dz,y+dy,x+dx] (zero outside)."""
    out = np.zeros_like(x)
    B, Z, Y, X = x.shape[:4]
    zs, ys, xs = slice(max(0, -dz), Z - max(0, dz)), slice(max(0, -dy), Y - max(0, dy)), \
        slice(max(0, -dx), X - max(0, dx))
    zsrc = slice(max(0, dz), Z - max(0, -dz))
    ysrc = slice(max(0, dy), Y - max(0, -dy))
    xsrc = slice(max(0, dx), X - max(0, -dx))
    out[:, zs, ys, xs] = x[:, zsrc, ysrc, xsrc]
    return out


def conv(x, w, b):
    y = np.zeros(x.shape[:4] + (w.shape[1],), dtype=np.float64)
    for t, (dz, dy, dx) in enumerate(TAPS):
        y += _shift(x, dz, dy, dx).astype(np.float64) @ w[t].T.astype(np.float64)
    return y + b


def conv_dgrad(g, w):
    """dX[c] = sum_tap G[c - off] W[tap]: the adjoint of conv in x."""
    dx = np.zeros(g.shape[:4] + (w.shape[2],), dtype=np.float64)
    for t, (oz, oy, ox) in enumerate(TAPS):
        dx += _shift(g.astype(np.float64) @ w[t].astype(np.float64), -oz, -oy, -ox)
    return dx


def conv_wgrad(g, x):
    co, ci = g.shape[-1], x.shape[-1]
    dw = np.zeros((27, co, ci))
    g2 = g.reshape(-1, co).astype(np.float64)
    for t, (dz, dy, dx) in enumerate(TAPS):
        dw[t] = g2.T @ _shift(x, dz, dy, dx).reshape(-1, ci).astype(np.float64)
    return dw, g2.sum(axis=0)


def pool(x):
    B, Z, Y, X, C = x.shape
    return x.reshape(B, Z // 2, 2, Y // 2, 2, X // 2, 2, C).mean(axis=(2, 4, 6))


def pool_back(g):
    return np.repeat(np.repeat(np.repeat(g, 2, 1), 2, 2), 2, 3) / 8.0


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 1), 2, 2), 2, 3)


def up_back(g):
    B, Z, Y, X, C = g.shape
    return g.reshape(B, Z // 2, 2, Y // 2, 2, X // 2, 2, C).sum(axis=(2, 4, 6))


class UNet:
    """Forward / backward of the network for one parameter vector."""

    def __init__(self, flat, bf16_mode: bool = True):
        self.q = bf16 if bf16_mode else (lambda a: np.asarray(a, dtype=np.float64))
        self.f32 = (lambda a: np.asarray(a, dtype=np.float32)) if bf16_mode else \
            (lambda a: np.asarray(a, dtype=np.float64))
        p = unpack(np.asarray(flat, dtype=np.float64))
        self.w = {n: (self.q(w), b) for n, (w, b) in p.items()}

    def _layer(self, name, x, relu=True):
        w, b = self.w[name]
        y = conv(x, w, b)
        return self.q(np.maximum(y, 0.0)) if relu else self.f32(y)

    def forward(self, x):
        a = {"x": self.q(x)}
        a["e0a"] = self._layer("e0a", a["x"])
        a["e0b"] = self._layer("e0b", a["e0a"])
        a["p0"] = self.q(pool(a["e0b"]))
        a["e1a"] = self._layer("e1a", a["p0"])
        a["e1b"] = self._layer("e1b", a["e1a"])
        a["p1"] = self.q(pool(a["e1b"]))
        a["e2a"] = self._layer("e2a", a["p1"])
        a["c1"] = np.concatenate([up(a["e2a"]), a["e1b"]], axis=-1)
        a["d1a"] = self._layer("d1a", a["c1"])
        a["d1b"] = self._layer("d1b", a["d1a"])
        a["c0"] = np.concatenate([up(a["d1b"]), a["e0b"]], axis=-1)
        a["d0a"] = self._layer("d0a", a["c0"])
        a["d0b"] = self._layer("d0b", a["d0a"])
        a["out"] = self._layer("out", a["d0b"], relu=False)[..., 0]
        self.a = a
        return a["out"]

    def backward(self, dout):
        """Gradients of every layer (dW, db) for d(loss)/d(out) = dout (after forward)."""
        a, grads = self.a, {}
        dout = self.f32(dout)[..., None]

        def through(name, x, dy, want_dx=True):
            w = self.w[name][0]
            g = self.q(dy * (a[name] > 0))
            grads[name] = conv_wgrad(g, x)
            return self.f32(conv_dgrad(g, w)) if want_dx else None

        grads["out"] = conv_wgrad(dout, a["d0b"])
        d = self.f32(conv_dgrad(dout, self.w["out"][0]))
        d = through("d0b", a["d0a"], d)
        dc0 = through("d0a", a["c0"], d)
        d_e0b = dc0[..., 32:]
        d = self.f32(up_back(dc0[..., :32]))
        d = through("d1b", a["d1a"], d)
        dc1 = through("d1a", a["c1"], d)
        d_e1b = dc1[..., 64:]
        d = self.f32(up_back(dc1[..., :64]))
        d = through("e2a", a["p1"], d)
        d_e1b = self.f32(d_e1b + pool_back(d))
        d = through("e1b", a["e1a"], d_e1b)
        d = through("e1a", a["p0"], d)
        d_e0b = self.f32(d_e0b + pool_back(d))
        d = through("e0b", a["e0a"], d_e0b)
        through("e0a", a["x"], d, want_dx=False)
        return np.concatenate([np.concatenate([grads[n][0].ravel(), grads[n][1].ravel()])
                               for n, _, _, _ in LAYERS])


def mse(out, target):
    """Loss = mean((out - target)^2) and its gradient."""
    d = np.asarray(out, np.float64) - np.asarray(target, np.float64)
    return float(np.mean(d * d)), 2.0 * d / d.size


def adam(flat, grad, m, v, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (bias-corrected), FP32 state; returns (flat, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return flat - lr * mh / (np.sqrt(vh) + eps), m, v


# ---- features and targets of the warm start (padded reference layout) ----

def laplacian(p, dx, dy, dz):
    """Neumann 7-point operator on the interior of a padded array whose ghosts
    mirror the boundary cells (the multigrid's ghost-free operator)."""
    c = p[1:-1, 1:-1, 1:-1]
    pe = np.concatenate([c[:, :, 1:], c[:, :, -1:]], axis=2)
    pw = np.concatenate([c[:, :, :1], c[:, :, :-1]], axis=2)
    pn = np.concatenate([c[:, 1:], c[:, -1:]], axis=1)
    ps = np.concatenate([c[:, :1], c[:, :-1]], axis=1)
    pu = np.concatenate([c[1:], c[-1:]], axis=0)
    pd = np.concatenate([c[:1], c[:-1]], axis=0)
    return (pe + pw - 2 * c) / dx ** 2 + (pn + ps - 2 * c) / dy ** 2 + (pu + pd - 2 * c) / dz ** 2


def restrict(f):
    K, J, I = f.shape
    return f.reshape(K // 2, 2, J // 2, 2, I // 2, 2).mean(axis=(1, 3, 5))


def features(p_warm, rhs, dx, dy, dz):
    """Network input from a solve's start: channel 0 the restricted residual of the
    warm start, channel 1 the restricted mean-free right-hand side, each divided by
    its RMS; returns (x [Z/2][Y/2][X/2][2], sigma = RMS of channel 0 before scaling)."""
    b = rhs[1:-1, 1:-1, 1:-1]
    b = b - b.mean()
    r = restrict(b - laplacian(p_warm, dx, dy, dz))
    rb = restrict(b)
    sr = float(np.sqrt(np.mean(r * r)))
    sb = float(np.sqrt(np.mean(rb * rb)))
    x = np.stack([r / (sr if sr > 0 else 1.0), rb / (sb if sb > 0 else 1.0)], axis=-1)
    return x.astype(np.float32), sr


def kappa(shape, dx, dy, dz):
    """pi^2 (1/Lx^2 + 1/Ly^2 + 1/Lz^2) for the interior shape (K, J, I): the
    scale of the Neumann operator's smallest non-zero eigenvalues."""
    K, J, I = shape
    return np.pi ** 2 * (1.0 / (I * dx) ** 2 + 1.0 / (J * dy) ** 2 + 1.0 / (K * dz) ** 2)


def target(p_warm, p_conv, sigma, dx, dy, dz):
    """Training target: restricted correction p_conv - p_warm in the network's
    units (times kappa, over sigma)."""
    e = p_conv[1:-1, 1:-1, 1:-1] - p_warm[1:-1, 1:-1, 1:-1]
    k = kappa(e.shape, dx, dy, dz)
    return (restrict(e) * k / (sigma if sigma > 0 else 1.0)).astype(np.float32)
