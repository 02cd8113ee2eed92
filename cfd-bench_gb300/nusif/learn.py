"""Training data and training loop of the learned pressure warm start.

The solver generates its own data: while a cavity runs, every `every`-th
solve records its pair (features of its warm start, restricted correction
to the converged pressure) straight into device memory (nusifSolverRecordPair).
The network then trains on random batches of those pairs with the library's
own forward / backward / Adam kernels (nusifUNetTrainStep). torch only holds
the device buffers.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from .params import cavity
from .sim import Simulation
from .unet import UNet


def splitmix64(seed: int):
    """Project PRNG for the case draws (seeded, platform independent)."""
    s = seed & 0xFFFFFFFFFFFFFFFF
    while True:
        s = (s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        yield (z ^ (z >> 31)) / 2.0 ** 64


def training_cases(runs: int, n: int, seed: int, solver: str = "mg-mixed",
                   guess: str = "extrapolate") -> list[dict]:
    """Lid-driven cavities at n^3 with Re ~ U[100, 5000] and lid ~ U[0.5, 2.0];
    `guess` is the plain warm start the network learns to improve on."""
    g = splitmix64(seed)
    out = []
    for _ in range(runs):
        re = 100.0 + 4900.0 * next(g)
        lid = 0.5 + 1.5 * next(g)
        out.append(cavity(n, re=re, lid=lid, te=1e9, tau=0.5, gamma=0.9, solver=solver,
                          rtol=1e-6, mg_guess=guess))
    return out


@dataclass
class PairSet:
    x: object      # torch float32 [S][Z][Y][X][2] (device)
    t: object      # torch float32 [S][Z][Y][X] (device)
    seconds: float


def generate_pairs(cases: list[dict], steps: int, every: int, device: str = "cuda",
                   skip: int = 0) -> PairSet:
    """Run every case `steps` time steps; every `every`-th solve from step
    `skip` on (the start-up transient from rest excluded) records one pair."""
    import torch
    per_run = (max(steps - skip, 0) + every - 1) // every
    i, j, k = cases[0]["imax"], cases[0]["jmax"], cases[0]["kmax"]
    S = per_run * len(cases)
    x = torch.empty((S, k // 2, j // 2, i // 2, 2), dtype=torch.float32, device=device)
    t = torch.empty((S, k // 2, j // 2, i // 2), dtype=torch.float32, device=device)
    t0 = time.perf_counter()
    s = 0
    for vals in cases:
        with Simulation(vals) as sim:
            for q in range(steps):
                if q >= skip and (q - skip) % every == 0:
                    sim.record_pair(x[s], t[s])
                    s += 1
                sim.step()
    torch.cuda.synchronize()
    return PairSet(x[:s], t[:s], time.perf_counter() - t0)


def train(net: UNet, data: PairSet, iters: int, batch: int = 8, lr: float = 1e-3,
          seed: int = 0, log_every: int = 0, lr_final: float | None = None
          ) -> list[tuple[int, float]]:
    """Adam on random batches of the pairs, the learning rate decaying on a
    cosine from lr to lr_final (default lr / 10); returns (iteration, loss)
    samples."""
    import math

    import torch
    lr_final = lr / 10 if lr_final is None else lr_final
    rng = np.random.default_rng(seed)
    S = data.x.shape[0]
    xb = torch.empty((batch,) + tuple(data.x.shape[1:]), dtype=torch.float32, device=data.x.device)
    tb = torch.empty((batch,) + tuple(data.t.shape[1:]), dtype=torch.float32, device=data.t.device)
    losses = []
    for it in range(iters):
        idx = torch.from_numpy(rng.integers(0, S, batch)).to(data.x.device)
        torch.index_select(data.x, 0, idx, out=xb)
        torch.index_select(data.t, 0, idx, out=tb)
        want = log_every and (it % log_every == 0 or it == iters - 1)
        lr_it = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * it / max(iters - 1, 1)))
        loss = net.train_step(xb, tb, lr=lr_it, update=True, want_loss=bool(want))
        if want:
            losses.append((it, loss))
    return losses


def validation_loss(net: UNet, data: PairSet) -> float:
    """Mean loss over the pairs without updating the network."""
    total = 0.0
    for s in range(data.x.shape[0]):
        total += net.train_step(data.x[s:s + 1], data.t[s:s + 1], update=False)
    return total / data.x.shape[0]


def save_params(net: UNet, path, meta: dict | None = None) -> None:
    """The network's FP32 parameters (flat, the C ABI's layout) and a
    description of how they were trained, as a compressed .npz file."""
    import json
    from pathlib import Path
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(path, params=net.params(), meta=np.array(json.dumps(meta or {})))


def load_net(path, seed: int = 0) -> UNet:
    """A network with the parameters saved by save_params."""
    z = np.load(path, allow_pickle=False)
    net = UNet(seed=seed)
    net.set_params(z["params"])
    return net


def saved_meta(path) -> dict:
    import json
    return json.loads(str(np.load(path, allow_pickle=False)["meta"]))
