"""The learned warm start inside the multigrid solve: features and targets
against the oracle's definitions, the fallback to the plain warm start, and
what a trained network gains over the method without it."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu


def _prepare(sim):
    """The step up to the solve (reference order)."""
    sim.compute_timestep()
    sim.set_boundary_conditions()
    sim.set_special_boundary_condition()
    sim.compute_fg()
    sim.compute_rhs()


def test_features_and_target_match_oracle(nusif_lib):
    import torch
    from nusif import Simulation
    from nusif.params import cavity
    n = 16
    with Simulation(cavity(n, re=500.0, te=1e9, solver="mg", rtol=1e-8)) as sim:
        for _ in range(3):
            sim.step()
        _prepare(sim)
        p0, rhs = sim.field("p"), sim.field("rhs")
        x = torch.zeros((n // 2,) * 3 + (2,), dtype=torch.float32, device="cuda")
        t = torch.zeros((n // 2,) * 3, dtype=torch.float32, device="cuda")
        sim.record_pair(x, t)
        sim.solve()
        pstar = sim.field("p")
        h = 1.0 / n
        xr, sigma = U.features(p0, rhs, h, h, h)
        tr = U.target(p0, pstar, sigma, h, h, h)
        np.testing.assert_allclose(x.cpu().numpy(), xr, rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(t.cpu().numpy(), tr, rtol=1e-4, atol=1e-4 * np.abs(tr).max())


@pytest.mark.parametrize("solver", ["mg", "mg-mixed"])
def test_rejected_guess_leaves_the_solve_unchanged(nusif_lib, solver):
    """A network with zero output layer proposes p1 = p0 (never smaller
    residual): it is rejected every step and the run is bit-identical to the
    run without a network."""
    from nusif import Simulation, UNet
    from nusif.params import cavity
    vals = cavity(16, re=800.0, te=1e9, solver=solver, rtol=1e-7)
    with UNet(seed=2) as net:
        p = net.params()
        p[-(27 * 16 + 1):] = 0.0  # output layer weights and bias
        net.set_params(p)
        with Simulation(vals) as a, Simulation(vals) as b:
            b.set_guess_net(net)
            for _ in range(5):
                ia, ib = a.step(), b.step()
                used, rw, rg = b.guess_stats()
                assert not used and rg == rw
                assert ia.it == ib.it
            for f in "uvwp":
                np.testing.assert_array_equal(a.field(f), b.field(f))


def test_guess_is_taken_only_when_better(nusif_lib):
    """An untrained network: whatever it proposes, the solve starts from the
    smaller of the two residuals and still ends at rtol."""
    from nusif import Simulation, UNet
    from nusif.params import cavity
    with UNet(seed=3) as net, Simulation(cavity(16, re=300.0, te=1e9, solver="mg-mixed",
                                                rtol=1e-6)) as sim:
        sim.set_guess_net(net)
        for _ in range(4):
            info = sim.step()
            used, rw, rg = sim.guess_stats()
            assert used == (rg < rw)  # restricted residuals, the decision criterion
            assert info.res <= 1e-6


@pytest.mark.parametrize("guess", ["extrapolate", "previous"])
def test_trained_guess_gains(nusif_lib, guess):
    """End to end on 32^3 cavities: pairs recorded by the solver, a short
    training, then a cavity at an unseen Re and lid speed (same resolution).
    What the trained network gains over the plain warm start: its guess is
    taken in most steps and cuts the restricted residual that the V-cycles
    pay for; the run never needs more V-cycles than without it. (The gain is
    well below the 10x that one V-cycle buys, so the cycle count itself does
    not drop at these sizes; bench.py --workload learned reports it.)"""
    from nusif import Simulation, UNet
    from nusif.learn import generate_pairs, train, training_cases
    from nusif.params import cavity
    cases = training_cases(6, 32, seed=42, guess=guess)
    data = generate_pairs(cases, steps=66, every=3, skip=6)
    with UNet(seed=0) as net:
        log = train(net, data, iters=600, batch=8, lr=1e-3, log_every=100)
        assert log[-1][1] < 0.1 * log[0][1], log
        vals = cavity(32, re=2750.0, lid=1.25, te=1e9, tau=0.5, solver="mg-mixed", rtol=1e-6,
                      mg_guess=guess)
        cyc = {}
        ratio = []
        taken = 0
        for use in (False, True):
            with Simulation(vals) as sim:
                if use:
                    sim.set_guess_net(net)
                its = []
                for s in range(40):
                    info = sim.step()
                    assert info.res <= 1e-6
                    its.append(info.it)
                    if use and s >= 5:
                        used, rw, rg = sim.guess_stats()
                        taken += used
                        ratio.append(rg / rw)
                cyc[use] = sum(its[5:])
    assert taken >= 20, (taken, ratio)
    assert np.median(ratio) < 0.9, ratio
    assert cyc[True] <= cyc[False], cyc


def test_probe_backs_off_after_rejections(nusif_lib):
    """mg_probe 4: a network whose guess always loses runs in steps 1 and 2,
    then - after two rejections in a row - only every 4th step (6 and 10 of
    12); in between the plain warm start is used, so the run stays
    bit-identical to one without a network."""
    from nusif import Simulation, UNet
    from nusif.params import cavity
    vals = cavity(16, re=800.0, te=1e9, solver="mg-mixed", rtol=1e-7, mg_probe=4)
    with UNet(seed=2) as net:
        p = net.params()
        p[-(27 * 16 + 1):] = 0.0  # output layer weights and bias: p1 = p0, never better
        net.set_params(p)
        with Simulation(vals) as a, Simulation(vals) as b:
            b.set_guess_net(net)
            for _ in range(12):
                ia, ib = a.step(), b.step()
                assert ia.it == ib.it
            assert b.guess_counts() == (4, 0)
            for f in "uvwp":
                np.testing.assert_array_equal(a.field(f), b.field(f))
