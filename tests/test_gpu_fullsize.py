"""Parity at the benchmark's full size (256^3, the lid-driven cavity at Re 1000):
the heaviest operators and a short red-black solve against the oracle on the
same inputs, and size-independent properties of whole mixed-precision steps
(the true residual of the returned pressure, the discrete divergence left by
the projection, agreement with FP64 multigrid)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from test_oracle_mg import neumann_residual

pytestmark = pytest.mark.gpu

N = 256


def _vals(solver="rb", **over):
    from nusif.params import config2
    v = config2(solver=solver)
    v.update(imax=N, jmax=N, kmax=N)
    v.update(over)
    return v


@pytest.mark.parametrize("arith", ["df32", "fp64"])
def test_operators_at_256_match_oracle(nusif_lib, oracle_mod, arith):
    from nusif import Simulation
    o = oracle_mod
    v = _vals(fg_arith=arith)
    rng = np.random.default_rng(2561)
    with Simulation(v) as sim:
        shape = sim.padded_shape
        g = o.grid(N, N, N, v["xlength"], v["ylength"], v["zlength"])
        u, w3, w = (0.5 * rng.standard_normal(shape) for _ in range(3))
        for f, a in (("u", u), ("v", w3), ("w", w)):
            sim.set_field(f, a)
        dt = 0.004
        sim.d.dt = dt
        sim.compute_fg()
        f, gg, h = (np.zeros(shape) for _ in range(3))
        o.op_fgh(g, v["re"], v["gamma"], v["gx"], v["gy"], v["gz"], dt, u.copy(), w3.copy(),
                 w.copy(), f, gg, h)
        for name, ref in (("f", f), ("g", gg), ("h", h)):
            assert rel_err(sim.field(name), ref) < 1e-13, name
        sim.compute_rhs()
        rhs = np.zeros(shape)
        o.op_rhs(g, dt, f, gg, h, rhs)
        assert rel_err(sim.field("rhs"), rhs) < 1e-13
        p = rng.standard_normal(shape)
        sim.set_field("p", p)
        sim.adapt_uv()
        uu, vv, ww = u.copy(), w3.copy(), w.copy()
        o.op_adapt(g, dt, f, gg, h, p, uu, vv, ww)
        for name, ref in (("u", uu), ("v", vv), ("w", ww)):
            assert rel_err(sim.field(name), ref) < 1e-13, name


@pytest.mark.parametrize("arith", ["df32", "fp64"])
def test_red_black_at_256_matches_oracle(nusif_lib, oracle_mod, arith):
    """Twelve red-black SOR iterations at 256^3 (residual in FP32 pairs and in
    FP64 instructions): the reference's carried residual and the pressure
    agree with the oracle."""
    from nusif import Simulation
    o = oracle_mod
    v = _vals(itermax=12, eps=1e-30, arith=arith)
    rng = np.random.default_rng(2562)
    with Simulation(v) as sim:
        g = o.grid(N, N, N, v["xlength"], v["ylength"], v["zlength"])
        p = rng.standard_normal(sim.padded_shape)
        rhs = rng.standard_normal(sim.padded_shape)
        sim.set_field("p", p)
        sim.set_field("rhs", rhs)
        res = sim.solve()
        it, res_c = o.op_solve_rb(g, v["eps"], v["omg"], v["itermax"], p, rhs)
        assert sim.iterations == it == 12
        assert res == pytest.approx(res_c, rel=1e-11)
        assert rel_err(sim.field("p"), p) < 1e-11


def _divergence(sim):
    g = sim.d.grid
    u, v, w = (sim.field(f) for f in "uvw")
    return ((u[1:-1, 1:-1, 1:-1] - u[1:-1, 1:-1, :-2]) / g.dx +
            (v[1:-1, 1:-1, 1:-1] - v[1:-1, :-2, 1:-1]) / g.dy +
            (w[1:-1, 1:-1, 1:-1] - w[:-2, 1:-1, 1:-1]) / g.dz)


def test_mixed_steps_at_256_properties(nusif_lib):
    """Four steps of the benchmark case with mixed-precision multigrid and the
    quadratic warm start: the pressure's true residual (numpy, FP64) is below
    1e-6 of the mean-free right-hand side; the projection leaves the discrete
    divergence div u = dt (s + r), s the rhs mean, r the residual; and the
    velocities agree with FP64 multigrid to the solver tolerance."""
    from nusif import Simulation
    runs = {}
    for solver in ("mg-mixed", "mg"):
        with Simulation(_vals(solver, mg_guess="quadratic")) as sim:
            for _ in range(4):
                info = sim.step()
                assert info.res <= 1e-6
            g = sim.d.grid
            p, rhs = sim.field("p"), sim.field("rhs")
            rel = neumann_residual(p, rhs, (g.dx, g.dy, g.dz))
            assert rel <= 1e-6 * 1.001, (solver, rel)
            b = rhs[1:-1, 1:-1, 1:-1]
            s = b.mean()
            div = _divergence(sim)
            dt = sim.dt
            assert np.linalg.norm(div - dt * s) <= 1.01e-6 * dt * np.linalg.norm(b - s) + 1e-12
            runs[solver] = {f: sim.field(f) for f in "uvw"}
    for f in "uvw":
        assert rel_err(runs["mg-mixed"][f], runs["mg"][f]) < 1e-5, f
