"""Whole-run parity of the CUDA library against the reference's golden runs
and against the CPU oracle.

The bar: identical solver iteration counts every step, fields within 1e-10
relative every step, and final u, v, w, p within 1e-8 after the 64^3 cavity
run (Re 1000, tau 0.5, t_end 1.0, red-black SOR omega 1.7, eps 1e-3,
itermax 500: 235 steps, 82,285 iterations in the reference).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_values, load_golden, rel_err

pytestmark = pytest.mark.gpu

RUNS = ["cavity8_rb", "ragged_rb", "canal_rb", "bcmix_rb", "mgref_l3", "mgref_l1",
        "cavity_tau0_rb"]


def _vals_with_solver(vals, solver):
    v = dict(vals)
    v["solver"] = solver
    return v


@pytest.mark.parametrize("name", RUNS)
def test_golden_run(nusif_lib, name):
    from nusif import Simulation
    z = load_golden(f"run_{name}.npz")
    vals = _vals_with_solver(golden_values(z), str(z["solver"]))
    keep = set(int(k) for k in z["keep"])
    with Simulation(vals) as sim:
        for s in range(1, len(z["it"]) + 1):
            info = sim.step()
            assert info.it == z["it"][s - 1], f"step {s}"
            assert info.dt == pytest.approx(z["dt"][s - 1], rel=1e-10)
            assert info.res == pytest.approx(z["res"][s - 1], rel=1e-8, abs=1e-300)
            if s in keep:
                for f in "uvwp":
                    assert rel_err(sim.field(f), z[f"{f}_{s}"]) < 1e-10, (s, f)


def test_config1_full_run_matches_reference(nusif_lib):
    """The whole 64^3 cavity: per-step iteration counts exact, dt and residual
    close, final fields (sampled every 4th cell, plus whole-field sums) to 1e-8."""
    from nusif import Simulation, config1
    z = load_golden("config1_rb.npz")
    with Simulation(config1()) as sim:
        infos = sim.run()
        its = np.array([i.it for i in infos])
        assert len(infos) == len(z["it"])
        mism = np.nonzero(its != z["it"])[0]
        assert mism.size == 0, f"iteration counts differ at steps {mism[:10]}"
        np.testing.assert_allclose([i.dt for i in infos], z["dt"], rtol=1e-9)
        np.testing.assert_allclose([i.res for i in infos], z["res"], rtol=1e-6)
        assert sim.t == pytest.approx(float(z["t_end"]), rel=1e-12)
        sl = (slice(1, -1, 4),) * 3
        for f in "uvwp":
            a = sim.field(f)
            assert rel_err(a[sl], z[f"{f}_sample"]) < 1e-8, f
            inner = a[1:-1, 1:-1, 1:-1]
            assert float(inner.sum()) == pytest.approx(float(z[f"{f}_sum"]), rel=1e-8,
                                                       abs=1e-8 * np.sqrt(float(z[f"{f}_sumsq"])))
            assert float((inner * inner).sum()) == pytest.approx(float(z[f"{f}_sumsq"]),
                                                                 rel=1e-8)


@pytest.mark.parametrize("solver", ["rb", "mg-ref"])
def test_run_matches_oracle_every_step(nusif_lib, oracle_mod, solver):
    """A 24^3 cavity for 20 steps: fields within 1e-10 after every step."""
    from nusif import Simulation
    from nusif.params import cavity
    vals = cavity(24, te=1e9, omg=1.7, eps=1e-4, itermax=400, levels=2, presmooth=8,
                  postsmooth=4, solver=solver)
    run = oracle_mod.OracleRun(vals, solver)
    with Simulation(vals) as sim:
        for s in range(20):
            a = sim.step()
            it, res, dt, t = run.step()
            assert a.it == it
            assert a.dt == pytest.approx(dt, rel=1e-10)
            for f in "uvwp":
                assert rel_err(sim.field(f), run.field(f)) < 1e-10, (s, f)
