"""Drop-in parity at the benchmark configuration: the 256^3 lid-driven cavity
(Re 1000, tau 0.5, gamma 0.9).

- Red-black SOR (omega 1.7, eps 1e-6, itermax 10000): the first two time
  steps against the reference itself (tests/golden/config2_rb.npz, made by
  tests/golden/make_golden.py --config2 from the reference compiled from
  source). Bar: identical iteration counts, dt to 1e-10, the carried residual
  to 1e-8, fields within 1e-10 relative on a stride-9 lattice of the padded
  array (ghosts included) and in whole-interior sums.
- The reference's multigrid build (6 levels, 2 + 2 sweeps): three steps
  against config2_mgref.npz, same field bar.
- The corrected FP64 V-cycle solve of a real step's right-hand side (step 3 of
  the benchmark case) against the CPU restatement oracle/nusif_oracle_mg.c:
  identical cycle counts, pressure within 1e-10.
- The mixed-precision solve of the same right-hand side against the oracle's
  FP64 solve to 1e-9: the true FP64 residual below rtol = 1e-6 and the
  mean-free pressure within 1e-5 of the solution's magnitude. A residual of
  1e-6 bounds the pressure error only up to the operator's conditioning: on
  this system the oracle's own FP64 solve stopped at 1e-6 is 1.4e-6 away from
  the 1e-9 solution, its mixed solve 1.7e-6.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_values, load_golden, rel_err
from test_oracle_mg import neumann_residual

pytestmark = pytest.mark.gpu

N = 256


def _check_golden_steps(z, solver: str, steps: int, it_exact: bool) -> None:
    from nusif import Simulation
    vals = dict(golden_values(z), solver=solver)
    stride = int(z["stride"])
    sl = (slice(0, None, stride),) * 3
    with Simulation(vals) as sim:
        for s in range(1, steps + 1):
            info = sim.step()
            if it_exact:
                assert info.it == int(z["it"][s - 1]), f"step {s}: iterations"
            assert info.dt == pytest.approx(float(z["dt"][s - 1]), rel=1e-10)
            assert info.res == pytest.approx(float(z["res"][s - 1]), rel=1e-8)
            for f in "uvwp":
                a = sim.field(f)
                assert rel_err(a[sl], z[f"{f}_sample_{s}"]) < 1e-10, (s, f)
                inner = a[1:-1, 1:-1, 1:-1]
                sumsq = float(z[f"{f}_sumsq_{s}"])
                assert float(inner.sum()) == pytest.approx(
                    float(z[f"{f}_sum_{s}"]), rel=1e-10, abs=1e-10 * np.sqrt(sumsq) * N ** 1.5)
                assert float((inner * inner).sum()) == pytest.approx(sumsq, rel=1e-10)


def test_config2_red_black_steps_match_reference(nusif_lib):
    """Two time steps of 10000 red-black iterations each (the reference's
    residual stays above eps^2) against the reference's own output."""
    z = load_golden("config2_rb.npz")
    assert list(z["it"]) == [10000, 10000]
    _check_golden_steps(z, "rb", len(z["it"]), it_exact=True)


def test_config2_reference_multigrid_steps_match_reference(nusif_lib):
    z = load_golden("config2_mgref.npz")
    _check_golden_steps(z, "mg-ref", len(z["res"]), it_exact=False)


@pytest.fixture(scope="module")
def step3_system(nusif_lib):
    """p (the previous step's pressure) and rhs of the benchmark case's third
    time step, stepped with FP64 multigrid: the system one solve of the
    benchmark sees."""
    from nusif import Simulation
    from nusif.params import config2
    with Simulation(config2(solver="mg")) as sim:
        for _ in range(2):
            sim.step()
        sim.compute_timestep()
        sim.set_boundary_conditions()
        sim.set_special_boundary_condition()
        sim.compute_fg()
        sim.compute_rhs()
        g = sim.d.grid
        return {"p": sim.field("p"), "rhs": sim.field("rhs"),
                "h": (g.dx, g.dy, g.dz), "len": (g.xlength, g.ylength, g.zlength)}


def _solve_gpu(solver: str, system: dict, rtol: float, **over):
    from nusif import Simulation
    from nusif.params import config2
    with Simulation(config2(solver=solver, rtol=rtol, mg_cycles=60, **over)) as sim:
        sim.set_field("p", system["p"])
        sim.set_field("rhs", system["rhs"])
        rel = sim.solve()
        return rel, sim.iterations, sim.field("p")


def test_fp64_multigrid_at_256_matches_oracle(step3_system, oracle_mod):
    o = oracle_mod
    rtol = 1e-6
    rel, cyc, p = _solve_gpu("mg", step3_system, rtol)
    og = o.grid(N, N, N, *step3_system["len"])
    pc = step3_system["p"].copy()
    cyc_c, rel_c = o.op_mg_solve(og, "mg", pc, step3_system["rhs"].copy(), rtol=rtol,
                                 maxcycles=60)
    assert cyc == cyc_c and cyc_c < 60
    assert rel == pytest.approx(rel_c, rel=1e-6)
    assert rel_err(p[1:-1, 1:-1, 1:-1], pc[1:-1, 1:-1, 1:-1]) < 1e-10
    assert neumann_residual(p, step3_system["rhs"], step3_system["h"]) <= rtol * 1.001


def test_mixed_multigrid_at_256_matches_oracle_fp64(step3_system, oracle_mod):
    """The benchmark's mixed-precision shape (V(1,1), omega 1.3, at most 4 FP32
    cycles per FP64 residual) against the oracle's FP64 V-cycle solution."""
    o = oracle_mod
    rtol = 1e-6
    rel, cyc, p = _solve_gpu("mg-mixed", step3_system, rtol, mg_pre=1, mg_post=1,
                             mg_inner=4, mg_omega=1.3)
    assert rel <= rtol and cyc < 60
    assert neumann_residual(p, step3_system["rhs"], step3_system["h"]) <= rtol * 1.001
    og = o.grid(N, N, N, *step3_system["len"])
    p64 = step3_system["p"].copy()
    cyc_c, _ = o.op_mg_solve(og, "mg", p64, step3_system["rhs"].copy(), rtol=1e-9,
                             maxcycles=60)
    assert cyc_c < 60
    a = p[1:-1, 1:-1, 1:-1]
    b = p64[1:-1, 1:-1, 1:-1]
    a, b = a - a.mean(), b - b.mean()
    assert np.max(np.abs(a - b)) <= 1e-5 * np.max(np.abs(b))
