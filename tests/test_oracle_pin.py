"""Pins the CPU oracle: against the golden vectors the reference produced
(everywhere) and bit-for-bit against the reference compiled from source
(where oracle/build_ref.sh could run, i.e. with the reference sources present).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_values, load_golden, rel_err

RUNS = ["cavity8_rb", "ragged_rb", "canal_rb", "bcmix_rb", "mgref_l3", "mgref_l1",
        "cavity_tau0_rb"]


@pytest.mark.parametrize("name", RUNS)
def test_oracle_matches_golden_runs(oracle_mod, name):
    z = load_golden(f"run_{name}.npz")
    vals = golden_values(z)
    run = oracle_mod.OracleRun(vals, str(z["solver"]))
    keep = set(int(k) for k in z["keep"])
    for s in range(1, len(z["it"]) + 1):
        it, res, dt, t = run.step()
        assert it == z["it"][s - 1], f"step {s}: iterations {it} vs {z['it'][s - 1]}"
        assert dt == pytest.approx(z["dt"][s - 1], rel=1e-12)
        assert res == pytest.approx(z["res"][s - 1], rel=1e-9, abs=1e-300)
        if s in keep:
            for f in "uvwp":
                assert rel_err(run.field(f), z[f"{f}_{s}"]) < 1e-11, (name, s, f)


def test_oracle_matches_golden_config1_head(oracle_mod):
    """First 12 steps of the 64^3 cavity: iteration counts, residual and dt."""
    from nusif.params import config1
    z = load_golden("config1_rb.npz")
    assert golden_values(z) == config1()
    run = oracle_mod.OracleRun(config1(), "rb", fast=True)
    for s in range(12):
        it, res, dt, t = run.step()
        assert it == z["it"][s]
        assert dt == pytest.approx(z["dt"][s], rel=1e-12)
        assert res == pytest.approx(z["res"][s], rel=1e-8)


def _kat_grid(oracle_mod, vals):
    return oracle_mod.grid(vals["imax"], vals["jmax"], vals["kmax"], vals["xlength"],
                           vals["ylength"], vals["zlength"])


def test_oracle_matches_golden_operators(oracle_mod):
    o = oracle_mod
    z = load_golden("kat_ops.npz")
    v = golden_values(z)
    g = _kat_grid(o, v)
    dt = float(z["dt_in"])
    fresh = lambda: {f: z[f"in_{f}"].copy() for f in ("u", "v", "w", "p", "rhs", "f", "g", "h")}

    a = fresh()
    dtbound = 0.5 * v["re"] * 1.0 / (1 / g.dx ** 2 + 1 / g.dy ** 2 + 1 / g.dz ** 2)
    assert dtbound == pytest.approx(float(z["dtbound"]), rel=1e-15)
    assert o.op_timestep(g, dtbound, a["u"], a["v"], a["w"], v["tau"]) == pytest.approx(
        float(z["timestep_dt"]), rel=1e-15)

    a = fresh()
    o.op_set_bc(g, [v[k] for k in o.BC_ORDER], a["u"], a["v"], a["w"])
    for f in "uvw":
        np.testing.assert_array_equal(a[f], z[f"bc_out_{f}"])

    a = fresh()
    o.op_special_bc(g, v["name"], a["u"])
    np.testing.assert_array_equal(a["u"], z["special_out_u"])

    a = fresh()
    o.op_fgh(g, v["re"], v["gamma"], v["gx"], v["gy"], v["gz"], dt, a["u"], a["v"], a["w"],
             a["f"], a["g"], a["h"])
    for f in "fgh":
        assert rel_err(a[f], z[f"fg_out_{f}"]) < 1e-14

    a = fresh()
    o.op_rhs(g, dt, a["f"], a["g"], a["h"], a["rhs"])
    assert rel_err(a["rhs"], z["rhs_out_rhs"]) < 1e-14

    a = fresh()
    o.op_normalize(g, a["p"])
    assert rel_err(a["p"], z["normalize_out_p"]) < 1e-14

    a = fresh()
    o.op_adapt(g, dt, a["f"], a["g"], a["h"], a["p"], a["u"], a["v"], a["w"])
    for f in "uvw":
        assert rel_err(a[f], z[f"adapt_out_{f}"]) < 1e-14

    a = fresh()
    it, res = o.op_solve_rb(g, v["eps"], v["omg"], v["itermax"], a["p"], a["rhs"])
    assert it == int(z["solve_it"])
    assert res == pytest.approx(float(z["solve_res"]), rel=1e-12)
    assert rel_err(a["p"], z["solve_out_p"]) < 1e-13


@pytest.mark.skipif("not __import__('oracle').ref_available('rb')",
                    reason="reference not compiled here (oracle/build_ref.sh)")
@pytest.mark.parametrize("solver", ["rb", "mg-ref"])
@pytest.mark.parametrize("case", [
    dict(n=8, te=1e9, omg=1.7, eps=1e-3, itermax=200, levels=3, presmooth=5, postsmooth=3),
    dict(n=(17, 9, 13), te=1e9, itermax=300, levels=1, presmooth=4),
    dict(n=(5, 6, 7), te=1e9, bcLeft=2, bcTop=3, bcBack=2, bcFront=4, gz=0.3, itermax=80,
         levels=2, presmooth=2, postsmooth=1),
])
def test_oracle_bitwise_vs_reference(oracle_mod, tmp_path, solver, case):
    """Strict builds of both: every field and scalar identical for 8 steps."""
    from nusif.params import cavity, write_par
    case = dict(case)
    vals = cavity(case.pop("n"), **case)
    par = write_par(tmp_path / "c.par", vals)
    ref = oracle_mod.RefDriver(par, solver)
    run = oracle_mod.OracleRun(vals, solver)
    for s in range(8):
        assert ref.step() == run.step()
        for f in ("u", "v", "w", "p", "rhs", "f", "g", "h"):
            np.testing.assert_array_equal(ref.field(f), run.field(f), err_msg=f"{f} step {s}")
