"""The CPU restatement of the corrected multigrid (no reference counterpart:
the reference's multigrid never applies its coarse-grid correction). Pinned
by properties instead: the level hierarchy of the benchmark grids, the
reported residual equals an independent numpy residual, and the solution
agrees with the converged red-black solution of the same right-hand side."""
from __future__ import annotations

import numpy as np
import pytest


def neumann_residual(p: np.ndarray, rhs: np.ndarray, h) -> float:
    """||b - A p|| / ||b|| with b = rhs - mean(rhs), ghost-free Neumann walls (numpy)."""
    x = p[1:-1, 1:-1, 1:-1]
    b = rhs[1:-1, 1:-1, 1:-1]
    b = b - b.mean()
    xp = np.pad(x, 1, mode="edge")  # a neighbour outside the domain is the cell itself
    hx, hy, hz = h
    lap = ((xp[1:-1, 1:-1, 2:] + xp[1:-1, 1:-1, :-2] - 2 * x) / hx ** 2 +
           (xp[1:-1, 2:, 1:-1] + xp[1:-1, :-2, 1:-1] - 2 * x) / hy ** 2 +
           (xp[2:, 1:-1, 1:-1] + xp[:-2, 1:-1, 1:-1] - 2 * x) / hz ** 2)
    return float(np.linalg.norm(b - lap) / np.linalg.norm(b))


def test_level_hierarchies(oracle_mod):
    o = oracle_mod
    assert o.op_mg_levels(o.grid(256, 256, 256)) == [(256,) * 3, (128,) * 3, (64,) * 3, (32,) * 3,
                                                    (16,) * 3, (8,) * 3]
    ch = o.op_mg_levels(o.grid(512, 128, 128, 4.0, 1.0, 1.0))
    assert ch[0] == (512, 128, 128) and ch[-1] == (8, 8, 8) and len(ch) == 7
    assert o.op_mg_levels(o.grid(17, 9, 13)) == [(17, 9, 13)]
    assert len(o.op_mg_levels(o.grid(64, 64, 64), cap=2)) == 2


@pytest.mark.parametrize("mode", ["mg", "mg-mixed"])
@pytest.mark.parametrize("dims", [(32, 32, 32), (32, 16, 48)])
def test_reported_residual_is_true_residual(oracle_mod, mode, dims):
    o = oracle_mod
    g = o.grid(*dims, 1.0, 0.7, 1.3)
    rng = np.random.default_rng(3)
    shape = (dims[2] + 2, dims[1] + 2, dims[0] + 2)
    rhs = rng.standard_normal(shape)
    p = rng.standard_normal(shape)
    cyc, rel = o.op_mg_solve(g, mode, p, rhs, rtol=1e-8)
    assert rel <= 1e-8
    assert 1 <= cyc < 30
    assert neumann_residual(p, rhs, (g.dx, g.dy, g.dz)) == pytest.approx(rel, rel=1e-3)
    # ghosts refreshed: Neumann copies of the boundary cells
    np.testing.assert_array_equal(p[0, 1:-1, 1:-1], p[1, 1:-1, 1:-1])
    np.testing.assert_array_equal(p[1:-1, 1:-1, -1], p[1:-1, 1:-1, -2])


def test_mg_agrees_with_converged_red_black(oracle_mod):
    """Same Neumann problem: the V-cycle solution equals the red-black one up to a constant."""
    o = oracle_mod
    n = 16
    g = o.grid(n, n, n)
    rng = np.random.default_rng(5)
    shape = (n + 2,) * 3
    rhs = rng.standard_normal(shape)
    rhs[1:-1, 1:-1, 1:-1] -= rhs[1:-1, 1:-1, 1:-1].mean()
    p_mg = np.zeros(shape)
    o.op_mg_solve(g, "mg", p_mg, rhs, rtol=1e-12)
    p_rb = np.zeros(shape)
    o.op_solve_rb(g, 1e-15, 1.9, 20000, p_rb, rhs)
    a = p_mg[1:-1, 1:-1, 1:-1] - p_mg[1:-1, 1:-1, 1:-1].mean()
    b = p_rb[1:-1, 1:-1, 1:-1] - p_rb[1:-1, 1:-1, 1:-1].mean()
    assert np.max(np.abs(a - b)) < 1e-9 * np.max(np.abs(b))


def test_mixed_agrees_with_fp64(oracle_mod):
    o = oracle_mod
    n = 32
    g = o.grid(n, n, n)
    rng = np.random.default_rng(9)
    shape = (n + 2,) * 3
    rhs = rng.standard_normal(shape)
    p0 = rng.standard_normal(shape)
    pa, pb = p0.copy(), p0.copy()
    o.op_mg_solve(g, "mg", pa, rhs, rtol=1e-10)
    ca, ra = o.op_mg_solve(g, "mg-mixed", pb, rhs, rtol=1e-10)
    assert ra <= 1e-10
    a = pa[1:-1, 1:-1, 1:-1] - pa[1:-1, 1:-1, 1:-1].mean()
    b = pb[1:-1, 1:-1, 1:-1] - pb[1:-1, 1:-1, 1:-1].mean()
    assert np.max(np.abs(a - b)) < 1e-7 * np.max(np.abs(a))
