"""GPU multigrid solvers ("mg": FP64 V-cycles, "mg-mixed": FP32 V-cycles in
FP64 iterative refinement) against their CPU restatement
(oracle/nusif_oracle_mg.c) and against an independent numpy residual.

Tolerances: FP64 V-cycles must use the same number of cycles as the oracle
and give the pressure to 1e-10 of its magnitude (FMA and reduction order
only). FP32 arithmetic on the GPU rounds differently from the CPU's FP32, so
mixed precision is held to the stop criterion itself: the true residual of
the returned pressure is below rtol, the cycle count is within one of the
oracle's, and the pressure agrees with the FP64 solution to 1e-6 of its
magnitude after the Neumann null space (the mean) is removed.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from test_oracle_mg import neumann_residual

pytestmark = pytest.mark.gpu

DIMS = [(16, 16, 16), (32, 32, 32), (64, 32, 16), (48, 16, 32), (33, 17, 9), (8, 8, 8)]


def _sim(dims, solver, rtol, **over):
    from nusif import Simulation
    from nusif.params import cavity
    vals = cavity(dims, xlength=1.0, ylength=0.8, zlength=1.2, te=1e9, solver=solver,
                  rtol=rtol, **over)
    return Simulation(vals)


def _interior_demeaned(p):
    a = p[1:-1, 1:-1, 1:-1]
    return a - a.mean()


@pytest.mark.parametrize("dims", DIMS)
def test_mg_fp64_matches_oracle(nusif_lib, oracle_mod, dims):
    o = oracle_mod
    rng = np.random.default_rng(17)
    rtol = 1e-9
    with _sim(dims, "mg", rtol, mg_cycles=60) as sim:
        g = sim.d.grid
        og = o.grid(*dims, g.xlength, g.ylength, g.zlength)
        p0 = rng.standard_normal(sim.padded_shape)
        rhs = rng.standard_normal(sim.padded_shape)
        sim.set_field("p", p0)
        sim.set_field("rhs", rhs)
        rel = sim.solve()
        cyc = sim.iterations
        pc = p0.copy()
        cyc_c, rel_c = o.op_mg_solve(og, "mg", pc, rhs, rtol=rtol, maxcycles=60)
        assert cyc == cyc_c
        assert rel == pytest.approx(rel_c, rel=1e-6)
        p = sim.field("p")
        assert rel_err(p[1:-1, 1:-1, 1:-1], pc[1:-1, 1:-1, 1:-1]) < 1e-10
        assert neumann_residual(p, rhs, (g.dx, g.dy, g.dz)) == pytest.approx(rel, rel=1e-3)
        np.testing.assert_array_equal(sim.field("rhs"), rhs)
        np.testing.assert_array_equal(p[0, 1:-1, 1:-1], p[1, 1:-1, 1:-1])


@pytest.mark.parametrize("dims", DIMS)
def test_mg_mixed_matches_oracle(nusif_lib, oracle_mod, dims):
    o = oracle_mod
    rng = np.random.default_rng(23)
    rtol = 1e-8
    with _sim(dims, "mg-mixed", rtol, mg_cycles=60) as sim:
        g = sim.d.grid
        og = o.grid(*dims, g.xlength, g.ylength, g.zlength)
        p0 = rng.standard_normal(sim.padded_shape)
        rhs = rng.standard_normal(sim.padded_shape)
        sim.set_field("p", p0)
        sim.set_field("rhs", rhs)
        rel = sim.solve()
        cyc = sim.iterations
        p = sim.field("p")
        true_rel = neumann_residual(p, rhs, (g.dx, g.dy, g.dz))
        pc = p0.copy()
        cyc_c, rel_c = o.op_mg_solve(og, "mg-mixed", pc, rhs, rtol=rtol, maxcycles=60)
        p64 = p0.copy()
        o.op_mg_solve(og, "mg", p64, rhs, rtol=rtol, maxcycles=60)
        if cyc_c < 60:
            assert rel <= rtol
            assert true_rel <= rtol * 1.001
            assert abs(cyc - cyc_c) <= 1
            a, b = _interior_demeaned(p), _interior_demeaned(p64)
            assert np.max(np.abs(a - b)) <= 1e-6 * np.max(np.abs(b))
        else:  # not converging in the cap (no coarsening possible): same cap reached
            assert cyc == cyc_c
        assert true_rel == pytest.approx(rel, rel=1e-3)


@pytest.mark.parametrize("dims", [(64, 32, 16), (33, 17, 9), (40, 24, 20)])
def test_mixed_residual_in_pairs_matches_fp64(nusif_lib, oracle_mod, dims):
    """The mixed solver's fine residual in FP32 pairs (key arith df32, the
    default) against the FP64-instruction kernel (arith fp64). rtol 1e30
    stops every solve after its first residual, so solve() returns ||b - A p||
    / ||b|| of the given p: a random p (no cancellation: 1e-12 relative) and
    the oracle's FP64 solution to 1e-9, where b - A p cancels down to 1e-9 of
    ||b|| and the pair arithmetic's error (a few 2^-47 diag |p|) must stay
    below 2% of the norm, 1e-11 of ||b|| -- three orders under the rtol of
    every benchmark case (1e-6, 1e-8)."""
    o = oracle_mod
    rng = np.random.default_rng(29)
    rhs = None
    rels = {}
    for arith in ("df32", "fp64"):
        with _sim(dims, "mg-mixed", 1e30, arith=arith) as sim:
            g = sim.d.grid
            if rhs is None:
                rhs = rng.standard_normal(sim.padded_shape)
                p_rand = rng.standard_normal(sim.padded_shape)
                og = o.grid(*dims, g.xlength, g.ylength, g.zlength)
                p_conv = np.zeros(sim.padded_shape)
                cyc, rel_c = o.op_mg_solve(og, "mg", p_conv, rhs, rtol=1e-9, maxcycles=400)
                assert cyc < 400 and rel_c <= 1e-9
            sim.set_field("rhs", rhs)
            out = []
            for p in (p_rand, p_conv):
                sim.set_field("p", p)
                out.append(sim.solve())
                # one residual, no correction (the solve still writes p's Neumann ghosts)
                np.testing.assert_array_equal(sim.field("p")[1:-1, 1:-1, 1:-1],
                                              p[1:-1, 1:-1, 1:-1])
            rels[arith] = out
    assert rels["df32"][0] == pytest.approx(rels["fp64"][0], rel=1e-12)
    assert rels["fp64"][1] == pytest.approx(rel_c, rel=1e-3)
    assert rels["df32"][1] == pytest.approx(rels["fp64"][1], rel=2e-2)


@pytest.mark.parametrize("dims", [(32, 32, 32), (33, 17, 9)])
def test_mixed_solve_in_pairs_matches_fp64_residual(nusif_lib, dims):
    """A whole mixed solve with the residual in pairs and in FP64 instructions:
    both end below rtol, with cycle counts within one (a residual within 2^-47
    of a FP32 rounding boundary can round its FP32 copy the other way) and
    pressures within 5e-8 of their magnitude (both are rtol = 1e-8 solutions)."""
    rng = np.random.default_rng(31)
    p0 = rhs = None
    res = {}
    for arith in ("df32", "fp64"):
        with _sim(dims, "mg-mixed", 1e-8, mg_cycles=60, arith=arith) as sim:
            if p0 is None:
                p0 = rng.standard_normal(sim.padded_shape)
                rhs = rng.standard_normal(sim.padded_shape)
            sim.set_field("p", p0)
            sim.set_field("rhs", rhs)
            rel = sim.solve()
            res[arith] = (rel, sim.iterations, _interior_demeaned(sim.field("p")))
    (r1, c1, a), (r2, c2, b) = res["df32"], res["fp64"]
    assert r1 <= 1e-8 and r2 <= 1e-8
    assert abs(c1 - c2) <= 1
    assert np.max(np.abs(a - b)) <= 5e-8 * np.max(np.abs(b))


@pytest.mark.parametrize("solver", ["mg", "mg-mixed"])
def test_mg_zero_rhs_returns_at_once(nusif_lib, solver):
    with _sim((16, 16, 16), solver, 1e-6) as sim:
        p0 = np.random.default_rng(1).standard_normal(sim.padded_shape)
        sim.set_field("p", p0)
        sim.set_field("rhs", np.full(sim.padded_shape, 3.25))  # constant: mean-free part is 0
        assert sim.solve() == 0.0
        assert sim.iterations == 0
        np.testing.assert_array_equal(sim.field("p")[1:-1, 1:-1, 1:-1], p0[1:-1, 1:-1, 1:-1])


@pytest.mark.parametrize("solver", ["mg", "mg-mixed"])
def test_mg_time_loop_matches_oracle(nusif_lib, oracle_mod, solver):
    """A 32^3 cavity for 10 steps: the V-cycle solvers inside the time loop."""
    from nusif import Simulation
    from nusif.params import cavity
    vals = cavity(32, te=1e9, solver=solver, rtol=1e-8)
    run = oracle_mod.OracleRun(vals, solver)
    tol = 1e-9 if solver == "mg" else 1e-5
    with Simulation(vals) as sim:
        for s in range(10):
            a = sim.step()
            it, res, dt, t = run.step()
            assert a.dt == pytest.approx(dt, rel=1e-6 if solver == "mg-mixed" else 1e-10)
            if solver == "mg":
                assert a.it == it
            assert a.res <= 1e-8
            for f in "uvw":
                assert rel_err(sim.field(f), run.field(f)) < tol, (s, f)


@pytest.mark.parametrize("solver,guess", [("mg", "extrapolate"), ("mg-mixed", "extrapolate"),
                                          ("mg-mixed", "quadratic"), ("mg-mixed", "cubic")])
def test_mg_extrapolated_guess(nusif_lib, solver, guess):
    """mg_guess extrapolate / quadratic start each solve from 2 p(n-1) - p(n-2)
    / 3 p(n-1) - 3 p(n-2) + p(n-3): every step still ends at rtol, the
    velocities stay those of the previous-p guess to the solver tolerance, and
    the time loop needs fewer V-cycles."""
    from nusif import Simulation
    from nusif.params import cavity
    base = cavity(32, re=1000.0, te=1e9, solver=solver, rtol=1e-8)
    cycles = {}
    fields = {}
    for g in ("previous", guess):
        with Simulation(dict(base, mg_guess=g)) as sim:
            its = []
            for _ in range(12):
                a = sim.step()
                assert a.res <= 1e-8
                its.append(a.it)
            cycles[g] = sum(its[4:])
            fields[g] = {f: sim.field(f) for f in "uvw"}
    assert cycles[guess] < cycles["previous"]
    for f in "uvw":
        assert rel_err(fields[guess][f], fields["previous"][f]) < 1e-5, f


@pytest.mark.parametrize("guess", ["extrapolate", "quadratic", "cubic"])
def test_warm_start_values(nusif_lib, guess):
    """The warm start itself: with rtol 1e30 a solve stops after its first
    residual, so p after solve() is the extrapolated start. Four solves from
    pressures A, B, C, D give A, 2B - A, then 3C - 3B + A and 3D - 3C + B
    (quadratic; the history buffers alternate roles), 3C - 3B + A and
    4D - 6C + 4B - A (cubic; three buffers rotate) or 2C - B and 2D - C
    (linear), over the whole interior."""
    rng = np.random.default_rng(43)
    with _sim((24, 16, 12), "mg-mixed", 1e30, mg_guess=guess) as sim:
        shape = sim.padded_shape
        pres = [rng.standard_normal(shape) for _ in range(4)]
        sim.set_field("rhs", rng.standard_normal(shape))
        got = []
        for q in range(4):
            sim.set_field("p", pres[q])
            sim.solve()
            got.append(sim.field("p")[1:-1, 1:-1, 1:-1])
        A, B, C, D = (x[1:-1, 1:-1, 1:-1] for x in pres)
        if guess == "quadratic":
            want = [A, 2 * B - A, 3 * (C - B) + A, 3 * (D - C) + B]
        elif guess == "cubic":
            want = [A, 2 * B - A, 3 * (C - B) + A, 4 * D - 6 * C + 4 * B - A]
        else:
            want = [A, 2 * B - A, 2 * C - B, 2 * D - C]
        for q in range(4):
            assert rel_err(got[q], want[q]) < 1e-15, q


def _rb_sweep_f32(x, b, h):
    """Two-pass red-black Gauss-Seidel (first colour (i+j+k) even, 0-based),
    ghost-free Neumann operator, float32 with float64 sums (numpy)."""
    x = x.astype(np.float32).copy()
    ex, ey, ez = (np.float32(1.0 / (s * s)) for s in h)
    diag = np.float32(2.0 * (1.0 / h[0] ** 2 + 1.0 / h[1] ** 2 + 1.0 / h[2] ** 2))
    k, j, i = np.meshgrid(*[np.arange(n) for n in x.shape], indexing="ij")
    for colour in (0, 1):
        xp = np.pad(x, 1, mode="edge")
        c = xp[1:-1, 1:-1, 1:-1]
        lap = (ex * (xp[1:-1, 1:-1, :-2] + xp[1:-1, 1:-1, 2:]) + ey * (xp[1:-1, :-2, 1:-1] +
               xp[1:-1, 2:, 1:-1]) + ez * (xp[:-2, 1:-1, 1:-1] + xp[2:, 1:-1, 1:-1]) - diag * c)
        new = c - (b - lap) / diag
        m = ((i + j + k) & 1) == colour
        x[m] = new[m]
    return x


@pytest.mark.parametrize("dims", [(64, 16, 8), (128, 24, 40), (20, 12, 16), (36, 9, 70), (4, 3, 5)])
def test_fp32_one_kernel_sweep_is_exact_red_black(nusif_lib, dims):
    """The one-kernel FP32 sweep equals two red-black passes (to FP32 rounding:
    contraction and summation order), on ragged tiles and chunk edges."""
    import ctypes as C

    import torch
    nx, ny, nz = dims
    rng = np.random.default_rng(31)
    x = rng.standard_normal((nz, ny, nx)).astype(np.float32)
    b = rng.standard_normal((nz, ny, nx)).astype(np.float32)
    h = (1.0 / nx, 0.8 / ny, 1.2 / nz)
    want = x
    for s in (1, 2, 3):
        want = _rb_sweep_f32(want, b, h)
        xd, bd = torch.from_numpy(x).cuda(), torch.from_numpy(b).cuda()
        out = torch.empty_like(xd)
        rc = nusif_lib.nusifSmoothRBF32(C.c_void_p(xd.data_ptr()), C.c_void_p(bd.data_ptr()),
                                        C.c_void_p(out.data_ptr()), nx, ny, nz, *h, s)
        assert rc == 0
        got = out.cpu().numpy()
        scale = np.abs(want).max()
        assert np.max(np.abs(got - want)) <= 2e-5 * scale, (s, np.max(np.abs(got - want)) / scale)


@pytest.mark.parametrize("dims", [(128, 24, 40), (256, 16, 12), (128, 8, 70), (384, 40, 9)])
def test_register_tiled_sweep_equals_shared_memory_sweep(nusif_lib, dims, monkeypatch):
    """k_rbgs_sweep_v (rows a multiple of 128 cells, columns of 8: x-neighbours
    by shuffle, z-neighbours in registers) gives the same bits as k_rbgs_sweep
    (NUSIF_SWEEP=tile64), from a start and from zero, for one to three sweeps,
    on chunked planes and x-tiles with both x walls inside one tile row."""
    import ctypes as C

    import torch
    nx, ny, nz = dims
    rng = np.random.default_rng(37)
    x = torch.from_numpy(rng.standard_normal((nz, ny, nx)).astype(np.float32)).cuda()
    b = torch.from_numpy(rng.standard_normal((nz, ny, nx)).astype(np.float32)).cuda()
    h = (1.1 / nx, 0.7 / ny, 1.3 / nz)
    for start in (x, None):
        for s in (1, 2, 3):
            got = {}
            for kernel in ("tile64", "vector"):
                if kernel == "tile64":
                    monkeypatch.setenv("NUSIF_SWEEP", "tile64")
                else:
                    monkeypatch.delenv("NUSIF_SWEEP", raising=False)
                out = torch.empty_like(x)
                rc = nusif_lib.nusifSmoothRBF32(
                    C.c_void_p(start.data_ptr()) if start is not None else None,
                    C.c_void_p(b.data_ptr()), C.c_void_p(out.data_ptr()), nx, ny, nz, *h, s)
                assert rc == 0
                got[kernel] = out.cpu().numpy()
            np.testing.assert_array_equal(got["vector"], got["tile64"])


@pytest.mark.parametrize("solver,pre,post", [("mg", 2, 2), ("mg-mixed", 2, 2), ("mg-mixed", 3, 3),
                                             ("mg-mixed", 3, 1), ("mg-mixed", 2, 1)])
def test_graph_solve_matches_host_driven_solve(nusif_lib, solver, pre, post):
    """The solve as one CUDA graph (while-loops over units and over FP32
    V-cycles) is the host-driven solve launch for launch: same V-cycles, same
    fields bit for bit. (2, 1) has an odd sweep count per level and keeps
    the host-driven path in both runs.)"""
    from nusif import Simulation
    from nusif.params import cavity
    base = cavity((32, 24, 16), re=900.0, te=1e9, solver=solver, rtol=1e-7, mg_pre=pre,
                  mg_post=post, mg_guess="extrapolate")
    with Simulation(dict(base, mg_graph=1)) as a, Simulation(dict(base, mg_graph=0)) as b:
        for _ in range(6):
            ia, ib = a.step(), b.step()
            assert ia.it == ib.it
            assert ia.res == ib.res
        for f in "uvwp":
            np.testing.assert_array_equal(a.field(f), b.field(f))


@pytest.mark.parametrize("pre,post,theta,omega", [(1, 1, 0.9, 1.2), (1, 1, 0.99, 1.0),
                                                    (1, 3, 0.99, 1.3), (3, 1, 0.95, 1.1)])
def test_odd_sweep_counts_converge(nusif_lib, pre, post, theta, omega):
    """The FP32 smoother moves x between two buffers. When the correction meets
    its target in a V-cycle's fine restriction, the rest of that cycle is
    skipped; with odd sweep counts the skipped sweeps must still carry x to
    the buffer the fold reads (else the fold adds a stale correction and the
    refinement stalls just above rtol). Every step converges, within a few
    V-cycles, and the graph solve equals the host-driven one."""
    from nusif import Simulation
    from nusif.params import cavity
    base = cavity((48, 40, 32), re=1200.0, te=1e9, solver="mg-mixed", rtol=1e-7, mg_pre=pre,
                  mg_post=post, mg_theta=theta, mg_omega=omega, mg_inner=4, mg_cycles=40,
                  mg_guess="quadratic")
    graphs = [1, 0] if (pre + post) % 2 == 0 else [0]
    runs = []
    for graph in graphs:
        with Simulation(dict(base, mg_graph=graph)) as sim:
            infos = [sim.step() for _ in range(8)]
            for info in infos:
                assert info.res <= 1e-7, (graph, [(i.it, i.res) for i in infos])
                assert info.it <= 24
            runs.append(([(i.it, i.res) for i in infos], sim.field("p")))
    if len(runs) == 2:
        assert runs[0][0] == runs[1][0]
        np.testing.assert_array_equal(runs[0][1], runs[1][1])


@pytest.mark.parametrize("chunk", [1, 3, 7, 64])
def test_sweep_chunk_depth_does_not_change_results(nusif_lib, chunk):
    """The FP32 one-kernel sweep's planes per block (autotuned by default,
    forced here with mg_chunk) only splits the work: every cell is computed
    the same way, so the fields are the same bit for bit."""
    from nusif import Simulation
    from nusif.params import cavity
    base = cavity((64, 40, 48), re=800.0, te=1e9, solver="mg-mixed", rtol=1e-7,
                  mg_guess="quadratic")
    with Simulation(dict(base, mg_chunk=0)) as a, Simulation(dict(base, mg_chunk=chunk)) as b:
        for _ in range(4):
            ia, ib = a.step(), b.step()
            assert ia.it == ib.it and ia.res == ib.res
        for f in "uvwp":
            np.testing.assert_array_equal(a.field(f), b.field(f))


@pytest.mark.parametrize("solver", ["mg", "mg-mixed"])
def test_one_kernel_coarse_tail_matches(nusif_lib, solver):
    """mg_tail runs the small levels of each V-cycle in one single-block
    kernel with the per-level kernels' arithmetic: the same fields bit for bit."""
    from nusif import Simulation
    from nusif.params import cavity
    base = cavity(64, re=700.0, te=1e9, solver=solver, rtol=1e-7, mg_guess="quadratic")
    with Simulation(dict(base, mg_tail=0)) as a, Simulation(dict(base, mg_tail=4096)) as b:
        for _ in range(5):
            ia, ib = a.step(), b.step()
            assert ia.it == ib.it
        for f in "uvwp":
            np.testing.assert_array_equal(a.field(f), b.field(f))


@pytest.mark.parametrize("dims", [(64, 16, 8), (20, 12, 16), (36, 9, 70), (4, 3, 5), (128, 24, 40)])
def test_fp32_zero_start_sweep_is_exact_red_black(nusif_lib, dims):
    """The first pre-sweep of every V-cycle level starts from x = 0 and runs as
    one stencil pass over b (k_rb_zero_sweep): it equals a two-pass red-black
    sweep from zero, and the sweeps after it continue exactly."""
    import ctypes as C

    import torch
    nx, ny, nz = dims
    rng = np.random.default_rng(43)
    b = rng.standard_normal((nz, ny, nx)).astype(np.float32)
    h = (1.0 / nx, 0.8 / ny, 1.2 / nz)
    want = np.zeros_like(b)
    for s in (1, 2, 3):
        want = _rb_sweep_f32(want, b, h)
        bd = torch.from_numpy(b).cuda()
        out = torch.empty_like(bd)
        rc = nusif_lib.nusifSmoothRBF32(None, C.c_void_p(bd.data_ptr()),
                                        C.c_void_p(out.data_ptr()), nx, ny, nz, *h, s)
        assert rc == 0
        got = out.cpu().numpy()
        scale = np.abs(want).max()
        assert np.abs(got - want).max() <= 2e-5 * scale, (s, np.abs(got - want).max() / scale)


def _bits_f64(rng, n):
    """Random binary64 patterns over every exponent (normal, subnormal, zero,
    infinity, NaN), with round-to-nearest ties and near-ties for binary32."""
    b = rng.integers(0, 2 ** 63, size=n, dtype=np.int64).astype(np.uint64)
    b |= rng.integers(0, 2, size=n, dtype=np.uint64) << np.uint64(63)
    exp = rng.integers(0, 2048, size=n, dtype=np.uint64)
    near = rng.integers(0, 2, size=n).astype(bool)  # half of them near the binary32 range
    exp[near] = rng.integers(860, 1160, size=int(near.sum()), dtype=np.uint64)
    b = (b & ~(np.uint64(0x7ff) << np.uint64(52))) | (exp << np.uint64(52))
    low = np.uint64(0x1fffffff)
    ties = rng.integers(0, 4, size=n)
    b[ties == 0] = (b[ties == 0] & ~low) | np.uint64(0x10000000)          # exact ties
    b[ties == 1] = (b[ties == 1] & ~low) | np.uint64(0x10000001)          # just above
    b[ties == 2] = (b[ties == 2] & ~low) | np.uint64(0x0fffffff)          # just below
    edge = np.array([0, 1 << 63, 0x7ff0000000000000, 0xfff0000000000000, 0x7ff8000000000000,
                     0x47efffffe0000000, 0x47efffffefffffff, 0x47effffff0000000,
                     0x3810000000000000, 0x380fffffffffffff, 0x36a0000000000000,
                     0x3690000000000000, 0x0000000000000001, 0x000fffffffffffff],
                    dtype=np.uint64)
    return np.concatenate([edge, b]).view(np.float64)


def test_integer_pipe_conversions_match_hardware(nusif_lib):
    """The mixed-precision kernels convert FP64 <-> FP32 with integer
    operations; on random bit patterns of every class (ties, float subnormal
    and overflow range, zeros, infinities, NaN) they return exactly what the
    hardware conversion returns."""
    import ctypes as C

    import torch
    rng = np.random.default_rng(77)
    x = torch.from_numpy(_bits_f64(rng, 1 << 21)).cuda()
    y = torch.empty(x.shape, dtype=torch.float32, device="cuda")
    assert nusif_lib.nusifConvertF64ToF32(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                          x.numel()) == 0
    want = x.float()
    nan = torch.isnan(want)
    assert torch.equal(torch.isnan(y), nan)
    assert torch.equal(y[~nan].view(torch.int32), want[~nan].view(torch.int32))
    # widening: every float class, from random 32-bit patterns
    f = torch.from_numpy(rng.integers(0, 2 ** 32, size=1 << 21, dtype=np.uint64)
                         .astype(np.uint32).view(np.float32)).cuda()
    d = torch.empty(f.shape, dtype=torch.float64, device="cuda")
    assert nusif_lib.nusifConvertF32ToF64(C.c_void_p(f.data_ptr()), C.c_void_p(d.data_ptr()),
                                          f.numel()) == 0
    want = f.double()
    nan = torch.isnan(want)
    assert torch.equal(torch.isnan(d), nan)
    assert torch.equal(d[~nan].view(torch.int64), want[~nan].view(torch.int64))
