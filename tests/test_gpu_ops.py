"""Per-operator parity of the CUDA library (through the C ABI) against the
golden vectors of the reference and against the CPU oracle on seeded random
fields at small, odd and ragged sizes.

Tolerances: the GPU evaluates the reference's FP64 expressions with fused
multiply-adds and reordered sums, so results may differ in the last bits.
Boundary copies are exact; arithmetic operators must agree to 1e-13 of the
field's magnitude; the red-black solve must give the same iteration count and
fields to 1e-11. computeFG runs in both of its arithmetic forms (fg_arith
df32: face fluxes in pairs of FP32 numbers, the default; fp64: FP64
instructions), both held to the same 1e-13.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_values, load_golden, rel_err

pytestmark = pytest.mark.gpu

NAMES = ("u", "v", "w", "p", "rhs", "f", "g", "h")
TOL = 1e-13


def _sim(vals):
    from nusif import Simulation
    return Simulation(vals)


def _upload(sim, arrays):
    for f, a in arrays.items():
        sim.set_field(f, a)


def test_operators_match_golden(nusif_lib):
    z = load_golden("kat_ops.npz")
    v = golden_values(z)
    inputs = {f: z[f"in_{f}"] for f in NAMES}
    with _sim(v) as sim:
        assert sim.d.dtBound == pytest.approx(float(z["dtbound"]), rel=1e-15)

        def run(op):
            _upload(sim, inputs)
            sim.d.dt = float(z["dt_in"])
            getattr(sim, op)()

        run("compute_timestep")
        assert sim.d.dt == pytest.approx(float(z["timestep_dt"]), rel=1e-15)
        run("set_boundary_conditions")
        for f in "uvw":
            np.testing.assert_array_equal(sim.field(f), z[f"bc_out_{f}"])
        run("set_special_boundary_condition")
        np.testing.assert_array_equal(sim.field("u"), z["special_out_u"])
        run("compute_fg")
        for f in "fgh":
            assert rel_err(sim.field(f), z[f"fg_out_{f}"]) < TOL, f
        run("compute_rhs")
        assert rel_err(sim.field("rhs"), z["rhs_out_rhs"]) < TOL
        run("normalize_pressure")
        assert rel_err(sim.field("p"), z["normalize_out_p"]) < TOL
        run("adapt_uv")
        for f in "uvw":
            assert rel_err(sim.field(f), z[f"adapt_out_{f}"]) < TOL, f
        _upload(sim, inputs)
        res = sim.solve()
        assert sim.iterations == int(z["solve_it"])
        assert res == pytest.approx(float(z["solve_res"]), rel=1e-11)
        assert rel_err(sim.field("p"), z["solve_out_p"]) < 1e-11


SIZES = [(5, 5, 5), (8, 8, 8), (17, 9, 13), (33, 33, 33), (64, 3, 7), (1, 4, 6)]
BCS = [(1, 1, 1, 1, 1, 1), (2, 3, 2, 1, 3, 4), (3, 3, 1, 1, 2, 2)]


def _case(dims, bc, name="dcavity", **over):
    from nusif.params import cavity
    keys = ("bcLeft", "bcRight", "bcBottom", "bcTop", "bcFront", "bcBack")
    base = dict(xlength=1.1, ylength=0.8, zlength=1.3, name=name, re=300.0, gamma=0.85,
                gx=0.05, gy=-0.1, gz=0.02, tau=0.5, te=1e9, omg=1.7, eps=1e-6, itermax=25)
    base.update(zip(keys, bc))
    base.update(over)
    return cavity(dims, **base)


@pytest.mark.parametrize("arith", ["df32", "fp64"])
@pytest.mark.parametrize("dims", SIZES)
@pytest.mark.parametrize("bci", range(len(BCS)))
def test_operators_match_oracle_random(nusif_lib, oracle_mod, dims, bci, arith):
    o = oracle_mod
    name = "canal" if bci == 2 else "dcavity"
    v = _case(dims, BCS[bci], name=name, lid=1.25, inflow=0.75, fg_arith=arith)
    rng = np.random.default_rng(abs(hash((dims, bci))) % (2 ** 32))
    with _sim(v) as sim:
        shape = sim.padded_shape
        inputs = {f: rng.standard_normal(shape) for f in NAMES}
        g = o.grid(*dims, v["xlength"], v["ylength"], v["zlength"])
        dt = 0.0123

        def gpu(op):
            _upload(sim, inputs)
            sim.d.dt = dt
            getattr(sim, op)()

        def cpu():
            return {f: inputs[f].copy() for f in NAMES}

        gpu("compute_timestep")
        a = cpu()
        assert sim.d.dt == o.op_timestep(g, sim.d.dtBound, a["u"], a["v"], a["w"], v["tau"])

        gpu("set_boundary_conditions")
        a = cpu()
        o.op_set_bc(g, [v[k] for k in o.BC_ORDER], a["u"], a["v"], a["w"])
        for f in "uvw":
            np.testing.assert_array_equal(sim.field(f), a[f])

        gpu("set_special_boundary_condition")
        a = cpu()
        o.op_special_bc(g, name, a["u"], lid=1.25, inflow=0.75)
        np.testing.assert_array_equal(sim.field("u"), a["u"])

        gpu("compute_fg")
        a = cpu()
        o.op_fgh(g, v["re"], v["gamma"], v["gx"], v["gy"], v["gz"], dt, a["u"], a["v"],
                 a["w"], a["f"], a["g"], a["h"])
        for f in "fgh":
            assert rel_err(sim.field(f), a[f]) < TOL, f

        gpu("compute_rhs")
        a = cpu()
        o.op_rhs(g, dt, a["f"], a["g"], a["h"], a["rhs"])
        assert rel_err(sim.field("rhs"), a["rhs"]) < TOL

        gpu("normalize_pressure")
        a = cpu()
        o.op_normalize(g, a["p"])
        assert rel_err(sim.field("p"), a["p"]) < TOL

        gpu("adapt_uv")
        a = cpu()
        o.op_adapt(g, dt, a["f"], a["g"], a["h"], a["p"], a["u"], a["v"], a["w"])
        for f in "uvw":
            assert rel_err(sim.field(f), a[f]) < TOL, f

        # untouched fields stay untouched (no stray writes)
        for f in ("f", "g", "h", "rhs", "p"):
            np.testing.assert_array_equal(sim.field(f), inputs[f])


@pytest.mark.parametrize("arith", ["df32", "fp64"])
@pytest.mark.parametrize("dims", [(8, 8, 8), (17, 9, 13), (33, 33, 33), (2, 5, 3)])
def test_rb_solve_matches_oracle(nusif_lib, oracle_mod, dims, arith):
    """Red-black SOR with its residual in FP32 pairs (arith df32, the default)
    and in FP64 instructions: the same iteration count as the oracle, the
    carried residual and the pressure to 1e-11."""
    o = oracle_mod
    v = _case(dims, BCS[0], itermax=60, eps=1e-9, arith=arith)
    rng = np.random.default_rng(7)
    with _sim(v) as sim:
        g = o.grid(*dims, v["xlength"], v["ylength"], v["zlength"])
        p = rng.standard_normal(sim.padded_shape)
        rhs = rng.standard_normal(sim.padded_shape)
        sim.set_field("p", p)
        sim.set_field("rhs", rhs)
        res = sim.solve()
        pc = p.copy()
        it, res_c = o.op_solve_rb(g, v["eps"], v["omg"], v["itermax"], pc, rhs)
        assert sim.iterations == it
        assert res == pytest.approx(res_c, rel=1e-11)
        assert rel_err(sim.field("p"), pc) < 1e-11
        np.testing.assert_array_equal(sim.field("rhs"), rhs)


@pytest.mark.parametrize("levels,pre,post", [(3, 5, 3), (1, 4, 2), (2, 0, 2)])
def test_mg_ref_solve_matches_oracle(nusif_lib, oracle_mod, levels, pre, post):
    o = oracle_mod
    dims = (12, 10, 9)
    v = _case(dims, BCS[0], solver="mg-ref", levels=levels, presmooth=pre, postsmooth=post)
    rng = np.random.default_rng(11)
    with _sim(v) as sim:
        g = o.grid(*dims, v["xlength"], v["ylength"], v["zlength"])
        p = rng.standard_normal(sim.padded_shape)
        rhs = rng.standard_normal(sim.padded_shape)
        sim.set_field("p", p)
        sim.set_field("rhs", rhs)
        res = sim.solve()
        pc = p.copy()
        res_c = o.op_solve_mg_ref(g, v["omg"], levels, pre, post, pc, rhs)
        assert res == pytest.approx(res_c, rel=1e-12)
        assert rel_err(sim.field("p"), pc) < 1e-12


@pytest.mark.parametrize("dims", [(3, 3, 3), (8, 6, 4), (33, 17, 9)])
def test_field_copies_pinned_pageable_unaligned(nusif_lib, dims):
    """nusifUploadField / nusifDownloadField round trips, bit for bit, from
    page-locked host memory, from pageable memory and from a page-locked array
    8 bytes off 16-byte alignment; (3,3,3) pads to an odd number of doubles."""
    import ctypes as C

    import torch

    from nusif import abi
    from nusif.params import cavity
    rng = np.random.default_rng(5)
    with _sim(cavity(dims, te=1e9)) as sim:
        n = int(np.prod(sim.padded_shape))
        idx = abi.FIELD_INDEX
        pinned = torch.empty(n + 1, dtype=torch.float64, pin_memory=True)
        for name, kind in (("u", "pinned"), ("p", "pageable"), ("w", "unaligned")):
            a = rng.standard_normal(n)
            if kind == "pinned":
                buf = pinned.numpy()[:n]
            elif kind == "unaligned":
                buf = pinned.numpy()[1:n + 1]
            else:
                buf = np.empty(n)
            buf[:] = a
            ptr = C.cast(buf.ctypes.data, abi.c_double_p)
            assert nusif_lib.nusifUploadField(C.byref(sim.d), idx[name], ptr) == 0
            abi.check(nusif_lib)
            np.testing.assert_array_equal(sim.field(name).reshape(-1), a)
            buf[:] = 0.0
            assert nusif_lib.nusifDownloadField(C.byref(sim.d), idx[name], ptr) == 0
            abi.check(nusif_lib)
            np.testing.assert_array_equal(buf, a)


def test_queued_field_copies_match_synchronous_copies(nusif_lib):
    """Three time steps of a 24^3 cavity, each step's u, v, w, p uploaded from
    and downloaded to pinned host arrays: with the queued copies
    (nusifUploadFieldAsync / nusifDownloadFieldAsync / nusifWaitCopies, the
    library's kernels waiting on the device for the fields they use) the host
    arrays end bit-identical to the same loop with the synchronous copies,
    also with p's download queued between solve() and adaptUV (which reads p
    while the copy runs and does not wait for it)."""
    import ctypes as C

    import torch

    from nusif import Simulation, abi
    from nusif.params import cavity
    vals = cavity(24, te=1e9, solver="mg-mixed", rtol=1e-8, mg_guess="quadratic")
    idx = abi.FIELD_INDEX
    out = {}
    for mode in ("sync", "queued", "p_early"):
        with Simulation(vals) as sim:
            n = int(np.prod(sim.padded_shape))
            host = {f: torch.zeros(n, dtype=torch.float64, pin_memory=True) for f in "uvwp"}
            ptrs = {f: C.cast(host[f].data_ptr(), abi.c_double_p) for f in "uvwp"}
            down = nusif_lib.nusifDownloadField if mode == "sync" else \
                nusif_lib.nusifDownloadFieldAsync
            for _ in range(3):
                for f in "uvwp":
                    fn = nusif_lib.nusifUploadField if mode == "sync" else \
                        nusif_lib.nusifUploadFieldAsync
                    assert fn(C.byref(sim.d), idx[f], ptrs[f]) == 0
                early = "p" if mode == "p_early" else ""
                sim.step(after_solve=(lambda: down(C.byref(sim.d), idx["p"], ptrs["p"]))
                         if early else None)
                for f in "uvwp":
                    if f == early:
                        continue
                    assert down(C.byref(sim.d), idx[f], ptrs[f]) == 0
                assert nusif_lib.nusifWaitCopies() == 0
                abi.check(nusif_lib)
            out[mode] = {f: host[f].numpy().copy() for f in "uvwp"}
            for f in "uvwp":  # the device fields are the downloaded ones
                np.testing.assert_array_equal(sim.field(f).reshape(-1), out[mode][f])
    for f in "uvwp":
        assert np.any(out["sync"][f] != 0.0) or f != "u"
        np.testing.assert_array_equal(out["queued"][f], out["sync"][f])
        np.testing.assert_array_equal(out["p_early"][f], out["sync"][f])


def test_write_after_queued_download_waits_for_it(nusif_lib):
    """A queued download of p followed at once by an entry point that writes p
    (normalizePressure): the write waits for the copy on the device, so the
    host array holds p as it was when the download was queued."""
    import ctypes as C

    import torch

    from nusif import Simulation, abi
    from nusif.params import cavity
    rng = np.random.default_rng(61)
    with Simulation(cavity((40, 36, 33), te=1e9)) as sim:
        p0 = rng.standard_normal(sim.padded_shape) + 3.0
        sim.set_field("p", p0)
        n = int(np.prod(sim.padded_shape))
        host = torch.zeros(n, dtype=torch.float64, pin_memory=True)
        ptr = C.cast(host.data_ptr(), abi.c_double_p)
        assert nusif_lib.nusifDownloadFieldAsync(C.byref(sim.d), abi.FIELD_INDEX["p"], ptr) == 0
        sim.normalize_pressure()  # subtracts the mean from p on the device
        assert nusif_lib.nusifWaitCopies() == 0
        abi.check(nusif_lib)
        np.testing.assert_array_equal(host.numpy().reshape(sim.padded_shape), p0)
        assert not np.array_equal(sim.field("p"), p0)
