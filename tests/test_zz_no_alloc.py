"""The allocation-free red-black solve (nusifSolveRBStatic) against solve().

Callers that cannot allocate device memory -- hosts that hand out only
pre-sized device buffers, runtimes that reserve all device memory at
start-up -- use nusifSolveRBStatic, whose scratch is a fixed __device__ array
inside the library. It relaxes in FP64 instructions, so it must give what
solve() with the rb solver and the key arith fp64 gives on the same inputs: the same iteration count, the residual and the pressure
within the tolerance of the other red-black tests (1e-11 relative), on two
calls in a row (the second call must not inherit the first call's counter or
state), and a call must leave the device's free memory unchanged. This file
is collected last so that a run stopping at the first failure has run every
other test already.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _solve_both(nusif_lib, sim, p0, rhs, eps, itermax):
    from nusif import abi
    sim.s.eps, sim.s.itermax = eps, itermax
    sim.set_field("p", p0)
    sim.set_field("rhs", rhs)
    res_ref = sim.solve()
    it_ref = sim.iterations
    p_ref = sim.field("p")

    sim.set_field("p", p0)
    g = sim.d.grid
    res, it = C.c_double(), C.c_int()
    code = nusif_lib.nusifSolveRBStatic(sim.d.p, sim.d.rhs, g.imax, g.jmax, g.kmax, g.dx, g.dy,
                                        g.dz, sim.d.omega, eps, itermax, C.byref(res),
                                        C.byref(it))
    abi.check(nusif_lib)
    assert code == 0
    return (res_ref, it_ref, p_ref), (res.value, it.value, sim.field("p"))


@pytest.mark.parametrize("dims", [(33, 17, 9), (64, 64, 64)])
def test_static_solve_matches_solve_twice(nusif_lib, dims):
    from nusif import Simulation
    from nusif.params import cavity
    rng = np.random.default_rng(2026)
    with Simulation(cavity(dims, omg=1.7, xlength=1.2, zlength=0.9, te=1e9,
                           arith="fp64")) as sim:
        shape = sim.padded_shape
        for call, (eps, itermax) in enumerate([(1e-3, 400), (1e-9, 37)]):
            p0 = rng.standard_normal(shape)
            rhs = rng.standard_normal(shape)
            (r0, i0, p_ref), (r1, i1, p_new) = _solve_both(nusif_lib, sim, p0, rhs, eps, itermax)
            assert i1 == i0, f"call {call}: iterations {i1} vs {i0}"
            assert r1 == pytest.approx(r0, rel=1e-11)
            assert rel_err(p_new, p_ref) < 1e-11
            np.testing.assert_array_equal(sim.field("rhs"), rhs)


def _free_device_bytes() -> int:
    import torch
    free, _ = torch.cuda.mem_get_info()
    return int(free)


def test_static_solve_allocates_nothing(nusif_lib):
    """After one call (kernels loaded, scratch address looked up), a second
    call on another grid leaves the device's free memory where it was."""
    from nusif import Simulation, abi
    from nusif.params import cavity
    rng = np.random.default_rng(7)
    sims = [Simulation(cavity(d, omg=1.7, te=1e9)) for d in ((24, 20, 16), (40, 12, 28))]
    try:
        for sim in sims:
            sim.set_field("p", rng.standard_normal(sim.padded_shape))
            sim.set_field("rhs", rng.standard_normal(sim.padded_shape))

        def call(sim):
            g = sim.d.grid
            res, it = C.c_double(), C.c_int()
            code = nusif_lib.nusifSolveRBStatic(sim.d.p, sim.d.rhs, g.imax, g.jmax, g.kmax,
                                                g.dx, g.dy, g.dz, 1.7, 1e-4, 200,
                                                C.byref(res), C.byref(it))
            abi.check(nusif_lib)
            assert code == 0 and it.value > 0

        call(sims[0])
        before = _free_device_bytes()
        call(sims[1])
        assert _free_device_bytes() == before
    finally:
        for sim in sims:
            sim.close()


def test_static_solve_rejects_oversized_grid(nusif_lib):
    res, it = C.c_double(), C.c_int()
    dummy = C.cast(C.c_void_p(256), C.POINTER(C.c_double))  # never dereferenced: rejected first
    code = nusif_lib.nusifSolveRBStatic(dummy, dummy, 1024, 1024, 1024, 1e-3, 1e-3, 1e-3, 1.7,
                                        1e-6, 10, C.byref(res), C.byref(it))
    buf = C.create_string_buffer(512)
    assert code == 2
    assert nusif_lib.nusifGetLastError(buf, 512) == 2
    assert b"static" in buf.value or b"index range" in buf.value
