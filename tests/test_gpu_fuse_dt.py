"""Key fuse_dt: adaptUV keeps the maxima of the velocities it writes and the
next computeTimestep reads only the ghost shell (computeTimestep +
maxElement, reference src/discretization.c:391-453). dt and every field must
equal the unfused run bit for bit (the unfused maxima are checked against the
oracle in test_gpu_ops.py), including when something else writes u, v, w
between adaptUV and computeTimestep."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from nusif import Simulation
from nusif.params import CANAL, cavity

pytestmark = pytest.mark.gpu

CASES = {
    # the lid's ghost values are the largest |u|: the shell decides u's maximum
    "cavity": cavity((24, 20, 16), re=500.0, te=1e9, solver="mg", rtol=1e-8),
    # inflow 2 on the left, outflow on the right: the interior decides
    "canal": dict(CANAL, imax=40, jmax=12, kmax=10, te=1e9, solver="mg", rtol=1e-8),
    # slip, outflow and periodic walls
    "bcmix": cavity((20, 16, 12), re=300.0, te=1e9, solver="mg", rtol=1e-8, bcLeft=2,
                    bcRight=3, bcBottom=1, bcTop=1, bcFront=4, bcBack=4, u_init=0.5),
}


def _counts(sim):
    shell, full = C.c_longlong(), C.c_longlong()
    assert sim.lib.nusifTimestepCounts(C.byref(sim.d), C.byref(shell), C.byref(full)) == 0
    return shell.value, full.value


def _run(vals, fuse, steps, between=None):
    dts = []
    with Simulation(dict(vals, fuse_dt=fuse)) as sim:
        for n in range(steps):
            dts.append(sim.step().dt)
            if between is not None:
                between(sim, n)
        fields = {f: sim.field(f) for f in "uvwp"}
        counts = _counts(sim)
    return dts, fields, counts


def _same(a, b):
    assert a[0] == b[0], (a[0], b[0])
    for f in "uvwp":
        np.testing.assert_array_equal(a[1][f], b[1][f], err_msg=f)


@pytest.mark.parametrize("case", sorted(CASES))
def test_fused_maxima_give_the_same_run(nusif_lib, case):
    steps = 8
    fused, plain = _run(CASES[case], 1, steps), _run(CASES[case], 0, steps)
    _same(fused, plain)
    # the first computeTimestep has no adaptUV before it; every later one uses the shell
    assert fused[2] == (steps - 1, 1), fused[2]
    assert plain[2] == (0, steps), plain[2]


def _bc_after_adapt(sim, n):
    sim.set_boundary_conditions()


def _upload_after_adapt(sim, n):
    u = sim.field("u")
    u[1:-1, 1:-1, 1:-1] *= 1.0 + 0.25 * (n % 3)
    sim.set_field("u", u)


def _adapt_twice(sim, n):
    if n % 2 == 0:
        sim.adapt_uv()


@pytest.mark.parametrize("between", [_bc_after_adapt, _upload_after_adapt, _adapt_twice])
def test_writes_between_adapt_and_timestep_fall_back(nusif_lib, between):
    steps = 6
    vals = CASES["canal"]
    fused, plain = _run(vals, 1, steps, between), _run(vals, 0, steps, between)
    _same(fused, plain)
    shell, full = fused[2]
    if between is _adapt_twice:  # steps after a second adaptUV read the whole arrays
        assert full == 1 + steps // 2 and shell == steps - full, fused[2]
    else:  # every write makes the kept maxima stale
        assert (shell, full) == (0, steps), fused[2]
