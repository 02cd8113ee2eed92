"""Batched instances (one CUDA graph per step, device-side dt) against the
same cases stepped one at a time through the ordinary entry points.

The batch runs the same kernels with the same arithmetic (dt is computed on
the device with the host's expressions, the multigrid solve runs in a graph
while-loop that stops where the host-driven solve stops), so fields and times
must agree exactly and no step may end above rtol."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    from nusif.params import cavity
    return [
        cavity(16, re=300.0, solver="mg-mixed", rtol=1e-6, te=1e9),
        cavity((20, 12, 16), re=1500.0, lid=1.3, solver="mg-mixed", rtol=1e-6, te=1e9),
        cavity(32, re=800.0, solver="mg", rtol=1e-7, te=1e9),
        cavity((24, 32, 16), re=4000.0, lid=0.6, solver="mg-mixed", rtol=1e-6, te=1e9),
    ]


def _compare(batch, cases, steps):
    from nusif import Simulation
    for q, vals in enumerate(cases):
        with Simulation(vals) as sim:
            cycles = 0
            for _ in range(steps):
                cycles = sim.step().it
            st = batch.stats(q)
            assert st.nt == steps, q
            assert st.unconverged == 0, (q, st)
            assert st.cycles == cycles, (q, st)
            assert st.t == sim.t, q
            assert st.dt == sim.dt, q
            for f in "uvwp":
                np.testing.assert_array_equal(batch.field(q, f), sim.field(f), err_msg=f"{q}{f}")


@pytest.mark.parametrize("tune", [False, True])
def test_batch_matches_single_instances(nusif_lib, tune):
    from nusif import Batch
    cases = _cases()
    steps = 6
    with Batch(cases, tune=tune) as batch:
        batch.step(steps)
        _compare(batch, cases, steps)


def test_batch_warm_start_matches(nusif_lib):
    """The extrapolated warm starts run inside the captured step too."""
    from nusif import Batch
    cases = [dict(c, mg_guess=g) for c, g in zip(_cases(), ["quadratic", "extrapolate",
                                                             "quadratic", "previous"])]
    with Batch(cases, tune=False) as batch:
        batch.step(7)
        _compare(batch, cases, 7)


def test_batch_fixed_queue_long_enough_matches(nusif_lib):
    from nusif import Batch
    cases = _cases()
    with Batch(cases, queue=24, tune=False) as batch:
        batch.step(4)
        _compare(batch, cases, 4)


def test_batch_short_queue_is_counted(nusif_lib):
    """A fixed queue of one V-cycle cannot reach rtol = 1e-7: every step is
    counted as unconverged and exactly one cycle ran."""
    from nusif import Batch
    from nusif.params import cavity
    with Batch([cavity(32, re=800.0, solver="mg", rtol=1e-7, te=1e9)], queue=1,
               tune=False) as batch:
        batch.step(3)
        st = batch.stats(0)
        assert st.unconverged == 3
        assert st.cycles == 1


def test_batch_rejects_red_black_cases(nusif_lib):
    from nusif import Batch, NusifError
    from nusif.params import cavity
    with pytest.raises(NusifError):
        Batch([cavity(8, solver="rb", te=1e9)])
