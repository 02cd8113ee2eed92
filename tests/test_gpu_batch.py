"""Batched instances (one CUDA graph per step, device-side dt) against the
same cases stepped one at a time through the ordinary entry points.

The batch runs the same kernels with the same arithmetic (dt is computed on
the device with the host's expressions), so fields and times must agree
exactly; no step may end above rtol with the default queue."""
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


@pytest.mark.parametrize("tune", [False, True])
def test_batch_matches_single_instances(nusif_lib, tune):
    from nusif import Batch, Simulation
    cases = _cases()
    steps = 6
    with Batch(cases, queue=4, tune=tune) as batch:
        batch.step(steps)
        for q, vals in enumerate(cases):
            with Simulation(vals) as sim:
                for _ in range(steps):
                    sim.step()
                st = batch.stats(q)
                assert st.nt == steps
                assert st.unconverged == 0
                assert st.t == sim.t
                assert st.dt == sim.dt
                for f in "uvwp":
                    np.testing.assert_array_equal(batch.field(q, f), sim.field(f), err_msg=f"{q}{f}")


def test_batch_rejects_red_black_cases(nusif_lib):
    from nusif import Batch, NusifError
    from nusif.params import cavity
    with pytest.raises(NusifError):
        Batch([cavity(8, solver="rb", te=1e9)])
