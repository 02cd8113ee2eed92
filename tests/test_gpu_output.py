"""Output path: the reference program's residual.dat and dcavity.vtk (written
by the reference itself, tests/golden/program_cavity10/) reproduced through
the library, and the device-side result collection against numpy."""
from __future__ import annotations

import struct

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASE = GOLDEN / "program_cavity10"


def _vtk_sections(text: str):
    lines = text.splitlines()
    header = lines[:10]
    p_start = 10
    n = int(lines[7].split()[1])
    pressure = np.array([float(x) for x in lines[p_start:p_start + n]])
    assert lines[p_start + n] == "VECTORS velocity double"
    vel = np.array([[float(x) for x in ln.split()] for ln in lines[p_start + n + 1:]])
    return header, pressure, vel


def test_program_outputs_match_reference(nusif_lib, tmp_path):
    from nusif import Simulation
    with Simulation(CASE / "case.par") as sim:
        sim.run(residual_file=tmp_path / "residual.dat")
        sim.write_vtk(tmp_path / "dcavity.vtk")
        sim.write_vtk(tmp_path / "dcavity_bin.vtk", binary=True)
        n = int(np.prod(sim.dims))
    ref_res = (CASE / "residual.dat").read_text().splitlines()
    got_res = (tmp_path / "residual.dat").read_text().splitlines()
    assert len(got_res) == len(ref_res)
    for a, b in zip(got_res, ref_res):
        ta, ra = (float(x) for x in a.split(","))
        tb, rb = (float(x) for x in b.split(","))
        assert ta == pytest.approx(tb, abs=1.5e-6) and ra == pytest.approx(rb, abs=1.5e-6)
    h_ref, p_ref, v_ref = _vtk_sections((CASE / "dcavity.vtk").read_text())
    h_got, p_got, v_got = _vtk_sections((tmp_path / "dcavity.vtk").read_text())
    assert h_got == h_ref
    np.testing.assert_allclose(p_got, p_ref, atol=1.5e-6, rtol=0)
    np.testing.assert_allclose(v_got, v_ref, atol=1.5e-6, rtol=0)
    # binary: same header with BINARY, big-endian doubles
    raw = (tmp_path / "dcavity_bin.vtk").read_bytes()
    head_end = raw.index(b"LOOKUP_TABLE default\n") + len(b"LOOKUP_TABLE default\n")
    assert raw[:head_end].decode().splitlines()[2] == "BINARY"
    p_bin = np.array(struct.unpack(f">{n}d", raw[head_end:head_end + 8 * n]))
    np.testing.assert_allclose(p_bin, p_ref, atol=6e-7, rtol=0)
    rest = raw[head_end + 8 * n:]
    assert rest.startswith(b"\nVECTORS velocity double\n")
    vel = np.array(struct.unpack(f">{3 * n}d", rest[25:25 + 24 * n])).reshape(n, 3)
    np.testing.assert_allclose(vel, v_ref, atol=6e-7, rtol=0)


def test_collect_matches_numpy(nusif_lib):
    from nusif import Simulation
    from nusif.params import cavity
    rng = np.random.default_rng(4)
    with Simulation(cavity((11, 7, 5), te=1e9)) as sim:
        fields = {f: rng.standard_normal(sim.padded_shape) for f in "uvwp"}
        for f, a in fields.items():
            sim.set_field(f, a)
        got = sim.collect()
    u, v, w, p = (fields[f] for f in "uvwp")
    np.testing.assert_array_equal(got["p"], p[1:-1, 1:-1, 1:-1])
    np.testing.assert_array_equal(got["u"], (u[1:-1, 1:-1, 1:-1] + u[1:-1, 1:-1, :-2]) / 2.0)
    np.testing.assert_array_equal(got["v"], (v[1:-1, 1:-1, 1:-1] + v[1:-1, :-2, 1:-1]) / 2.0)
    np.testing.assert_array_equal(got["w"], (w[1:-1, 1:-1, 1:-1] + w[:-2, 1:-1, 1:-1]) / 2.0)


def test_host_fields_are_readable_through_the_struct_pointers(nusif_lib):
    """host_fields 1: the eight fields live in managed memory kept in HBM, so
    host code - the reference's output stage (src/main.c:122-133, which hands
    d.u, d.v, d.w, d.p to commCollectResult) - reads them through the
    Discretization's own pointers; the run is bit-identical to one in plain
    device memory."""
    import torch

    from nusif import Simulation
    from nusif.params import cavity
    base = cavity((24, 16, 20), re=500.0, te=1e9)
    with Simulation(dict(base, host_fields=1)) as a, Simulation(base) as b:
        for _ in range(3):
            a.step()
            b.step()
        torch.cuda.synchronize()
        shape = a.padded_shape
        n = int(np.prod(shape))
        for f in "uvwp":
            host = np.ctypeslib.as_array(getattr(a.d, f), shape=(n,)).reshape(shape).copy()
            np.testing.assert_array_equal(host, a.field(f))
            np.testing.assert_array_equal(a.field(f), b.field(f))
