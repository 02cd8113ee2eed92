"""The link-time drop-in: the reference's own main.c and the objects it keeps
(comm, progress, timing, allocate, profiler, sequential VTK writer) compile
unchanged against the reference headers and link against the library in
place of parameter.o, discretization.o and solver-*.o (the link line of the
integration notes). Host only: where no GPU is present the program must stop
with the reference's error behaviour (a message and EXIT_FAILURE), not crash.
Needs the reference sources; skipped where they are absent."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

import oracle  # noqa: E402  (test infrastructure: where the reference was built from)

_REF_ROOT = oracle.reference_source_root()
REF = (_REF_ROOT / "src") if _REF_ROOT else Path("/nonexistent")
KEPT = ["main.c", "comm.c", "progress.c", "timing.c", "allocate.c", "profiler.c",
        "vtkWriter-seq.c"]
LIB = ROOT / "cfd-bench_gb300" / "lib"


def _have_gpu() -> bool:
    from conftest import gpu_available
    return gpu_available()


@pytest.fixture(scope="module")
def linked(tmp_path_factory, nusif_lib):
    if not all((REF / f).exists() for f in KEPT) or shutil.which("gcc") is None:
        pytest.skip("reference sources or gcc not available")
    out = tmp_path_factory.mktemp("link")
    objs = []
    for f in KEPT:
        o = out / (Path(f).stem + ".o")
        subprocess.run(["gcc", "-O2", "-std=c99", "-D_GNU_SOURCE", "-DARRAY_ALIGNMENT=64",
                        "-I", str(REF), "-c", str(REF / f), "-o", str(o)], check=True,
                       capture_output=True)
        objs.append(str(o))
    exe = out / "nusif_gb300_main"
    r = subprocess.run(["gcc", "-o", str(exe), *objs, "-L", str(LIB), "-lnusif_gb300",
                        f"-Wl,-rpath,{LIB}", "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_reference_main_links_against_the_library(linked):
    assert linked.exists()
    # every library function the program calls is defined by the library
    und = subprocess.run(["nm", "-u", str(linked)], capture_output=True, text=True).stdout
    for name in ("initParameter", "readParameter", "initDiscretization", "computeTimestep",
                 "setBoundaryConditions", "setSpecialBoundaryCondition", "computeFG",
                 "computeRHS", "normalizePressure", "adaptUV", "initSolver", "solve"):
        assert name in und, name  # resolved at load time from libnusif_gb300.so


def test_reference_main_without_gpu_exits_like_the_reference(linked, tmp_path):
    if _have_gpu():
        pytest.skip("a GPU is present: the program would run")
    par = tmp_path / "t.par"
    par.write_text("name dcavity\nimax 8\njmax 8\nkmax 8\nte 0.01\ntau 0.5\nitermax 10\n"
                   "eps 0.001\nomg 1.7\ngamma 0.9\nre 10.0\n")
    r = subprocess.run([str(linked), str(par)], capture_output=True, text=True, timeout=120,
                       cwd=tmp_path)
    assert r.returncode == 1, (r.returncode, r.stderr[-500:])
    assert "Error" in r.stderr
    assert "Parameters for dcavity" in r.stdout  # the reference's own printParameter call ran
