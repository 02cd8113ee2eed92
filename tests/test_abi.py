"""The C ABI without a GPU: the library loads, exports every entry point the
header declares, and its structs have the reference's layouts."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

HEADER = ROOT / "include" / "nusif_gb300.h"
import oracle  # noqa: E402  (test infrastructure: where the reference was built from)

_REF_ROOT = oracle.reference_source_root()
REF_SRC = (_REF_ROOT / "src") if _REF_ROOT else Path("/nonexistent")


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    return re.findall(r"^NUSIF_API\s+[\w\s\*]+?\b(\w+)\(", text, flags=re.M)


def test_header_declares_reference_entry_points():
    names = set(declared_functions())
    reference = {"initParameter", "readParameter", "printParameter", "initDiscretization",
                 "computeTimestep", "setBoundaryConditions", "setSpecialBoundaryCondition",
                 "computeFG", "computeRHS", "normalizePressure", "adaptUV", "initSolver",
                 "solve"}
    assert reference <= names


def test_library_exports_every_declared_symbol(nusif_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(nusif_lib._name)],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        assert hasattr(nusif_lib, n)


LAYOUT_PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include HEADER_UNDER_TEST
#define P(T, m) printf(#T "." #m " %zu\n", offsetof(T, m));
int main(void) {
  printf("Parameter %zu\nDiscretization %zu\nSolver %zu\nGrid %zu\nCommType %zu\n",
         sizeof(Parameter), sizeof(Discretization), sizeof(Solver), sizeof(Grid), sizeof(CommType));
  P(Parameter, name) P(Parameter, levels) P(Parameter, u_init) P(Parameter, itermax)
  P(Discretization, p) P(Discretization, w) P(Discretization, itermax) P(Discretization, dt)
  P(Discretization, problem) P(Discretization, bcBack) P(Discretization, comm)
  P(Solver, grid) P(Solver, r) P(Solver, levels) P(Solver, comm) P(Solver, problem)
  return 0;
}
"""


def _probe(tmp_path, includes: list[str], header: str) -> str:
    src = tmp_path / "probe.c"
    src.write_text(LAYOUT_PROBE.replace("HEADER_UNDER_TEST", header))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c99", *includes, "-o", str(exe), str(src)], check=True)
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout


def _ctypes_layout() -> str:
    from nusif import abi
    lines = [f"Parameter {C.sizeof(abi.Parameter)}", f"Discretization {C.sizeof(abi.Discretization)}",
             f"Solver {C.sizeof(abi.Solver)}", f"Grid {C.sizeof(abi.Grid)}",
             f"CommType {C.sizeof(abi.CommType)}"]
    for T, members in [(abi.Parameter, ["name", "levels", "u_init", "itermax"]),
                       (abi.Discretization, ["p", "w", "itermax", "dt", "problem", "bcBack", "comm"]),
                       (abi.Solver, ["grid", "r", "levels", "comm", "problem"])]:
        for m in members:
            lines.append(f"{T.__name__}.{m} {getattr(T, m).offset}")
    return "\n".join(lines) + "\n"


def test_ctypes_mirror_matches_header(tmp_path):
    assert _probe(tmp_path, [f"-I{ROOT / 'include'}"], '"nusif_gb300.h"') == _ctypes_layout()


@pytest.mark.skipif(not (REF_SRC / "solver.h").exists(), reason="reference sources absent")
def test_struct_layouts_match_reference_headers(tmp_path):
    mine = _probe(tmp_path, [f"-I{ROOT / 'include'}"], '"nusif_gb300.h"')
    ref = _probe(tmp_path, [f"-I{REF_SRC}", "-D_GNU_SOURCE"],
                 '"parameter.h"\n#include "discretization.h"\n#include "solver.h"')
    assert mine == ref


def test_error_mode_records_instead_of_exiting(nusif_lib):
    from nusif import abi
    p = abi.Parameter()
    nusif_lib.initParameter(C.byref(p))
    nusif_lib.readParameter(C.byref(p), b"/nonexistent/case.par")
    buf = C.create_string_buffer(256)
    assert nusif_lib.nusifGetLastError(buf, 256) == 3
    assert b"Could not open parameter file" in buf.value
    assert nusif_lib.nusifGetLastError(buf, 256) == 0


def test_unknown_solver_is_rejected(nusif_lib):
    from nusif import abi
    p = abi.Parameter()
    nusif_lib.initParameter(C.byref(p))
    assert nusif_lib.nusifParameterSet(C.byref(p), b"solver", b"cg") != 0
    assert nusif_lib.nusifGetLastError(None, 0) != 0


def test_calls_on_uninitialised_structs_fail_cleanly(nusif_lib):
    from nusif import abi
    d = abi.Discretization()
    nusif_lib.computeFG(C.byref(d))
    assert nusif_lib.nusifGetLastError(None, 0) == 4
    s = abi.Solver()
    assert nusif_lib.nusifSolverIterations(C.byref(s)) == -1
