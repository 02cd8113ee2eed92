"""Host check of the double-float helpers the FP64-bound stencils use
(cfd-bench_gb300/csrc/df32.cuh). split() builds the pair without conversion
instructions (GB300 runs them on its FP64 pipe): its low part must carry the
same bits as the rounded integer -> float conversion it replaces, hi + lo must
equal x to 2^-47 |x| (2^-97 absolute for |x| < 2^-74), and widen() must be the
exact binary32 -> binary64 conversion for every float class. The same source
compiles for the device; the GPU parity tests cover it there."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_split_and_widen_on_the_host(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "df32_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", str(ROOT / "cfd-bench_gb300" / "csrc"),
                    str(ROOT / "tests" / "df32_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "2000000"], check=True, capture_output=True, text=True)
    checked, bad_lo, bad_err, bad_widen = map(int, out.stdout.split())
    assert checked > 200000
    assert (bad_lo, bad_err, bad_widen) == (0, 0, 0)
