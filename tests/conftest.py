"""Shared test set-up: import paths, the ``gpu`` marker, common helpers.

``-m "not gpu"`` covers the oracle (against the reference and the golden
vectors), the host logic and the C ABI of the library without launching
kernels. ``-m gpu`` runs the CUDA library against the oracle and the golden
vectors through the C ABI.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "cfd-bench_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


def gpu_available() -> bool:
    try:
        import ctypes
        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcuda.so.1"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return False
        if hasattr(cudart, "cuInit"):
            return cudart.cuInit(0) == 0
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def nusif_lib():
    """The built library (built on demand); fails loudly when it cannot be built."""
    import nusif
    from nusif.abi import LIB_PATH
    if not LIB_PATH.exists():
        sys.path.insert(0, str(ROOT / "cfd-bench_gb300"))
        import build as _b  # cfd-bench_gb300/build.py
        _b.build()
    return nusif.load_library()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(autouse=True)
def _require_gpu(request):
    if request.node.get_closest_marker("gpu") and not gpu_available():
        pytest.skip("no CUDA GPU")


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a-b| / max(max|b|, tiny): the relative field error used by the parity tests."""
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


def load_golden(name: str):
    return np.load(GOLDEN / name, allow_pickle=False)


def golden_values(z) -> dict:
    import ast
    return ast.literal_eval(str(z["values"]))
