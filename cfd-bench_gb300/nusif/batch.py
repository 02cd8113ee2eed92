"""Many independent NuSiF instances advanced together (C ABI nusifBatch*).

Each instance is a .par case of its own (grids may differ); one time step of
all of them is one CUDA-graph launch. Fields are read through the same
download call as a single Simulation.
"""
from __future__ import annotations

import ctypes as C
import tempfile
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import abi
from .params import write_par


@dataclass
class InstanceStats:
    t: float
    dt: float
    nt: int
    cycles: int          # V-cycles of the last step
    unconverged: int     # steps whose solve ended above rtol
    fg_planes: int       # autotuned planes per block of the F/G/H kernel


class Batch:
    def __init__(self, cases: list[dict | str | Path], queue: int = 0, tune: bool = True):
        """queue = 0: each step's multigrid solve is a CUDA graph while-loop that
        stops at rtol, as the host-driven solve does; queue > 0: a fixed number of
        device-gated multigrid units per step (steps left above rtol are counted)."""
        self.lib = abi.load_library()
        self._tmp = tempfile.TemporaryDirectory(prefix="nusif_batch_")
        paths = []
        for q, c in enumerate(cases):
            if isinstance(c, dict):
                c = write_par(Path(self._tmp.name) / f"case{q}.par", c)
            paths.append(str(c).encode())
        arr = (C.c_char_p * len(paths))(*paths)
        self.handle = self.lib.nusifBatchCreate(len(paths), arr, queue, int(tune))
        abi.check(self.lib)
        if not self.handle:
            raise abi.NusifError("nusifBatchCreate failed")
        self.n = len(paths)

    def step(self, steps: int = 1) -> None:
        self.lib.nusifBatchStep(self.handle, steps)
        abi.check(self.lib)

    def _instance(self, idx: int):
        d = C.POINTER(abi.Discretization)()
        s = C.POINTER(abi.Solver)()
        self.lib.nusifBatchInstance(self.handle, idx, C.byref(d), C.byref(s))
        abi.check(self.lib)
        return d, s

    def dims(self, idx: int) -> tuple[int, int, int]:
        d, _ = self._instance(idx)
        g = d.contents.grid
        return g.imax, g.jmax, g.kmax

    def field(self, idx: int, name: str) -> np.ndarray:
        d, _ = self._instance(idx)
        i, j, k = self.dims(idx)
        out = np.empty((k + 2, j + 2, i + 2), dtype=np.float64)
        self.lib.nusifDownloadField(d, abi.FIELD_INDEX[name], out.ctypes.data_as(abi.c_double_p))
        abi.check(self.lib)
        return out

    def stats(self, idx: int) -> InstanceStats:
        t, dt = C.c_double(), C.c_double()
        nt, cyc, unc, kb = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self.lib.nusifBatchStats(self.handle, idx, C.byref(t), C.byref(dt), C.byref(nt),
                                 C.byref(cyc), C.byref(unc), C.byref(kb))
        abi.check(self.lib)
        return InstanceStats(t.value, dt.value, nt.value, cyc.value, unc.value, kb.value)

    def close(self) -> None:
        if self.handle:
            self.lib.nusifBatchFree(self.handle)
            self.handle = None
        self._tmp.cleanup()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
