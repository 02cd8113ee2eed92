"""Host driver over the C ABI: the reference time loop (src/main.c:53-88).

``Simulation`` owns one Parameter / Discretization / Solver triple of the
library and advances it with exactly the reference's call order. Every call
goes through the shared library; errors raise ``NusifError``.
"""
from __future__ import annotations

import ctypes as C
import tempfile
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import abi
from .params import write_par

# keys the reference parser knows (src/parameter.c:65-95); the rest are extensions
REFERENCE_KEYS = {
    "xlength", "ylength", "zlength", "imax", "jmax", "kmax", "itermax", "levels",
    "presmooth", "postsmooth", "eps", "omg", "re", "tau", "gamma", "dt", "te",
    "gx", "gy", "gz", "name", "bcLeft", "bcRight", "bcBottom", "bcTop", "bcFront",
    "bcBack", "u_init", "v_init", "w_init", "p_init",
}


@dataclass
class StepInfo:
    nt: int        # steps done after this one
    t: float       # time after this step
    dt: float      # step size used
    res: float     # value solve() returned
    it: int        # solver iterations (RB) / V-cycles (MG); 0 for mg-ref


class Simulation:
    """One NuSiF case on the GPU, driven through the C ABI."""

    def __init__(self, par: str | Path | dict):
        self.lib = abi.load_library()
        lib = self.lib
        self._tmp = None
        if isinstance(par, dict):
            self._tmp = tempfile.TemporaryDirectory(prefix="nusif_")
            par = write_par(Path(self._tmp.name) / "case.par", par)
        self.par_path = str(par)
        self.param = abi.Parameter()
        lib.initParameter(C.byref(self.param))
        lib.readParameter(C.byref(self.param), self.par_path.encode())
        abi.check(lib)
        self.d = abi.Discretization()
        lib.initDiscretization(C.byref(self.d), C.byref(self.param))
        abi.check(lib)
        self.s = abi.Solver()
        lib.initSolver(C.byref(self.s), C.byref(self.d), C.byref(self.param))
        abi.check(lib)
        self.t = 0.0
        self.nt = 0
        self._closed = False

    # ---- geometry ----
    @property
    def dims(self) -> tuple[int, int, int]:
        g = self.d.grid
        return g.imax, g.jmax, g.kmax

    @property
    def padded_shape(self) -> tuple[int, int, int]:
        i, j, k = self.dims
        return (k + 2, j + 2, i + 2)

    @property
    def dt(self) -> float:
        return self.d.dt

    @property
    def te(self) -> float:
        return self.d.te

    # ---- fields ----
    def field(self, name: str) -> np.ndarray:
        out = np.empty(self.padded_shape, dtype=np.float64)
        self.lib.nusifDownloadField(C.byref(self.d), abi.FIELD_INDEX[name],
                                    out.ctypes.data_as(abi.c_double_p))
        abi.check(self.lib)
        return out

    def set_field(self, name: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.padded_shape)
        self.lib.nusifUploadField(C.byref(self.d), abi.FIELD_INDEX[name],
                                  a.ctypes.data_as(abi.c_double_p))
        abi.check(self.lib)

    # ---- reference operators, one C-ABI call each ----
    def _call(self, name: str) -> None:
        getattr(self.lib, name)(C.byref(self.d))
        abi.check(self.lib)

    def compute_timestep(self): self._call("computeTimestep")
    def set_boundary_conditions(self): self._call("setBoundaryConditions")
    def set_special_boundary_condition(self): self._call("setSpecialBoundaryCondition")
    def compute_fg(self): self._call("computeFG")
    def compute_rhs(self): self._call("computeRHS")
    def normalize_pressure(self): self._call("normalizePressure")
    def adapt_uv(self): self._call("adaptUV")

    def set_guess_net(self, net) -> None:
        """Warm-start every later solve with the network (None: plain warm start)."""
        self.lib.nusifSolverSetGuessNet(C.byref(self.s), net.handle if net is not None else None)
        abi.check(self.lib)

    def record_pair(self, x, t) -> None:
        """The next solve writes its features into x and its target into t
        (float32 CUDA tensors [kmax/2][jmax/2][imax/2][2] and [..])."""
        self.lib.nusifSolverRecordPair(C.byref(self.s), C.c_void_p(x.data_ptr()),
                                       C.c_void_p(t.data_ptr()))
        abi.check(self.lib)

    def guess_stats(self) -> tuple[bool, float, float]:
        """(guess taken, relative residual of the plain warm start, of the guess)."""
        used, rw, rg = C.c_int(), C.c_double(), C.c_double()
        self.lib.nusifSolverGuessStats(C.byref(self.s), C.byref(used), C.byref(rw), C.byref(rg))
        abi.check(self.lib)
        return bool(used.value), rw.value, rg.value

    def guess_counts(self) -> tuple[int, int]:
        """(network evaluations, guesses taken) since set_guess_net."""
        ev, tk = C.c_longlong(), C.c_longlong()
        self.lib.nusifSolverGuessCounts(C.byref(self.s), C.byref(ev), C.byref(tk))
        abi.check(self.lib)
        return ev.value, tk.value

    def solve(self) -> float:
        res = self.lib.solve(C.byref(self.s), self.d.p, self.d.rhs)
        abi.check(self.lib)
        return res

    @property
    def iterations(self) -> int:
        return self.lib.nusifSolverIterations(C.byref(self.s))

    # ---- the time loop body, reference src/main.c:61-79 ----
    def step(self, after_solve=None) -> StepInfo:
        """One time step. ``after_solve``: called between solve() and adaptUV
        (p is final there: a queued download of p can overlap adaptUV)."""
        if self.d.tau > 0.0:
            self.compute_timestep()
        self.set_boundary_conditions()
        self.set_special_boundary_condition()
        self.compute_fg()
        self.compute_rhs()
        if self.nt % 100 == 0:
            self.normalize_pressure()
        res = self.solve()
        it = self.iterations
        if after_solve is not None:
            after_solve()
        self.adapt_uv()
        dt = self.d.dt
        self.t += dt
        self.nt += 1
        return StepInfo(self.nt, self.t, dt, res, it)

    def run(self, max_steps: int | None = None, callback=None,
            residual_file: str | Path | None = None) -> list[StepInfo]:
        """``while (t <= te)`` (src/main.c:60), optionally capped at max_steps.

        ``residual_file``: write the reference's residual.dat, one "%f, %f" line
        of (time at the start of the step, solve() result) per step
        (src/main.c:74-76, src/progress.c:63-66)."""
        out = []
        fh = open(residual_file, "w") if residual_file else None
        try:
            while self.t <= self.te and (max_steps is None or len(out) < max_steps):
                t0 = self.t
                info = self.step()
                out.append(info)
                if fh:
                    fh.write("%f, %f\n" % (t0, info.res))
                if callback:
                    callback(self, info)
        finally:
            if fh:
                fh.close()
        return out

    # ---- output (reference src/main.c:97-143) ----
    def collect(self) -> dict[str, np.ndarray]:
        """Cell-centred u, v, w and interior p, shape (kmax, jmax, imax)
        (commCollectResult, src/comm.c:327-477)."""
        i, j, k = self.dims
        out = {f: np.empty((k, j, i), dtype=np.float64) for f in "uvwp"}
        self.lib.nusifCollectResult(C.byref(self.d), *(out[f].ctypes.data_as(abi.c_double_p)
                                                       for f in "uvwp"))
        abi.check(self.lib)
        return out

    def write_vtk(self, path: str | Path, binary: bool = False) -> None:
        """The reference's <problem>.vtk (src/vtkWriter-seq.c)."""
        self.lib.nusifWriteVTK(C.byref(self.d), str(path).encode(), int(binary))
        abi.check(self.lib)

    def close(self) -> None:
        if self._closed:
            return
        self.lib.nusifFreeSolver(C.byref(self.s))
        self.lib.nusifFreeDiscretization(C.byref(self.d))
        self._closed = True
        if self._tmp is not None:
            self._tmp.cleanup()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
