"""CPU oracle of the NuSiF hot path -- TEST INFRASTRUCTURE ONLY.

Loads ``liboracle.so`` (oracle/nusif_oracle.c, a C restatement of the
reference algorithms) and, where it was built from the reference sources,
``_ref/libnusif_ref_*.so`` (the reference itself, oracle/build_ref.sh).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
and only as the checker or the timed CPU baseline, never as the product.

Parity status: pinned. tests/test_oracle_pin.py checks this restatement
bit-for-bit against the reference compiled from source (here), and against
golden vectors the reference produced (tests/golden/, everywhere).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"


def reference_source_root() -> Path | None:
    """The reference tree oracle/build_ref.sh compiled from (NUSIF_REFERENCE
    overrides it), or None where the reference has not been built here."""
    env = os.environ.get("NUSIF_REFERENCE")
    if env:
        return Path(env)
    rec = REF_DIR / "source_root.txt"
    if rec.exists():
        root = Path(rec.read_text().strip())
        if (root / "src").is_dir():
            return root
    return None
LIB_STRICT = HERE / "liboracle.so"
LIB_FAST = HERE / "liboracle_fast.so"
SRC = HERE / "nusif_oracle.c"
SOURCES = [SRC, HERE / "nusif_oracle_mg.c"]
DEPS = SOURCES + [HERE / "nusif_oracle.h", HERE / "nusif_oracle_mg.inc"]

# strict: no fast-math, no FMA contraction (bit-for-bit pin against the
# reference's strict build); fast: the reference's own -O3 -ffast-math
FLAGS = {
    LIB_STRICT: ["-O2", "-ffp-contract=off"],
    LIB_FAST: ["-O3", "-ffast-math"],
}

d_p = C.POINTER(C.c_double)


def build(force: bool = False) -> None:
    cc = os.environ.get("CC", "gcc")
    for lib, opt in FLAGS.items():
        if not force and lib.exists() and lib.stat().st_mtime >= max(
                d.stat().st_mtime for d in DEPS):
            continue
        tmp = lib.with_suffix(".so.tmp")
        subprocess.run([cc, "-std=c99", "-shared", "-fPIC", *opt, "-o", str(tmp),
                        *map(str, SOURCES), "-lm"], check=True)
        os.replace(tmp, lib)


class OrGrid(C.Structure):
    _fields_ = [("imax", C.c_int), ("jmax", C.c_int), ("kmax", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double)]


class OrCase(C.Structure):
    _fields_ = [("imax", C.c_int), ("jmax", C.c_int), ("kmax", C.c_int),
                ("xlength", C.c_double), ("ylength", C.c_double), ("zlength", C.c_double),
                ("re", C.c_double), ("gamma", C.c_double), ("tau", C.c_double),
                ("te", C.c_double), ("dt0", C.c_double),
                ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double),
                ("u_init", C.c_double), ("v_init", C.c_double), ("w_init", C.c_double),
                ("p_init", C.c_double),
                ("bc", C.c_int * 6), ("problem", C.c_int),
                ("lid", C.c_double), ("inflow", C.c_double),
                ("eps", C.c_double), ("omega", C.c_double), ("itermax", C.c_int),
                ("solver", C.c_int), ("levels", C.c_int), ("presmooth", C.c_int),
                ("postsmooth", C.c_int), ("rtol", C.c_double), ("mg_levels", C.c_int),
                ("mg_pre", C.c_int), ("mg_post", C.c_int), ("mg_coarse", C.c_int),
                ("mg_cycles", C.c_int), ("mg_inner", C.c_int)]


class OrState(C.Structure):
    _fields_ = [("g", OrGrid), ("c", OrCase),
                ("u", d_p), ("v", d_p), ("w", d_p), ("p", d_p), ("rhs", d_p),
                ("f", d_p), ("gf", d_p), ("h", d_p),
                ("dt", C.c_double), ("t", C.c_double), ("dtBound", C.c_double),
                ("nt", C.c_int)]


_libs: dict[Path, C.CDLL] = {}


def load(fast: bool = False) -> C.CDLL:
    path = LIB_FAST if fast else LIB_STRICT
    if path in _libs:
        return _libs[path]
    if not path.exists():
        build()
    lib = C.CDLL(str(path))
    lib.or_max_abs.restype = C.c_double
    lib.or_max_abs.argtypes = [d_p, C.c_size_t]
    lib.or_timestep.restype = C.c_double
    lib.or_timestep.argtypes = [C.c_double] * 8
    lib.or_normalize_pressure.restype = C.c_double
    lib.or_solve_rb.restype = C.c_int
    lib.or_solve_rb.argtypes = [C.POINTER(OrGrid), C.c_double, C.c_double, C.c_int, d_p, d_p,
                                d_p]
    lib.or_solve_mg_ref.restype = C.c_double
    lib.or_solve_mg_ref.argtypes = [C.POINTER(OrGrid), C.c_double, C.c_int, C.c_int, C.c_int,
                                    d_p, d_p]
    lib.or_mg_solve.restype = C.c_int
    lib.or_mg_solve.argtypes = [C.POINTER(OrGrid), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                C.c_int, C.c_int, C.c_double, d_p, d_p, d_p]
    lib.or_mg_levels.restype = C.c_int
    lib.or_mg_levels.argtypes = [C.POINTER(OrGrid), C.c_int, C.POINTER(C.c_int)]
    lib.or_state_init.argtypes = [C.POINTER(OrState), C.POINTER(OrCase)]
    lib.or_state_step.argtypes = [C.POINTER(OrState), d_p]
    lib.or_state_step.restype = C.c_int
    lib.or_state_free.argtypes = [C.POINTER(OrState)]
    _libs[path] = lib
    return lib


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(d_p)


def grid(imax: int, jmax: int, kmax: int, xl=1.0, yl=1.0, zl=1.0) -> OrGrid:
    return OrGrid(imax, jmax, kmax, xl / imax, yl / jmax, zl / kmax)


PROBLEMS = {"dcavity": 1, "canal": 2}


def case_from_values(v: dict, solver: str = "rb") -> OrCase:
    """OrCase from a .par value dict (nusif.params style)."""
    c = OrCase()
    c.imax, c.jmax, c.kmax = v["imax"], v["jmax"], v["kmax"]
    c.xlength, c.ylength, c.zlength = v["xlength"], v["ylength"], v["zlength"]
    c.re, c.gamma, c.tau, c.te, c.dt0 = v["re"], v["gamma"], v["tau"], v["te"], v["dt"]
    c.gx, c.gy, c.gz = v["gx"], v["gy"], v["gz"]
    c.u_init, c.v_init, c.w_init, c.p_init = v["u_init"], v["v_init"], v["w_init"], v["p_init"]
    for q, key in enumerate(["bcLeft", "bcRight", "bcBottom", "bcTop", "bcFront", "bcBack"]):
        c.bc[q] = v[key]
    c.problem = PROBLEMS.get(v["name"], 0)
    c.lid = v.get("lid", 1.0)
    c.inflow = v.get("inflow", 2.0)
    c.eps, c.omega, c.itermax = v["eps"], v["omg"], v["itermax"]
    c.solver = {"rb": 0, "mg-ref": 1, "mg": 2, "mg-mixed": 3}[solver]
    c.levels, c.presmooth, c.postsmooth = v["levels"], v["presmooth"], v["postsmooth"]
    c.rtol = v.get("rtol", 1e-6)
    c.mg_levels, c.mg_pre, c.mg_post = v.get("mg_levels", 0), v.get("mg_pre", 2), v.get("mg_post", 2)
    c.mg_coarse, c.mg_cycles = v.get("mg_coarse", 0), v.get("mg_cycles", 100)
    c.mg_inner = v.get("mg_inner", 4)
    return c


class OracleRun:
    """The reference time loop on the CPU oracle."""

    def __init__(self, values: dict, solver: str = "rb", fast: bool = False):
        self.lib = load(fast)
        self.case = case_from_values(values, solver)
        self.st = OrState()
        if self.lib.or_state_init(C.byref(self.st), C.byref(self.case)) != 0:
            raise MemoryError("oracle allocation failed")
        g = self.st.g
        self.shape = (g.kmax + 2, g.jmax + 2, g.imax + 2)

    def field(self, name: str) -> np.ndarray:
        p = getattr(self.st, {"g": "gf"}.get(name, name))
        n = int(np.prod(self.shape))
        return np.ctypeslib.as_array(p, shape=(n,)).reshape(self.shape)

    def step(self):
        res = C.c_double()
        it = self.lib.or_state_step(C.byref(self.st), C.byref(res))
        return it, res.value, self.st.dt, self.st.t

    def close(self):
        if self.st.u:
            self.lib.or_state_free(C.byref(self.st))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- the reference itself, compiled from source (available where built) ----

def _ref_path(solver: str, fast: bool) -> Path:
    kind = {"rb": "rb", "mg-ref": "mg", "mg": "mg"}[solver]
    return REF_DIR / f"libnusif_ref_{kind}{'_fast' if fast else ''}.so"


def ref_available(solver: str = "rb", fast: bool = False) -> bool:
    return _ref_path(solver, fast).exists()


class RefDriver:
    """The reference's own objects driven one time step at a time (oracle/ref_driver.c).

    The reference keeps its state in globals, so one driver per library file is
    live at a time (a new driver re-initialises it).
    """

    def __init__(self, par_path: str | Path, solver: str = "rb", fast: bool = False):
        path = _ref_path(solver, fast)
        if not path.exists():
            raise FileNotFoundError(f"{path} missing (run oracle/build_ref.sh)")
        lib = C.CDLL(str(path))
        lib.refdrv_init.argtypes = [C.c_char_p]
        lib.refdrv_step.argtypes = [d_p, C.POINTER(C.c_int), d_p, d_p]
        lib.refdrv_field.restype = d_p
        lib.refdrv_field.argtypes = [C.c_int]
        lib.refdrv_time.restype = C.c_double
        lib.refdrv_te.restype = C.c_double
        lib.refdrv_dt.restype = C.c_double
        lib.refdrv_set_dt.argtypes = [C.c_double]
        lib.refdrv_dtbound.restype = C.c_double
        lib.refdrv_solve.restype = C.c_double
        lib.refdrv_solve.argtypes = [C.POINTER(C.c_int)]
        lib.refdrv_read_parameter.argtypes = [C.c_char_p, C.c_void_p]
        self.lib = lib
        lib.refdrv_init(str(par_path).encode())
        dims = (C.c_int * 3)()
        lib.refdrv_dims(dims)
        self.dims = tuple(dims)
        i, j, k = self.dims
        self.shape = (k + 2, j + 2, i + 2)

    FIELDS = {"u": 0, "v": 1, "w": 2, "p": 3, "rhs": 4, "f": 5, "g": 6, "h": 7}

    def field(self, name: str) -> np.ndarray:
        p = self.lib.refdrv_field(self.FIELDS[name])
        n = int(np.prod(self.shape))
        return np.ctypeslib.as_array(p, shape=(n,)).reshape(self.shape)

    def step(self):
        res, it, dt, t = C.c_double(), C.c_int(), C.c_double(), C.c_double()
        self.lib.refdrv_step(C.byref(res), C.byref(it), C.byref(dt), C.byref(t))
        # the multigrid build prints no iteration count: report 0 like the library
        return max(it.value, 0), res.value, dt.value, t.value

    @property
    def te(self) -> float:
        return self.lib.refdrv_te()

    @property
    def t(self) -> float:
        return self.lib.refdrv_time()


# ---- single operators of the restatement on numpy arrays (padded layout) ----

BC_ORDER = ("bcLeft", "bcRight", "bcBottom", "bcTop", "bcFront", "bcBack")


def op_max_abs(a: np.ndarray) -> float:
    return load().or_max_abs(ptr(a), a.size)


def op_timestep(g: OrGrid, dtbound: float, u, v, w, tau: float) -> float:
    lib = load()
    return lib.or_timestep(dtbound, g.dx, g.dy, g.dz, op_max_abs(u), op_max_abs(v),
                           op_max_abs(w), tau)


def op_set_bc(g: OrGrid, bc, u, v, w) -> None:
    arr = (C.c_int * 6)(*bc)
    load().or_set_bc(C.byref(g), arr, ptr(u), ptr(v), ptr(w))


def op_special_bc(g: OrGrid, problem: str, u, lid: float = 1.0, inflow: float = 2.0) -> None:
    load().or_special_bc(C.byref(g), C.c_int(PROBLEMS.get(problem, 0)), C.c_double(lid),
                         C.c_double(inflow), ptr(u))


def op_fgh(g: OrGrid, re, gamma, gx, gy, gz, dt, u, v, w, f, gf, h) -> None:
    d = C.c_double
    load().or_compute_fgh(C.byref(g), d(re), d(gamma), d(gx), d(gy), d(gz), d(dt), ptr(u),
                          ptr(v), ptr(w), ptr(f), ptr(gf), ptr(h))


def op_rhs(g: OrGrid, dt, f, gf, h, rhs) -> None:
    load().or_compute_rhs(C.byref(g), C.c_double(dt), ptr(f), ptr(gf), ptr(h), ptr(rhs))


def op_normalize(g: OrGrid, p) -> float:
    return load().or_normalize_pressure(C.byref(g), ptr(p))


def op_adapt(g: OrGrid, dt, f, gf, h, p, u, v, w) -> None:
    load().or_adapt_uv(C.byref(g), C.c_double(dt), ptr(f), ptr(gf), ptr(h), ptr(p), ptr(u),
                       ptr(v), ptr(w))


def op_solve_rb(g: OrGrid, eps, omega, itermax, p, rhs):
    res = C.c_double()
    it = load().or_solve_rb(C.byref(g), eps, omega, itermax, ptr(p), ptr(rhs), C.byref(res))
    return it, res.value


def op_solve_mg_ref(g: OrGrid, omega, levels, presmooth, postsmooth, p, rhs) -> float:
    return load().or_solve_mg_ref(C.byref(g), omega, levels, presmooth, postsmooth, ptr(p),
                                  ptr(rhs))


def op_mg_solve(g: OrGrid, mode: str, p, rhs, rtol=1e-6, pre=2, post=2, coarse_sweeps=0,
                maxcycles=100, level_cap=0, inner=4):
    """The library's corrected V-cycle solvers ("mg": FP64, "mg-mixed": FP32 in FP64).
    coarse_sweeps 0: exact coarsest solve; inner: FP32 V-cycles per FP64 residual."""
    rel = C.c_double()
    cyc = load().or_mg_solve(C.byref(g), {"mg": 0, "mg-mixed": 1}[mode], level_cap, pre, post,
                             coarse_sweeps, inner, maxcycles, rtol, ptr(p), ptr(rhs),
                             C.byref(rel))
    return cyc, rel.value


def op_mg_levels(g: OrGrid, cap: int = 0):
    dims = (C.c_int * 48)()
    n = load().or_mg_levels(C.byref(g), cap, dims)
    return [tuple(dims[3 * l:3 * l + 3]) for l in range(n)]
