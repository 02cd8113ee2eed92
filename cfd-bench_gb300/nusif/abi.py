"""ctypes mirror of include/nusif_gb300.h (the library's C ABI).

The struct layouts are the reference's (HPC-Dwarfs/CFD-Bench src/grid.h,
src/comm.h, src/parameter.h, src/discretization.h, src/solver.h, sequential
build). Loading fails loudly when the built library is missing: there is no
fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_DIR / "lib" / "libnusif_gb300.so"

c_double_p = C.POINTER(C.c_double)


class Grid(C.Structure):  # src/grid.h:8-12
    _fields_ = [("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("imax", C.c_int), ("jmax", C.c_int), ("kmax", C.c_int),
                ("xlength", C.c_double), ("ylength", C.c_double), ("zlength", C.c_double)]


class CommType(C.Structure):  # src/comm.h:33-44 (sequential)
    _fields_ = [("rank", C.c_int), ("size", C.c_int), ("neighbours", C.c_int * 6),
                ("coords", C.c_int * 3), ("dims", C.c_int * 3),
                ("imaxLocal", C.c_int), ("jmaxLocal", C.c_int), ("kmaxLocal", C.c_int)]


class Parameter(C.Structure):  # src/parameter.h:8-19
    _fields_ = [("imax", C.c_int), ("jmax", C.c_int), ("kmax", C.c_int),
                ("xlength", C.c_double), ("ylength", C.c_double), ("zlength", C.c_double),
                ("itermax", C.c_int), ("eps", C.c_double), ("omg", C.c_double),
                ("re", C.c_double), ("tau", C.c_double), ("gamma", C.c_double),
                ("te", C.c_double), ("dt", C.c_double),
                ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double),
                ("name", C.c_char_p),
                ("bcLeft", C.c_int), ("bcRight", C.c_int), ("bcBottom", C.c_int),
                ("bcTop", C.c_int), ("bcFront", C.c_int), ("bcBack", C.c_int),
                ("u_init", C.c_double), ("v_init", C.c_double), ("w_init", C.c_double),
                ("p_init", C.c_double),
                ("levels", C.c_int), ("presmooth", C.c_int), ("postsmooth", C.c_int)]


_FIELDS8 = [("p", c_double_p), ("rhs", c_double_p), ("f", c_double_p), ("g", c_double_p),
            ("h", c_double_p), ("u", c_double_p), ("v", c_double_p), ("w", c_double_p)]
_SCALARS = [("eps", C.c_double), ("omega", C.c_double), ("re", C.c_double),
            ("tau", C.c_double), ("gamma", C.c_double), ("gx", C.c_double),
            ("gy", C.c_double), ("gz", C.c_double), ("itermax", C.c_int),
            ("dt", C.c_double), ("te", C.c_double), ("dtBound", C.c_double),
            ("problem", C.c_char_p),
            ("bcLeft", C.c_int), ("bcRight", C.c_int), ("bcBottom", C.c_int),
            ("bcTop", C.c_int), ("bcFront", C.c_int), ("bcBack", C.c_int)]


class Discretization(C.Structure):  # src/discretization.h:14-32
    _fields_ = [("grid", Grid)] + _FIELDS8 + _SCALARS + [("comm", CommType)]


class Solver(C.Structure):  # src/solver.h:12-33
    _fields_ = ([("grid", C.POINTER(Grid))] + _FIELDS8 + _SCALARS +
                [("r", C.POINTER(c_double_p)), ("e", C.POINTER(c_double_p)),
                 ("levels", C.c_int), ("presmooth", C.c_int), ("postsmooth", C.c_int),
                 ("comm", C.POINTER(CommType))])


NUSIF_ERRORS_EXIT, NUSIF_ERRORS_RECORD = 0, 1
FIELD_INDEX = {"u": 0, "v": 1, "w": 2, "p": 3, "rhs": 4, "f": 5, "g": 6, "h": 7}

# (name, restype, argtypes) of every entry point declared in include/nusif_gb300.h
SIGNATURES = [
    ("initParameter", None, [C.POINTER(Parameter)]),
    ("readParameter", None, [C.POINTER(Parameter), C.c_char_p]),
    ("printParameter", None, [C.POINTER(Parameter)]),
    ("initDiscretization", None, [C.POINTER(Discretization), C.POINTER(Parameter)]),
    ("computeTimestep", None, [C.POINTER(Discretization)]),
    ("setBoundaryConditions", None, [C.POINTER(Discretization)]),
    ("setSpecialBoundaryCondition", None, [C.POINTER(Discretization)]),
    ("computeFG", None, [C.POINTER(Discretization)]),
    ("computeRHS", None, [C.POINTER(Discretization)]),
    ("normalizePressure", None, [C.POINTER(Discretization)]),
    ("adaptUV", None, [C.POINTER(Discretization)]),
    ("initSolver", None, [C.POINTER(Solver), C.POINTER(Discretization), C.POINTER(Parameter)]),
    ("solve", C.c_double, [C.POINTER(Solver), c_double_p, c_double_p]),
    ("nusifSetErrorMode", None, [C.c_int]),
    ("nusifGetLastError", C.c_int, [C.c_char_p, C.c_int]),
    ("nusifSetStream", None, [C.c_void_p]),
    ("nusifGetStream", C.c_void_p, []),
    ("nusifDownloadField", C.c_int, [C.POINTER(Discretization), C.c_int, c_double_p]),
    ("nusifUploadField", C.c_int, [C.POINTER(Discretization), C.c_int, c_double_p]),
    ("nusifUploadFieldAsync", C.c_int, [C.POINTER(Discretization), C.c_int, c_double_p]),
    ("nusifDownloadFieldAsync", C.c_int, [C.POINTER(Discretization), C.c_int, c_double_p]),
    ("nusifWaitCopies", C.c_int, []),
    ("nusifSolverIterations", C.c_int, [C.POINTER(Solver)]),
    ("nusifParameterSet", C.c_int, [C.POINTER(Parameter), C.c_char_p, C.c_char_p]),
    ("nusifFreeDiscretization", None, [C.POINTER(Discretization)]),
    ("nusifFreeSolver", None, [C.POINTER(Solver)]),
    ("nusifSolveRBStatic", C.c_int, [c_double_p, c_double_p, C.c_int, C.c_int, C.c_int,
                                     C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_int, c_double_p, C.POINTER(C.c_int)]),
    ("nusifCollectResult", C.c_int, [C.POINTER(Discretization), c_double_p, c_double_p,
                                     c_double_p, c_double_p]),
    ("nusifWriteVTK", C.c_int, [C.POINTER(Discretization), C.c_char_p, C.c_int]),
    ("nusifBatchCreate", C.c_void_p, [C.c_int, C.POINTER(C.c_char_p), C.c_int, C.c_int]),
    ("nusifBatchStep", C.c_int, [C.c_void_p, C.c_int]),
    ("nusifBatchSize", C.c_int, [C.c_void_p]),
    ("nusifBatchInstance", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.POINTER(Discretization)),
                                     C.POINTER(C.POINTER(Solver))]),
    ("nusifBatchStats", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("nusifBatchFree", None, [C.c_void_p]),
    ("nusifLaunchCount", C.c_ulonglong, []),
    ("nusifTimestepCounts", C.c_int, [C.POINTER(Discretization), C.POINTER(C.c_longlong),
                                      C.POINTER(C.c_longlong)]),
    ("nusifTimeKernel", C.c_int, [C.POINTER(Solver), c_double_p, c_double_p, C.c_int, C.c_int,
                                  C.POINTER(C.c_double)]),
    ("nusifVersion", C.c_char_p, []),
    ("nusifUNetCreate", C.c_void_p, [C.c_ulonglong]),
    ("nusifUNetFree", None, [C.c_void_p]),
    ("nusifUNetParamCount", C.c_longlong, [C.c_void_p]),
    ("nusifUNetGetParams", C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    ("nusifUNetSetParams", C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    ("nusifUNetGetGrads", C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    ("nusifUNetForward", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_void_p]),
    ("nusifUNetSetTensorCore", C.c_int, [C.c_void_p, C.c_int]),
    ("nusifUNetTrainStep", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                     C.c_int, C.c_int, C.c_float, C.c_int,
                                     C.POINTER(C.c_float)]),
    ("nusifSmoothRBF32", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                   C.c_int, C.c_double, C.c_double, C.c_double, C.c_int]),
    ("nusifConvertF64ToF32", C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    ("nusifConvertF32ToF64", C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    ("nusifSolverSetGuessNet", C.c_int, [C.POINTER(Solver), C.c_void_p]),
    ("nusifSolverRecordPair", C.c_int, [C.POINTER(Solver), C.c_void_p, C.c_void_p]),
    ("nusifSolverGuessStats", C.c_int, [C.POINTER(Solver), C.POINTER(C.c_int),
                                        C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("nusifSolverGuessCounts", C.c_int, [C.POINTER(Solver), C.POINTER(C.c_longlong),
                                         C.POINTER(C.c_longlong)]),
]

_lib = None


class NusifError(RuntimeError):
    """A library call reported an error (record mode)."""


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load the built library once; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is not built: run `python cfd-bench_gb300/build.py` "
            "(the GPU library has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    lib.nusifSetErrorMode(NUSIF_ERRORS_RECORD)
    if path is None:
        _lib = lib
    return lib


def check(lib: C.CDLL | None = None) -> None:
    """Raise NusifError if the last call recorded an error."""
    lib = lib or load_library()
    buf = C.create_string_buffer(1024)
    code = lib.nusifGetLastError(buf, 1024)
    if code:
        raise NusifError(f"nusif error {code}: {buf.value.decode(errors='replace')}")
