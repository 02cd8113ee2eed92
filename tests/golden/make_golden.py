"""Generate the golden vectors of tests/golden/ from the reference itself.

Runs the reference NuSiF sources, compiled from source by oracle/build_ref.sh
with the reference's own flags (-O3 -ffast-math, sequential), through
oracle/ref_driver.c, and stores what they produce:

  kat_ops.npz       one call of each reference operator on one set of seeded
                    random fields (9 x 7 x 5 cells): inputs, changed outputs
  run_<case>.npz    short whole runs: per-step iterations, residual, dt, t and
                    the padded u, v, w, p after selected steps
  config1_rb.npz    the 64^3 cavity (Re 1000, tau 0.5, te 1.0, RB omega 1.7,
                    eps 1e-3, itermax 500): per-step iterations, residual, dt
                    for all steps, plus the final fields sampled on every
                    4th interior cell and whole-field sums

Usage (needs the reference sources, i.e. this container):
    oracle/build_ref.sh && python tests/golden/make_golden.py [--skip-config1]
"""
from __future__ import annotations

import argparse
import ctypes as C
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "cfd-bench_gb300"))

import oracle  # noqa: E402
from nusif.params import cavity, config1, write_par, DCAVITY  # noqa: E402

OUT = Path(__file__).resolve().parent
SEED = 20261203


def run_case(name: str, values: dict, solver: str, steps: int, keep: list[int]) -> None:
    with tempfile.TemporaryDirectory() as d:
        par = write_par(Path(d) / "case.par", values)
        ref = oracle.RefDriver(par, solver, fast=True)
        rec = {"it": [], "res": [], "dt": [], "t": []}
        fields = {}
        for s in range(1, steps + 1):
            it, res, dt, t = ref.step()
            rec["it"].append(it)
            rec["res"].append(res)
            rec["dt"].append(dt)
            rec["t"].append(t)
            if s in keep:
                for f in "uvwp":
                    fields[f"{f}_{s}"] = ref.field(f).copy()
    np.savez_compressed(
        OUT / f"run_{name}.npz",
        values=np.array(repr(values)), solver=np.array(solver), keep=np.array(keep),
        it=np.array(rec["it"], dtype=np.int64), res=np.array(rec["res"]),
        dt=np.array(rec["dt"]), t=np.array(rec["t"]), **fields)
    print(f"run_{name}: {steps} steps, it={rec['it']}")


CHANGES = {"timestep": "", "bc": "uvw", "special": "u", "fg": "fgh", "rhs": ["rhs"],
           "normalize": "p", "adapt": "uvw", "solve": "p"}


def kat_ops() -> None:
    """Each reference operator once, from one set of seeded random fields."""
    rng = np.random.default_rng(SEED)
    vals = cavity((9, 7, 5), xlength=1.3, ylength=0.7, zlength=0.9, re=250.0, gamma=0.8,
                  gx=0.1, gy=-0.2, gz=0.05, te=1e9, tau=0.5, omg=1.6, eps=1e-9, itermax=7)
    out = {"values": np.array(repr(vals)), "dt_in": np.array(0.013)}
    names = ("u", "v", "w", "p", "rhs", "f", "g", "h")
    with tempfile.TemporaryDirectory() as d:
        par = write_par(Path(d) / "case.par", vals)
        ref = oracle.RefDriver(par, "rb", fast=True)
        lib = ref.lib
        inputs = {f: rng.standard_normal(ref.shape) for f in names}
        for f in names:
            out[f"in_{f}"] = inputs[f]
        ops = [("timestep", lib.refdrv_compute_timestep), ("bc", lib.refdrv_set_bc),
               ("special", lib.refdrv_special_bc), ("fg", lib.refdrv_compute_fg),
               ("rhs", lib.refdrv_compute_rhs), ("normalize", lib.refdrv_normalize),
               ("adapt", lib.refdrv_adapt_uv), ("solve", None)]
        for op, fn in ops:
            for f in names:
                ref.field(f)[...] = inputs[f]
            lib.refdrv_set_dt(C.c_double(0.013))
            if fn is None:
                it = C.c_int()
                out["solve_res"] = np.array(lib.refdrv_solve(C.byref(it)))
                out["solve_it"] = np.array(it.value)
            else:
                fn()
            out[f"{op}_dt"] = np.array(lib.refdrv_dt())
            for f in CHANGES[op]:
                out[f"{op}_out_{f}"] = ref.field(f).copy()
        out["dtbound"] = np.array(lib.refdrv_dtbound())
    np.savez_compressed(OUT / "kat_ops.npz", **out)
    print("kat_ops: written")


def config1_run() -> None:
    vals = config1()
    with tempfile.TemporaryDirectory() as d:
        par = write_par(Path(d) / "config1.par", vals)
        ref = oracle.RefDriver(par, "rb", fast=True)
        its, ress, dts = [], [], []
        while ref.t <= ref.te:
            it, res, dt, t = ref.step()
            its.append(it)
            ress.append(res)
            dts.append(dt)
        sl = (slice(1, -1, 4),) * 3
        out = {f"{f}_sample": ref.field(f)[sl].copy() for f in "uvwp"}
        for f in "uvwp":
            a = ref.field(f)[1:-1, 1:-1, 1:-1]
            out[f"{f}_sum"] = np.array(a.sum())
            out[f"{f}_sumsq"] = np.array((a * a).sum())
    np.savez_compressed(OUT / "config1_rb.npz", values=np.array(repr(vals)),
                        it=np.array(its, dtype=np.int64), res=np.array(ress),
                        dt=np.array(dts), t_end=np.array(ref.t), **out)
    print(f"config1_rb: {len(its)} steps, {sum(its)} iterations")


# sampled cells of a 258^3 padded field: every 9th index on each axis, ghosts
# included (0, 9, ..., 252), so both red-black colours and the walls appear
CONFIG2_STRIDE = 9


def config2_run(solver: str, steps: int) -> None:
    """The 256^3 benchmark cavity (Re 1000, tau 0.5, gamma 0.9) stepped by the
    reference: red-black SOR with omega 1.7, eps 1e-6, itermax 10000 (about 15
    minutes of one core per step), or the reference's multigrid build with 6
    levels and 2 + 2 sweeps. Stored per step: iterations, residual, dt, t; after
    every step the u, v, w, p samples on a stride-9 lattice of the padded array
    and whole-interior sums and sums of squares."""
    vals = cavity(256, re=1000.0, tau=0.5, te=1e9, omg=1.7, eps=1e-6, itermax=10000,
                  gamma=0.9, levels=6, presmooth=2, postsmooth=2)
    name = "config2_rb" if solver == "rb" else "config2_mgref"
    with tempfile.TemporaryDirectory() as d:
        par = write_par(Path(d) / "config2.par", vals)
        ref = oracle.RefDriver(par, solver, fast=True)
        rec = {"it": [], "res": [], "dt": [], "t": []}
        out = {}
        sl = (slice(0, None, CONFIG2_STRIDE),) * 3
        for s in range(1, steps + 1):
            it, res, dt, t = ref.step()
            for key, v in zip(("it", "res", "dt", "t"), (it, res, dt, t)):
                rec[key].append(v)
            for f in "uvwp":
                a = ref.field(f)
                out[f"{f}_sample_{s}"] = a[sl].copy()
                inner = a[1:-1, 1:-1, 1:-1]
                out[f"{f}_sum_{s}"] = np.array(inner.sum())
                out[f"{f}_sumsq_{s}"] = np.array((inner * inner).sum())
            print(f"{name}: step {s} it={it} res={res!r}", flush=True)
    np.savez_compressed(OUT / f"{name}.npz", values=np.array(repr(vals)),
                        solver=np.array(solver), stride=np.array(CONFIG2_STRIDE),
                        it=np.array(rec["it"], dtype=np.int64), res=np.array(rec["res"]),
                        dt=np.array(rec["dt"]), t=np.array(rec["t"]), **out)
    print(f"{name}: {steps} steps written")


def program_outputs() -> None:
    """The reference program (src/main.c) end to end on a 10^3 cavity: its
    residual.dat and dcavity.vtk, as written by the reference's own writers."""
    import shutil
    import subprocess
    exe = oracle.REF_DIR / "NusifSolver-rb"
    vals = cavity(10, te=1.2, omg=1.7, eps=1e-3, itermax=100)
    with tempfile.TemporaryDirectory() as d:
        par = write_par(Path(d) / "cavity10.par", vals)
        subprocess.run([str(exe), str(par)], cwd=d, check=True, stdout=subprocess.DEVNULL)
        out = OUT / "program_cavity10"
        out.mkdir(exist_ok=True)
        shutil.copy(Path(d) / "residual.dat", out / "residual.dat")
        shutil.copy(Path(d) / "dcavity.vtk", out / "dcavity.vtk")
        (out / "case.par").write_text(par.read_text())
    print("program_cavity10: residual.dat, dcavity.vtk")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--skip-config1", action="store_true")
    ap.add_argument("--config2", action="store_true",
                    help="only the 256^3 benchmark runs (about 30 minutes of one core)")
    args = ap.parse_args()
    if not oracle.ref_available("rb", fast=True):
        sys.exit("reference not built: run oracle/build_ref.sh first")
    if args.config2:
        config2_run("mg-ref", 3)
        config2_run("rb", 2)
        return
    kat_ops()
    run_case("cavity8_rb", cavity(8, te=1e9, omg=1.7, eps=1e-3, itermax=500), "rb", 12,
             [1, 6, 12])
    run_case("ragged_rb", cavity((17, 9, 13), xlength=1.7, zlength=1.3, te=1e9, omg=1.7,
                                 eps=1e-4, itermax=300), "rb", 5, [5])
    run_case("canal_rb", dict(DCAVITY, name="canal", bcLeft=3, bcRight=3, re=100.0,
                              u_init=1.0, xlength=3.0, ylength=1.0, zlength=1.0,
                              imax=12, jmax=6, kmax=6, te=1e9, itermax=200, eps=1e-4),
             "rb", 6, [6])
    run_case("bcmix_rb", cavity((10, 8, 6), bcLeft=2, bcRight=3, bcBottom=2, bcTop=1,
                                bcFront=3, bcBack=4, gy=-0.5, te=1e9, eps=1e-3,
                                itermax=100), "rb", 5, [5])
    run_case("mgref_l3", cavity(10, te=1e9, omg=1.7, levels=3, presmooth=5, postsmooth=3),
             "mg-ref", 4, [4])
    run_case("mgref_l1", cavity((9, 7, 8), te=1e9, omg=1.7, levels=1, presmooth=4,
                                postsmooth=2), "mg-ref", 3, [3])
    run_case("cavity_tau0_rb", cavity(6, tau=-1.0, dt=0.01, te=1e9, eps=1e-3, itermax=50),
             "rb", 4, [4])
    program_outputs()
    if not args.skip_config1:
        config1_run()


if __name__ == "__main__":
    main()
