"""Benchmark of the NuSiF per-timestep hot path on GB300.

Workload: the 3D lid-driven cavity at 256^3 cells (Re 1000, tau 0.5,
donor-cell gamma 0.9), one time step per "step": CFL reduction, velocity
boundary conditions, F/G/H, RHS, pressure solve, velocity update, all
through the library's C ABI (reference src/main.c:61-79). The pressure solve
is selected with --solver:
  mg-mixed  FP32 V-cycles in FP64 iterative refinement to 1e-6 relative residual
  mg        FP64 V-cycles to 1e-6 relative residual
  rb        the reference's red-black SOR (omega 1.7, eps 1e-6, itermax 10000)

Output: one JSON line (rank 0). ``value`` is device-timed ms per time step with
the state resident in HBM (8 FP64 fields of 137 MB: inputs far larger than
L2, so no flush is needed); ``e2e`` is the same step through the C ABI with
u, v, w, p uploaded from and downloaded to pinned host buffers every step.

``--impl reference`` times the reference's CPU implementation of the same
step on this machine's host cores (the reference compiled from source in
oracle/_ref when present, else the oracle's C restatement built with the
reference's flags), on a bounded sample scaled to one time step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "cfd-bench_gb300"))

METRIC = "ms/timestep at 256^3 to 1e-6 residual: learned+FP32-MG vs FP64 MG; HBM GB/s"
UNIT = "ms/timestep"
PEAKS = ROOT / "MEASURED_PEAKS.json"
TRAFFIC = ROOT / "profiles" / "traffic.json"
FALLBACK_HBM_GBS = 6800.0
# the warm-start network the headline arm uses, trained by
#   python bench.py --workload learned --save-net <this file>
# (64 cavities at 128^3, Re ~ U[100, 5000], lid ~ U[0.5, 2], seeded)
NET_PATH = ROOT / "cfd-bench_gb300" / "nusif" / "weights" / "unet_cavity128.npz"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=10,
                    help="untimed steps: the first few steps from rest need more V-cycles")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--solver", default=os.environ.get("NUSIF_BENCH_SOLVER", "auto"))
    ap.add_argument("--n", type=int, default=256, help="cells per axis of the cavity")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--arith", default="df32", choices=["df32", "fp64"],
                    help="FP64-bound stencils (computeFG, the mixed solver's fine residual) "
                         "in FP32 pairs (df32) or FP64 instructions (fp64)")
    ap.add_argument("--guess", default="quadratic",
                    choices=["previous", "extrapolate", "quadratic", "cubic"],
                    help="initial pressure of each V-cycle solve: p(n-1), 2 p(n-1) - p(n-2), "
                         "3 p(n-1) - 3 p(n-2) + p(n-3), or 4 p(n-1) - 6 p(n-2) + 4 p(n-3) - p(n-4)")
    ap.add_argument("--batch-n", type=int, default=96, help="instances of the batch workload")
    ap.add_argument("--workload", default="cavity",
                    choices=["cavity", "channel", "batch", "learned"],
                    help="cavity: the 256^3 benchmark; channel: mixed vs FP64 error study; "
                         "batch: 96 uneven cavities; learned: the U-Net warm start")
    ap.add_argument("--learn-runs", type=int, default=64, help="training cavities (learned)")
    ap.add_argument("--learn-n", type=int, default=128, help="training cavity edge (learned)")
    ap.add_argument("--learn-steps", type=int, default=300, help="steps per training run")
    ap.add_argument("--learn-iters", type=int, default=2000, help="Adam iterations (learned)")
    ap.add_argument("--learn-batch", type=int, default=8, help="pairs per Adam step (learned)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--phases", action="store_true",
                    help="add a per-call split of the step and per-level FP32 V-cycle times")
    ap.add_argument("--no-roofline", action="store_true",
                    help="skip the per-kernel timing launches (clean launch lists for ncu)")
    ap.add_argument("--no-graph", action="store_true",
                    help="host-driven solves instead of one graph per solve (the same kernels, "
                         "visible one by one to a profiler's launch list)")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the FP64 multigrid comparison run")
    ap.add_argument("--itermax", type=int, default=None,
                    help="cap of the red-black iterations per step (short profiling runs)")
    ap.add_argument("--rb-steps", type=int, default=2,
                    help="time steps of the like-for-like red-black arm (the reference's solver "
                         "on the GPU, itermax 10000: about 3.6 s per step at 256^3); 0 skips it")
    ap.add_argument("--error-steps", type=int, default=None,
                    help="steps of the field-error study of the headline solver against FP64 "
                         "multigrid (default: warmup + steps)")
    ap.add_argument("--ref-sweeps", type=int, default=100,
                    help="red-black sweeps timed per step by the reference arm")
    ap.add_argument("--net", default=str(NET_PATH),
                    help="trained warm-start network (learn.save_params file) of the headline "
                         "arm: learned guess + mixed-precision multigrid")
    ap.add_argument("--no-learned", action="store_true",
                    help="headline without the learned warm start (mixed-precision MG alone)")
    ap.add_argument("--save-net", default=None,
                    help="--workload learned: write the trained network here")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def hbm_peak():
    try:
        d = json.loads(PEAKS.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self, window: tuple[float, float] | None = None) -> dict:
        """Median SM clock and the throttle reasons seen; with a window (host
        perf_counter times of the timed region), only the samples inside it
        (or the one nearest to it when none falls inside)."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if window is not None and lines:
            inside = [x for x in lines if window[0] <= x[0] <= window[1]]
            lines = inside or [min(lines, key=lambda x: abs(x[0] - 0.5 * (window[0] + window[1])))]
        for _, ln in lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# (pre-sweeps, post-sweeps, most FP32 V-cycles per FP64 residual, smoother
# relaxation omega) of each solver in the benchmark. FP64 multigrid: V(2,2)
# red-black Gauss-Seidel, the reference configuration's cycle. Mixed
# precision: V(1,1) with omega 1.3, at most 4 FP32 V-cycles per FP64
# residual, the FP32 correction stopped at 0.9 rtol (the library default
# mg_theta) - the fastest of the shapes measured at 256^3 with the quadratic
# warm start.
MG_SHAPE = {"mg": (2, 2, 4, 1.0), "mg-mixed": (1, 1, 4, 1.3)}
# learned warm start: once the network's guess lost twice in a row it is
# evaluated only every LEARNED_PROBE-th step until a guess is taken again
LEARNED_PROBE = 8
# the FP64 arm with the same kind of tuning: V(1,2), omega 1.3 (fastest FP64
# shape measured at 256^3 with the quadratic warm start)
MG_SHAPE_FP64_TUNED = (1, 2, 4, 1.3)


def bench_case(n: int, solver: str, itermax: int | None = None,
               guess: str = "previous", shape: tuple | None = None,
               graph: bool = True, arith: str = "df32") -> dict:
    from nusif.params import config2
    vals = config2(solver=solver)
    # fuse_dt: adaptUV keeps its velocity maxima, computeTimestep reads the ghost shell
    vals.update(imax=n, jmax=n, kmax=n, arith=arith, fuse_dt=1)
    if itermax is not None:
        vals["itermax"] = itermax
    if solver in ("mg", "mg-mixed"):
        pre, post, inner, omega = shape or MG_SHAPE[solver]
        vals.update(mg_guess=guess, mg_pre=pre, mg_post=post, mg_inner=inner, mg_omega=omega,
                    mg_graph=1 if graph else 0)
    return vals


def load_headline_net(args, solver: str):
    """The trained warm-start network of the headline arm (mixed-precision MG
    only), or None (--no-learned, another solver, or no weights file)."""
    if args.no_learned or solver != "mg-mixed" or not Path(args.net).exists():
        return None
    from nusif.learn import load_net
    return load_net(args.net)


def learned_meta(path) -> dict:
    try:
        from nusif.learn import saved_meta
        return saved_meta(path)
    except Exception:
        return {}


def pick_solver(requested: str) -> str:
    return "mg-mixed" if requested == "auto" else requested


# ---------------------------------------------------------------- GPU arm

def timed_steps(sim, args, stream, local, world):
    """W untimed steps, then K steps between CUDA events (max over ranks)."""
    import torch
    lib = sim.lib
    clocks = ClockSampler(local)  # started early: nvidia-smi takes a while to report
    clocks.start()
    for _ in range(args.warmup):
        sim.step()
    torch.cuda.synchronize()
    launches0 = lib.nusifLaunchCount()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    infos = [sim.step() for _ in range(args.steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    if world > 1:
        torch.distributed.barrier()
    launches = lib.nusifLaunchCount() - launches0
    clk = clocks.stop((t0, t1))
    ms = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
    return {"ms_per_step": ms / args.steps, "iters": [i.it for i in infos],
            "res": [i.res for i in infos], "launches": int(launches), "clocks": clk}


def max_over_ranks(ms: float, world: int, device: str) -> float:
    """The slowest rank's time (replicas: the job ends with the last one)."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms_per_step_max: float, world: int) -> float:
    """Whole-job ms per time step: N replicas each advance one cavity per step."""
    return ms_per_step_max / world


def run_gpu(args, rank, world, local):
    import torch

    import nusif

    torch.cuda.set_device(local)
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    lib = nusif.load_library()
    lib.nusifSetStream(C.c_void_p(stream.cuda_stream))

    solver = pick_solver(args.solver)
    vals = bench_case(args.n, solver, args.itermax, args.guess, graph=not args.no_graph,
                      arith=args.arith)
    net = load_headline_net(args, solver)
    if net is not None:
        vals.update(mg_probe=LEARNED_PROBE)
    sim = nusif.Simulation(vals)
    if net is not None:
        sim.set_guess_net(net)
    i, j, k = sim.dims
    ncell = i * j * k
    padded = (i + 2) * (j + 2) * (k + 2)
    head = timed_steps(sim, args, stream, local, world)
    learned = None
    if net is not None:
        ev, taken = sim.guess_counts()
        learned = {"network": str(Path(args.net).name), "probe_every_after_two_rejections":
                   LEARNED_PROBE, "evaluations_incl_warmup": ev, "guesses_taken_incl_warmup": taken,
                   "trained": learned_meta(args.net)}

    # ---- dominant kernels, timed live with CUDA events on the library stream ----
    roofs = [] if args.no_roofline else kernel_rooflines(sim, solver, stream, ncell, args.arith)
    live_shares(roofs, solver, head["iters"], head["ms_per_step"], MG_SHAPE["mg-mixed"][2])

    phases = step_phases(sim, solver, stream) if args.phases else None

    # ---- e2e: same step through the C ABI with host buffers ----
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(sim, args, stream, padded)
    sim.close()

    # ---- the same solver without the network ----
    if net is not None:
        sim0 = nusif.Simulation(bench_case(args.n, solver, args.itermax, args.guess,
                                           graph=not args.no_graph, arith=args.arith))
        alone = timed_steps(sim0, args, stream, local, world)
        sim0.close()
        learned.update({"ms_per_step_without_network": alone["ms_per_step"],
                        "v_cycles_per_step_without_network": alone["iters"],
                        "speedup_from_network": alone["ms_per_step"] / head["ms_per_step"]})

    # ---- the comparison the metric names: plain FP64 multigrid, same case ----
    # (previous-p guess: plain FP64 multigrid; and with this run's guess)
    compare = None
    if solver == "mg-mixed" and not args.no_compare:
        compare = []
        arms = [("previous", MG_SHAPE["mg"]), (args.guess, MG_SHAPE["mg"]),
                (args.guess, MG_SHAPE_FP64_TUNED)]
        for g, shape in dict.fromkeys(arms):
            sim64 = nusif.Simulation(bench_case(args.n, "mg", args.itermax, g, shape,
                                                graph=not args.no_graph, arith=args.arith))
            ref64 = timed_steps(sim64, args, stream, local, world)
            sim64.close()
            compare.append({"solver": "mg (FP64 V-cycles, same rtol 1e-6)", "guess": g,
                            "v_cycle": "V(%d,%d), omega %.2f" % (shape[0], shape[1], shape[3]),
                            "ms_per_step": ref64["ms_per_step"],
                            "v_cycles_per_step": ref64["iters"],
                            "residual_per_step": ref64["res"],
                            "speedup_of_value": ref64["ms_per_step"] / head["ms_per_step"],
                            "mlups": mlups(ref64["iters"], ncell, ref64["ms_per_step"])})

    errors = None
    if solver != "mg" and solver.startswith("mg") and not args.no_compare and rank == 0:
        n_err = args.error_steps if args.error_steps is not None else args.warmup + args.steps
        if n_err > 0:
            errors = field_error_study(args, stream, solver, n_err, net)

    rb = None
    if solver != "rb" and args.rb_steps > 0 and not args.no_compare:
        rb = rb_arm(args, stream, local, world)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(vals, solver, head["iters"], args.ref_sweeps)

    if net is not None:
        net.close()
    if rank != 0:
        return None
    tol = ("relative residual 1e-6 (mean-free rhs)" if solver.startswith("mg")
           else "eps 1e-6 (RMS), itermax %d" % vals["itermax"])
    out = {
        "metric": METRIC,
        "value": replica_value(head["ms_per_step"], world),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": head["ms_per_step"],
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if solver in ("rb", "mg", "mg-ref") else "f64+f32",
        "data": "synthetic: lid-driven cavity from rest, no dataset",
        "config": {"workload": f"lid-driven cavity {i}x{j}x{k}, Re 1000, tau 0.5, "
                               f"pressure solve {solver}"
                               + (" with the learned warm start" if net is not None else ""),
                   "cells": ncell, "solver": solver, "tolerance": tol,
                   "learned_warm_start": net is not None,
                   "initial_guess": (args.guess if solver in ("mg", "mg-mixed") else "previous"),
                   "v_cycle": ("V(%d,%d), up to %d FP32 V-cycles per FP64 residual, "
                               "red-black smoother omega %.2f, FP32 correction to 0.9 rtol"
                               % MG_SHAPE["mg-mixed"] if solver == "mg-mixed" else
                               "V(%d,%d), omega %.2f" % (MG_SHAPE["mg"][0], MG_SHAPE["mg"][1],
                                                         MG_SHAPE["mg"][3])
                               if solver == "mg" else None),
                   "arith": ("computeFG and the mixed solver's fine residual in FP32 pairs "
                             "(double-float, about 2^-47 of the operands)" if args.arith == "df32"
                             else "all FP64 stencils in FP64 instructions"),
                   "solve_launch": ("host-driven launches" if args.no_graph else
                                    "one CUDA graph per solve (device while-loops)"),
                   "cfl_maxima": "fuse_dt 1: from adaptUV's output plus the ghost shell",
                   "l2": "no flush: 8 FP64 fields of %.0f MB each, far larger than L2" % (padded * 8 / 1e6),
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "solver_iterations_per_step": head["iters"],
        "residual_per_step": head["res"],
        "mlups": mlups(head["iters"], ncell, head["ms_per_step"]),
        "learned": learned,
        "compare_fp64_mg": compare,
        "error_vs_fp64_mg": errors,
        "compare_rb": rb,
        "roofline": dominant(roofs),
        "roofline_kernels": roofs,
        "phases": phases,
        "e2e": e2e,
        "gpu_launches": head["launches"],
        "clocks": head["clocks"],
        "cpu_baseline": cpu,
    }
    return out


def mlups(iters: list[int], ncell: int, ms_per_step: float) -> dict:
    """The reference's solver throughput, MLUPS = iterations x imax*jmax*kmax x
    1e-6 / solver seconds (src/profiler.c:61-74), with the whole step's time
    as the denominator (so a lower bound of the solver-only figure); for the
    multigrid solvers an iteration is one V-cycle or refinement unit. Also the
    time-step rate, cells x steps / seconds."""
    it = sum(iters) / max(len(iters), 1)
    sec = ms_per_step * 1e-3
    return {"solver_mlups": it * ncell * 1e-6 / sec if sec > 0 else None,
            "iterations_per_step": it,
            "timestep_mlups": ncell * 1e-6 / sec if sec > 0 else None,
            "definition": "iterations x cells x 1e-6 / step seconds (src/profiler.c:61-74, "
                          "whole step as the solver time)"}


def field_error_study(args, stream, solver: str, steps: int, net=None) -> dict:
    """The headline solver and FP64 multigrid (V(2,2), same rtol and warm
    start) stepped side by side from rest: after every step the L2 and Linf
    differences of u, v, w (relative to the FP64 velocity field as a whole)
    and of the mean-free p (relative to the FP64 mean-free p)."""
    import torch

    import nusif
    tv = bench_case(args.n, solver, args.itermax, args.guess, arith=args.arith)
    if net is not None:
        tv.update(mg_probe=LEARNED_PROBE)
    # the reference arm is FP64 throughout: FP64 V-cycles and every stencil in
    # FP64 instructions (arith fp64), so the difference covers the pair arithmetic too
    sims = {"test": nusif.Simulation(tv),
            "fp64": nusif.Simulation(bench_case(args.n, "mg", args.itermax, args.guess,
                                                arith="fp64"))}
    if net is not None:
        sims["test"].set_guess_net(net)
    shape = sims["fp64"].padded_shape

    def view(sim, f):
        return torch.as_tensor(DeviceArray(getattr(sim.d, f), shape),
                               device="cuda")[1:-1, 1:-1, 1:-1]

    err = {f: {"l2": [], "linf": []} for f in "uvwp"}
    for _ in range(steps):
        for sim in sims.values():
            sim.step()
        torch.cuda.synchronize()
        vel = {f: view(sims["fp64"], f) for f in "uvw"}
        vel_l2 = float(torch.sqrt(sum(torch.linalg.vector_norm(vel[f]) ** 2 for f in "uvw")))
        vel_max = float(max(vel[f].abs().max() for f in "uvw"))
        for f in "uvwp":
            a, b = view(sims["test"], f), view(sims["fp64"], f)
            if f == "p":
                a, b = a - a.mean(), b - b.mean()
                l2_ref, max_ref = float(torch.linalg.vector_norm(b)), float(b.abs().max())
            else:
                l2_ref, max_ref = vel_l2, vel_max
            d = a - b
            err[f]["l2"].append(float(torch.linalg.vector_norm(d)) / max(l2_ref, 1e-300))
            err[f]["linf"].append(float(d.abs().max()) / max(max_ref, 1e-300))
    for sim in sims.values():
        sim.close()
    return {"against": "FP64 multigrid V(2,2), every stencil in FP64 instructions, same rtol "
                       "1e-6 and warm start, stepped alongside",
            "steps": steps,
            "max": {f: {k: max(v) for k, v in err[f].items()} for f in "uvwp"},
            "final": {f: {k: v[-1] for k, v in err[f].items()} for f in "uvwp"},
            "per_step_l2": {f: err[f]["l2"] for f in "uvwp"}}


def rb_arm(args, stream, local, world) -> dict:
    """The drop-in with the reference's own solver: red-black SOR (omega 1.7,
    eps 1e-6, itermax 10000) on the GPU, the like-for-like counterpart of the
    reference arm; args.rb_steps time steps from rest after one untimed step."""
    import torch

    import nusif
    vals = bench_case(args.n, "rb", args.itermax, arith=args.arith)
    sim = nusif.Simulation(vals)
    sim.step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    infos = [sim.step() for _ in range(args.rb_steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.rb_steps
    ncell = vals["imax"] * vals["jmax"] * vals["kmax"]
    sim.close()
    its = [i.it for i in infos]
    return {"solver": "rb (the reference's red-black SOR, omega 1.7, eps 1e-6, itermax %d)"
                      % vals["itermax"],
            "steps_timed": args.rb_steps, "ms_per_step": ms, "iterations_per_step": its,
            "ms_per_sweep": ms / (sum(its) / len(its)) if sum(its) else None,
            "mlups": mlups(its, ncell, ms)}


def step_phases(sim, solver, stream, steps: int = 10) -> dict:
    """Where a step's time goes: CUDA events between the reference calls of
    `steps` more steps (the time each call keeps the library stream busy,
    host-side waits of computeTimestep and solve included), and for
    mg-mixed the fine FP64 residual and one FP32 V-cycle from each level down
    (nusifTimeKernel, which replays the V-cycle as a captured graph)."""
    import torch
    names = ["computeTimestep", "setBoundaryConditions", "setSpecialBoundaryCondition",
             "computeFG", "computeRHS", "solve", "adaptUV"]
    calls = [sim.compute_timestep, sim.set_boundary_conditions,
             sim.set_special_boundary_condition, sim.compute_fg, sim.compute_rhs, sim.solve,
             sim.adapt_uv]
    acc = [0.0] * len(names)
    total = 0.0
    for _ in range(steps):
        if sim.nt % 100 == 0:
            sim.normalize_pressure()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
        ev[0].record(stream)
        for q, call in enumerate(calls):
            call()
            ev[q + 1].record(stream)
        sim.t += sim.d.dt
        sim.nt += 1
        torch.cuda.synchronize()
        for q in range(len(names)):
            acc[q] += ev[q].elapsed_time(ev[q + 1])
        total += ev[0].elapsed_time(ev[-1])
    out = {"ms_per_step": total / steps, "ms": {n: a / steps for n, a in zip(names, acc)}}
    if solver == "mg-mixed":
        ms = C.c_double()
        lib = sim.lib
        lib.nusifTimeKernel(C.byref(sim.s), sim.d.p, sim.d.rhs, 1, 20, C.byref(ms))
        out["fp64_residual_ms"] = ms.value
        levels = []
        for lv in range(16):
            if lib.nusifTimeKernel(C.byref(sim.s), sim.d.p, sim.d.rhs, 2 + lv, 20,
                                   C.byref(ms)) != 0:
                lib.nusifGetLastError(None, 0)  # past the coarsest level: clear it
                break
            levels.append(ms.value)
        out["fp32_vcycle_from_level_ms"] = levels
    return out


def _profile_entry(kernel: str) -> dict:
    try:
        return json.loads(TRAFFIC.read_text()).get(kernel) or {}
    except Exception:
        return {}


def _traffic(kernel: str, ncell: int):
    """DRAM bytes per launch of a kernel from the committed ncu summary, scaled by cells."""
    entry = _profile_entry(kernel)
    b = entry.get("bytes_per_cell_per_launch")
    return b * ncell if b is not None else None


def dominant(roofs: list[dict]):
    """The entry of the kernel with the largest share of the step's device time:
    the live share (launch time x launches per step / ms per step) where the
    launches per step are known, else the share in the committed ncu launch
    list of the same step; ties or missing shares keep the first entry."""
    if not roofs:
        return None
    return max(roofs, key=lambda r: r.get("share_of_step_live") or r.get("share_of_step") or 0.0)


def live_shares(roofs: list[dict], solver: str, iters, ms_per_step: float, inner: int) -> None:
    """Adds ``launches_per_step`` and ``share_of_step_live`` to each entry:
    computeFG runs once per step; the mixed solver's fine sweep twice per FP32
    V-cycle (the solve graph's finest level starts every V-cycle from the
    residual kernel's zeroed correction with a general sweep) and its fine
    residual once per refinement step plus once before the first; the FP64
    smoother's colour pass 2 x (pre + post) per V-cycle; a red-black SOR
    iteration two colour passes."""
    if not iters or not ms_per_step:
        return
    mean_it = sum(iters) / len(iters)
    pre, post = MG_SHAPE["mg"][0], MG_SHAPE["mg"][1]
    for r in roofs:
        k = r.get("kernel", "")
        n = None
        if k.startswith("k_fgh"):
            n = 1.0
        elif k.startswith("k_rbgs_sweep"):
            n = 2.0 * mean_it
        elif k.startswith("k_mx_residual"):
            n = sum(-(-it // inner) + 1 for it in iters) / len(iters)
        elif k.startswith("k_mg_smooth"):
            n = 2.0 * (pre + post) * mean_it
        elif k.startswith("k_sor_pass"):
            n = 2.0 * mean_it
        if n is not None:
            r["launches_per_step"] = n
            r["share_of_step_live"] = r["launch_ms"] * n / ms_per_step


# FP64 issue peak of a GB300: 2 FP64 lanes per SM and clock
# (sm__sass_thread_inst_executed_op_dfma_pred_on.sum.peak_sustained = 304 for 152
# SMs) at the maximum SM clock of MEASURED_PEAKS.json (2070 MHz)
FP64_LANES_PER_CLOCK = 304


def _fp64_pipe(inst_per_cell: float, ncell: int, ms: float) -> dict:
    """Achieved FP64 instruction rate of an FP64-pipe-bound kernel (instructions
    per cell counted from its source) against the GPU's FP64 issue peak."""
    mhz = 2070.0
    try:
        mhz = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["sm_max_mhz"])
    except Exception:
        pass
    peak = FP64_LANES_PER_CLOCK * mhz * 1e6
    achieved = inst_per_cell * ncell / (ms * 1e-3)
    return {"fp64_inst_per_cell": inst_per_cell, "fp64_inst_per_s": achieved,
            "fp64_inst_peak_per_s": peak, "fp64_pipe_frac": achieved / peak}


def _roof(name, kernel_key, ms, algo_bytes, ncell, peak, src, **extra):
    achieved = algo_bytes / (ms * 1e-3) / 1e9
    prof = _profile_entry(kernel_key)
    d = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
         "frac": achieved / peak, "traffic": _traffic(kernel_key, ncell), "kernel": name,
         "launch_ms": ms, "algorithmic_bytes_per_launch": algo_bytes,
         "peak_source": src + " (MEASURED_PEAKS.json hbm_gbs)" if src == "measured" else src,
         "share_of_step": prof.get("share_of_step"),
         "ncu": {k: prof[k] for k in ("fp64_pipe_frac", "fma_pipe_frac", "alu_pipe_frac",
                                      "issue_active", "dram_frac") if k in prof} or None}
    d.update(extra)
    return d


def kernel_rooflines(sim, solver, stream, ncell, arith: str = "df32"):
    """Average launch duration (CUDA events) of the step's heaviest kernels and
    their achieved bandwidth on algorithmic bytes. The line's ``roofline`` is
    the entry with the largest measured share of the step."""
    import torch
    peak, src = hbm_peak()
    lib = sim.lib
    out = []
    ev = lambda: torch.cuda.Event(enable_timing=True)
    if solver == "rb":
        s = sim.s
        saved = (s.eps, s.itermax)
        n_it = 40
        s.eps, s.itermax = 0.0, n_it
        sim.solve()  # sets the chunk size
        torch.cuda.synchronize()
        e0, e1 = ev(), ev()
        e0.record(stream)
        sim.solve()
        e1.record(stream)
        torch.cuda.synchronize()
        s.eps, s.itermax = saved
        ms = e0.elapsed_time(e1) / (2 * n_it)
        out.append(_roof("k_sor_pass: one colour of a red-black SOR iteration (FP64)",
                         "k_sor_pass", ms, 12.0 * ncell, ncell, peak, src,
                         note="FP64-pipe bound: 10 FP64 instructions per update",
                         fp64_tflops=20.0 * ncell / 2 / (ms * 1e-3) / 1e12))
    elif solver in ("mg", "mg-mixed"):
        from nusif import abi
        msr = C.c_double()
        reps = 20
        lib.nusifTimeKernel(C.byref(sim.s), sim.d.p, sim.d.rhs, 0, reps, C.byref(msr))
        abi.check(lib)
        if solver == "mg-mixed":
            # one whole red-black sweep: x read, b read, x written (FP32)
            i, j, _ = sim.dims
            vec = i % 128 == 0 and j % 8 == 0  # the register-tiled kernel's levels
            out.append(_roof("k_rbgs_sweep_v: one fine FP32 red-black sweep (register-tiled, one "
                             "kernel)" if vec else
                             "k_rbgs_sweep: one fine FP32 red-black sweep (one kernel)",
                             "k_rbgs_sweep" if vec else "k_rbgs_sweep_tile64", msr.value,
                             12.0 * ncell, ncell, peak, src))
            lib.nusifTimeKernel(C.byref(sim.s), sim.d.p, sim.d.rhs, 1, reps, C.byref(msr))
            abi.check(lib)
            # p and b read (FP64), the FP32 residual written and the FP32 correction zeroed
            if arith == "df32":
                out.append(_roof("k_mx_residual_df: fine residual of p into FP32, double-float "
                                 "stencil (refinement)", "k_mx_residual_df", msr.value,
                                 20.0 * ncell, ncell, peak, src,
                                 note="stencil in FP32 pairs on the FP32 pipe"))
            else:
                out.append(_roof("k_mx_residual: FP64 residual of p into FP32 (refinement)",
                                 "k_mx_residual", msr.value, 20.0 * ncell, ncell, peak, src,
                                 note="FP64-pipe bound: 9 FP64 instructions per cell",
                                 fp64=_fp64_pipe(9.0, ncell, msr.value)))
        else:
            out.append(_roof("k_mg_smooth<double>: one colour pass of the fine FP64 smoother",
                             "k_mg_smooth_f64", msr.value, 12.0 * ncell, ncell, peak, src,
                             note="FP64-pipe bound"))
    # computeFG (flux form): reads u, v, w, writes f, g, h; idempotent for fixed u, v, w
    sim.compute_fg()
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    reps = 5
    e0.record(stream)
    for _ in range(reps):
        sim.compute_fg()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_fg = e0.elapsed_time(e1) / reps
    if arith == "df32":
        out.append(_roof("k_fgh_df: computeFG, face fluxes in double-float pairs", "k_fgh_df",
                         ms_fg, 48.0 * ncell, ncell, peak, src,
                         note="FP32-pipe / issue bound (pair arithmetic), not HBM"))
    else:
        g0 = sim.d.gx == 0.0 and sim.d.gy == 0.0 and sim.d.gz == 0.0
        fg_inst = 70.4 if g0 else 73.4  # per cell, counted from the kernel (halo share included)
        out.append(_roof("k_fgh_flux: computeFG (FP64)", "k_fgh_flux", ms_fg, 48.0 * ncell,
                         ncell, peak, src, note="FP64-pipe bound: about %.0f FP64 instructions "
                         "per cell" % fg_inst, fp64=_fp64_pipe(fg_inst, ncell, ms_fg)))
    return out


def run_e2e(sim, args, stream, padded):
    import numpy as np
    import torch
    from nusif import abi
    host = {f: torch.empty(padded, dtype=torch.float64, pin_memory=True) for f in "uvwp"}
    for f in "uvwp":
        host[f].numpy()[:] = sim.field(f).reshape(-1)
    lib = sim.lib
    ptrs = {f: C.cast(host[f].data_ptr(), abi.c_double_p) for f in "uvwp"}
    idx = abi.FIELD_INDEX
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        # queued copies: p's upload overlaps computeTimestep .. computeRHS, which do
        # not read p; every library call waits on the device for the fields it uses
        for f in "uvwp":
            lib.nusifUploadFieldAsync(C.byref(sim.d), idx[f], ptrs[f])
        # p is final after the solve: its download overlaps adaptUV, which only reads p
        sim.step(after_solve=lambda: lib.nusifDownloadFieldAsync(C.byref(sim.d), idx["p"],
                                                                 ptrs["p"]))
        for f in "uvw":
            lib.nusifDownloadFieldAsync(C.byref(sim.d), idx[f], ptrs[f])
        lib.nusifWaitCopies()
    torch.cuda.synchronize()
    abi.check(lib)
    ms = (time.perf_counter() - t0) * 1e3 / args.steps
    return {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 4 * 8 * padded,
            "d2h_bytes_per_step": 4 * 8 * padded,
            "path": "C ABI: nusifUploadFieldAsync x4 (pinned host arrays), the reference's "
                    "step calls with p's nusifDownloadFieldAsync between solve and adaptUV, "
                    "nusifDownloadFieldAsync x3, nusifWaitCopies"}


# ---------------------------------------------------------------- CPU side

def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


class CpuStepSampler:
    """The reference algorithm's time step on one host core, through the
    oracle's C restatement built with the reference's flags (-O3 -ffast-math):
    the non-solver operators once (src/main.c:61-70,79: CFL, boundary
    conditions, F/G/H, RHS, adaptUV) and a bounded number of red-black SOR
    iterations (src/solver-rb.c:54-160), timed separately. The state stays
    allocated between samples; the iterations run on the state's own p and
    rhs with eps 0, so none stops early."""

    def __init__(self, vals, fast=True):
        import numpy as np
        import oracle
        self.run = oracle.OracleRun(dict(vals, itermax=1), "rb", fast=fast)
        self.n = int(np.prod(self.run.shape))

    def sample(self, sweeps: int) -> tuple[float, float]:
        """(seconds of the non-solver operators, seconds of `sweeps` iterations)."""
        lib, st = self.run.lib, self.run.st
        g, n, d = st.g, self.n, C.c_double
        t0 = time.perf_counter()
        dt = lib.or_timestep(st.dtBound, g.dx, g.dy, g.dz, lib.or_max_abs(st.u, n),
                             lib.or_max_abs(st.v, n), lib.or_max_abs(st.w, n), st.c.tau)
        lib.or_set_bc(C.byref(g), st.c.bc, st.u, st.v, st.w)
        lib.or_special_bc(C.byref(g), st.c.problem, d(st.c.lid), d(st.c.inflow), st.u)
        lib.or_compute_fgh(C.byref(g), d(st.c.re), d(st.c.gamma), d(st.c.gx), d(st.c.gy),
                           d(st.c.gz), d(dt), st.u, st.v, st.w, st.f, st.gf, st.h)
        lib.or_compute_rhs(C.byref(g), d(dt), st.f, st.gf, st.h, st.rhs)
        lib.or_adapt_uv(C.byref(g), d(dt), st.f, st.gf, st.h, st.p, st.u, st.v, st.w)
        t_ns = time.perf_counter() - t0
        res = C.c_double()
        t0 = time.perf_counter()
        if sweeps > 0:
            lib.or_solve_rb(C.byref(g), 0.0, st.c.omega, sweeps, st.p, st.rhs, C.byref(res))
        return t_ns, time.perf_counter() - t0

    def close(self):
        self.run.close()


def cpu_baseline(vals, solver, gpu_iters, sweeps: int = 100):
    it = float(sum(gpu_iters)) / max(len(gpu_iters), 1) if solver == "rb" else float(vals["itermax"])
    smp = CpuStepSampler(vals)
    try:
        t_ns, t_sw = smp.sample(sweeps)
    finally:
        smp.close()
    t_it = t_sw / max(sweeps, 1)
    ms = (t_ns + it * t_it) * 1e3
    return {"value": ms, "unit": UNIT, "cores": 1, "kind": "port", "cpu_model": cpu_model(),
            "extrapolated": True, "sweeps_timed": sweeps, "sweeps_per_step_assumed": it,
            "timed_s": t_ns + t_sw,
            "sample": (f"one pass of the non-solver operators ({t_ns:.2f} s) plus {sweeps} "
                       f"red-black SOR iterations ({t_it * 1e3:.1f} ms each) at "
                       f"{vals['imax']}^3 on one host core, scaled to {it:.0f} iterations per "
                       f"step (the reference's red-black solve for this case)")}


def run_reference(args, rank, world):
    """The reference's CPU code path for the benchmark step: each step times
    the non-solver operators once and args.ref_sweeps red-black iterations
    on one core, and `value` extrapolates the step to the reference's
    itermax = 10000 iterations (every step of this case reaches itermax in
    the reference: tests/golden/config2_rb.npz)."""
    if rank != 0:
        return None
    solver = pick_solver(args.solver)
    vals = bench_case(args.n, solver, args.itermax)
    it = float(vals["itermax"])
    sweeps = args.ref_sweeps
    smp = CpuStepSampler(vals)
    ns, sw, wall = [], [], 0.0
    try:
        for s in range(args.warmup + args.steps):
            # warm-up steps run the operators and one sweep only (they warm caches and pages)
            t_ns, t_sw = smp.sample(sweeps if s >= args.warmup else 1)
            if s >= args.warmup:
                ns.append(t_ns)
                sw.append(t_sw)
                wall += t_ns + t_sw
    finally:
        smp.close()
    t_ns = sum(ns) / len(ns)
    t_it = sum(sw) / (len(sw) * max(sweeps, 1))
    ms = (t_ns + it * t_it) * 1e3
    n = vals["imax"]
    sample = (f"per step: the non-solver operators once ({t_ns:.2f} s) plus {sweeps} red-black "
              f"iterations ({t_it * 1e3:.1f} ms each), extrapolated to {it:.0f} iterations "
              f"(the reference's algorithm, oracle C restatement compiled with -O3 -ffast-math, "
              f"sequential, one core)")
    return {
        "impl": "reference",
        "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: lid-driven cavity from rest, no dataset",
        "config": {"workload": f"lid-driven cavity {n}x{n}x{n}, Re 1000, tau 0.5, "
                               f"reference red-black SOR solve (omega 1.7, eps 1e-6, itermax 10000)",
                   "cells": n ** 3, "solver": "rb (reference)"},
        "extrapolated": True, "sweeps_timed_per_step": sweeps,
        "sweeps_per_step_assumed": it, "timed_region_s": wall,
        "ms_per_sweep": t_it * 1e3, "non_solver_ms": t_ns * 1e3,
        "mlups": {"solver_mlups": n ** 3 * 1e-6 / t_it,
                  "definition": "iterations x cells x 1e-6 / solver seconds (src/profiler.c:61-74)"},
        "cpu_baseline": {"value": ms, "unit": UNIT, "cores": 1, "kind": "port",
                         "cpu_model": cpu_model(), "sample": sample},
        "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


class DeviceArray:
    """A device pointer seen by torch (plumbing for error norms on the GPU)."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": "<f8",
                                         "data": (ctypes_addr(ptr), False), "version": 3}


def ctypes_addr(p) -> int:
    return C.cast(p, C.c_void_p).value


def run_channel(args, local):
    """Channel flow 4x1x1 at 512x128x128 (inflow 1 at x=0, outflow at x=4,
    no-slip side walls, Re 100, fields from zero): mixed-precision multigrid
    and FP64 multigrid, both to a 1e-8 relative residual, stepped side by side;
    per-step L2 and Linf differences of u, v, w relative to the FP64 velocity
    field, and of p (without its mean) relative to the FP64 p."""
    import torch

    import nusif
    from nusif.params import channel
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    lib = nusif.load_library()
    lib.nusifSetStream(C.c_void_p(stream.cuda_stream))
    steps = args.steps
    # the FP64 run is FP64 throughout (every stencil in FP64 instructions)
    # fuse_dt: the CFL maxima from adaptUV in both runs (the same dt bit for bit)
    sims = {"mg-mixed": nusif.Simulation(channel(solver="mg-mixed", rtol=1e-8, arith=args.arith,
                                                 fuse_dt=1)),
            "mg": nusif.Simulation(channel(solver="mg", rtol=1e-8, arith="fp64", fuse_dt=1))}
    shape = sims["mg"].padded_shape

    def view(sim, f):
        return torch.as_tensor(DeviceArray(getattr(sim.d, f), shape), device="cuda")[1:-1, 1:-1, 1:-1]

    err = {f: {"l2": [], "linf": []} for f in "uvwp"}
    ms = {s: 0.0 for s in sims}
    cycles = {s: [] for s in sims}
    for _ in range(steps):
        for s, sim in sims.items():
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            info = sim.step()
            e1.record(stream)
            torch.cuda.synchronize()
            ms[s] += e0.elapsed_time(e1)
            cycles[s].append(info.it)
        # velocity components against the whole FP64 velocity field (v, w are
        # near zero in a channel, so their own norms would inflate the ratio)
        vel = {f: view(sims["mg"], f) for f in "uvw"}
        vel_l2 = float(torch.sqrt(sum(torch.linalg.vector_norm(vel[f]) ** 2 for f in "uvw")))
        vel_max = float(max(vel[f].abs().max() for f in "uvw"))
        for f in "uvwp":
            a, b = view(sims["mg-mixed"], f), view(sims["mg"], f)
            if f == "p":
                a, b = a - a.mean(), b - b.mean()
                l2_ref, max_ref = float(torch.linalg.vector_norm(b)), float(b.abs().max())
            else:
                l2_ref, max_ref = vel_l2, vel_max
            d = a - b
            err[f]["l2"].append(float(torch.linalg.vector_norm(d)) / max(l2_ref, 1e-300))
            err[f]["linf"].append(float(d.abs().max()) / max(max_ref, 1e-300))
    for sim in sims.values():
        sim.close()
    return {
        "metric": "channel 512x128x128, 4x1x1, Re 100: mixed-precision vs FP64 multigrid field error",
        "value": max(max(err[f]["l2"]) for f in "uvwp"), "unit": "max relative L2 difference",
        "higher_is_better": False, "steps": steps, "n_gpus": 1,
        "config": {"workload": "channel flow 512x128x128, inflow 1, outflow, no-slip walls, "
                               "Re 100, fields from zero", "rtol": 1e-8},
        "ms_per_step": {s: ms[s] / steps for s in ms},
        "v_cycles_per_step_mean": {s: sum(c) / len(c) for s, c in cycles.items()},
        "error_final": {f: {k: v[-1] for k, v in err[f].items()} for f in "uvwp"},
        "error_max": {f: {k: max(v) for k, v in err[f].items()} for f in "uvwp"},
        "error_every_50": {f: err[f]["l2"][::50] for f in "uvwp"},
    }


BATCH_SEED = 20261203


def batch_cases(n: int, seed: int = BATCH_SEED) -> list[dict]:
    """n lid-driven cavities: cube edges from {32, 48, 64, 96, 128}, Re ~ U[100, 5000],
    mixed-precision multigrid to a 1e-6 relative residual from the quadratic
    warm start (seeded)."""
    import numpy as np

    from nusif.params import cavity
    rng = np.random.default_rng(seed)
    edges = rng.choice([32, 48, 64, 96, 128], size=n)
    res = rng.uniform(100.0, 5000.0, size=n)
    return [cavity(int(e), re=float(r), te=1e9, solver="mg-mixed", rtol=1e-6,
                   mg_guess="quadratic") for e, r in zip(edges, res)]


def shard_cases(n: int, rank: int, world: int) -> list[int]:
    """Instance ids of one rank: rank, rank + world, ... The instances are
    independent (no exchange between them), so ranks share nothing on the
    data path and need no collective there."""
    return list(range(rank, n, world))


def batch_totals(updates: float, wall_s: float, world: int, device: str) -> tuple[float, float]:
    """(cell updates of all ranks, the slowest rank's wall time)."""
    if world <= 1:
        return updates, wall_s
    import torch
    import torch.distributed as dist
    u = torch.tensor([updates], dtype=torch.float64, device=device)
    w = torch.tensor([wall_s], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(w, op=dist.ReduceOp.MAX)
    return float(u.item()), float(w.item())


def instance_error(batch, q: int, case: dict, steps: int) -> dict:
    """Relative L2 difference of one batched instance against the same case
    stepped alone with plain FP64 multigrid (every stencil in FP64
    instructions): u, v, w against the FP64 velocity field, p mean-free."""
    import numpy as np

    import nusif
    ref = nusif.Simulation(dict(case, solver="mg", arith="fp64"))
    for _ in range(steps):
        ref.step()
    e = {}
    for f in "uvwp":
        a = batch.field(q, f)[1:-1, 1:-1, 1:-1]
        b = ref.field(f)[1:-1, 1:-1, 1:-1]
        if f == "p":
            a, b = a - a.mean(), b - b.mean()
        e[f] = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    ref.close()
    return {"instance": q, "edge": case["imax"], "re": round(case["re"], 1), "rel_l2": e}


def run_batch(args, rank, world, local):
    """All instances of this rank advanced together, one CUDA-graph launch per
    time step; aggregate cell updates per second over all ranks, and every
    instance's field difference against plain FP64 multigrid run alone."""
    import torch

    import nusif
    torch.cuda.set_device(local)
    device = "cuda"
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl")
    lib = nusif.load_library()
    all_cases = batch_cases(args.batch_n)
    mine = shard_cases(len(all_cases), rank, world)
    cases = [all_cases[q] for q in mine]
    cells = [c["imax"] * c["jmax"] * c["kmax"] for c in cases]
    t0 = time.perf_counter()
    batch = nusif.Batch(cases, queue=0, tune=True)
    setup_s = time.perf_counter() - t0
    batch.step(args.warmup)
    launches0 = lib.nusifLaunchCount()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    batch.step(args.steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if world > 1:
        torch.distributed.barrier()
    launches_outside = int(lib.nusifLaunchCount() - launches0)
    stats = [batch.stats(q) for q in range(batch.n)]
    updates, wall_max = batch_totals(float(sum(cells) * args.steps), wall, world, device)
    errs = []
    if not args.no_compare:
        for q, gq in enumerate(mine):
            e = instance_error(batch, q, cases[q], args.warmup + args.steps)
            e["instance"] = gq
            errs.append(e)
    batch.close()
    summary = {"unconverged_steps": sum(s.unconverged for s in stats),
               "v_cycles_min": min(s.cycles for s in stats),
               "v_cycles_max": max(s.cycles for s in stats),
               "fg_planes": sorted({s.fg_planes for s in stats}),
               "errors": errs, "cells": sum(cells), "instances": len(cases)}
    if world > 1:
        gathered = [None] * world
        torch.distributed.all_gather_object(gathered, summary)
    else:
        gathered = [summary]
    if rank != 0:
        return None
    errs = sorted((e for g in gathered for e in g["errors"]), key=lambda e: e["instance"])
    worst = {f: max((e["rel_l2"][f] for e in errs), default=None) for f in "uvwp"}
    return {
        "metric": "batched cavities: aggregate cell updates per second (mixed-precision MG to 1e-6)",
        "value": updates / wall_max, "unit": "cell-updates/s", "higher_is_better": True,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "scaling": "weak",
        "config": {"workload": f"{len(all_cases)} lid-driven cavities, edges from "
                               "{32,48,64,96,128}^3, Re ~ U[100,5000] (seeded), "
                               "one CUDA graph launch per time step", "seed": BATCH_SEED,
                   "cells_total": sum(g["cells"] for g in gathered),
                   "sharding": f"instances[rank::{world}] per rank, no data-path collective",
                   "mg_loop": "graph while-loop to rtol"},
        "ms_per_step": wall_max * 1e3 / args.steps,
        "setup_s": setup_s,
        "gpu_launches_outside_graphs": launches_outside,
        "unconverged_steps": sum(g["unconverged_steps"] for g in gathered),
        "v_cycles_last_step": {"min": min(g["v_cycles_min"] for g in gathered),
                               "max": max(g["v_cycles_max"] for g in gathered)},
        "fg_planes_chosen": sorted({p for g in gathered for p in g["fg_planes"]}),
        "error_vs_fp64_mg": {"against": "each case stepped alone with FP64 multigrid V(2,2), "
                                        "every stencil in FP64 instructions, same steps",
                             "instances_compared": len(errs), "steps": args.warmup + args.steps,
                             "max_rel_l2": worst, "per_instance": errs},
    }


LEARN_SEED = 20261204


def run_learned(args, local):
    """Learned warm start: pairs recorded by the solver on cavities at
    args.learn_n^3 (Re ~ U[100, 5000], lid ~ U[0.5, 2], seeded), the U-Net
    trained with the library's kernels, then evaluated as the warm start of
    mixed-precision multigrid on a cavity at args.n^3 and an unseen Re / lid,
    against the same run without the network (ms per step and V-cycles)."""
    import numpy as np
    import torch

    import nusif
    from nusif.learn import generate_pairs, train, training_cases
    torch.cuda.set_device(local)
    lib = nusif.load_library()
    stream = torch.cuda.current_stream()
    lib.nusifSetStream(C.c_void_p(stream.cuda_stream))
    cases = training_cases(args.learn_runs, args.learn_n, LEARN_SEED, guess=args.guess)
    data = generate_pairs(cases, steps=args.learn_steps, every=5, skip=10)
    net = nusif.UNet(seed=LEARN_SEED)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    log = train(net, data, iters=args.learn_iters, batch=args.learn_batch, lr=1e-3,
                log_every=max(args.learn_iters // 8, 1))
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    if args.save_net:
        from nusif.learn import save_params
        save_params(net, args.save_net, {
            "cases": f"{args.learn_runs} lid-driven cavities at {args.learn_n}^3, Re ~ U[100,5000], "
                     f"lid ~ U[0.5,2.0], seed {LEARN_SEED}",
            "pairs": int(data.x.shape[0]), "snapshots": f"every 5 steps from step 10 to "
                                                         f"{args.learn_steps}",
            "warm_start_base": args.guess, "adam_iters": args.learn_iters, "batch": args.learn_batch,
            "lr": "1e-3 cosine to 1e-4", "final_loss": log[-1][1] if log else None,
            "train_s": train_s})
    n = args.n
    evals = {}
    for use in (False, True):
        vals = bench_case(n, "mg-mixed", args.itermax, args.guess)
        # the network is probed every 8th step once its guess lost twice in a row
        vals.update(re=2750.0, lid=1.25, mg_probe=LEARNED_PROBE)
        sim = nusif.Simulation(vals)
        if use:
            sim.set_guess_net(net)
        for _ in range(args.warmup):
            sim.step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        its, taken, ratios = [], 0, []
        ms = 0.0
        for _ in range(args.steps):
            e0.record(stream)
            its.append(sim.step().it)
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
            if use:
                u, rw, rg = sim.guess_stats()
                taken += int(u)
                ratios.append(rg / rw if rw > 0 else 1.0)
        counts = sim.guess_counts() if use else (0, 0)
        sim.close()
        evals[use] = {"ms_per_step": ms / args.steps, "v_cycles_per_step": its}
        if use:
            evals[use].update({"guess_taken_steps": taken,
                               "restricted_residual_ratio_median": float(np.median(ratios)),
                               "network_evaluations_incl_warmup": counts[0],
                               "guesses_taken_incl_warmup": counts[1],
                               "probe_every_after_two_rejections": LEARNED_PROBE})
    net.close()
    return {
        "metric": "learned warm start: ms/timestep at %d^3 to 1e-6, mixed-precision MG with vs "
                  "without the trained U-Net" % n,
        "value": evals[True]["ms_per_step"], "unit": "ms/timestep", "higher_is_better": False,
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "dtype": "bf16 net, f64+f32 solve",
        "data": "synthetic: pairs recorded by the solver on seeded cavities",
        "config": {"workload": f"train on {args.learn_runs} cavities at {args.learn_n}^3 "
                               f"(Re ~ U[100,5000], lid ~ U[0.5,2.0], seed {LEARN_SEED}), "
                               f"snapshots every 5 steps from step 10 to {args.learn_steps}; "
                               f"evaluate at {n}^3, Re 2750, lid 1.25",
                   "warm_start_base": args.guess, "pairs": int(data.x.shape[0]),
                   "train_iters": args.learn_iters, "batch": args.learn_batch,
                   "lr": "1e-3 cosine to 1e-4"},
        "pair_generation_s": data.seconds, "train_s": train_s,
        "train_ms_per_iter": train_s * 1e3 / max(args.learn_iters, 1),
        "loss": log,
        "with_net": evals[True], "without_net": evals[False],
        "speedup_vs_without": evals[False]["ms_per_step"] / evals[True]["ms_per_step"],
    }


def main():
    args = parse_args()
    rank, world, local = dist_info()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload == "channel":
        out = run_channel(args, local) if rank == 0 else None
    elif args.workload == "batch":
        out = run_batch(args, rank, world, local)
    elif args.workload == "learned":
        out = run_learned(args, local) if rank == 0 else None
    else:
        out = run_gpu(args, rank, world, local)
    if out is not None and rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
