// Batched execution of many independent NuSiF instances (uneven grids).
//
// Every instance is an ordinary Parameter / Discretization / Solver triple
// (same entry points, same kernels). What the batch adds:
//  - a device-resident time step: the CFL maxima feed a one-thread kernel
//    that computes dt with the host's expressions (computeTimestep,
//    discretization.c:431-453) into StepScalars, which F/G/H, RHS and adaptUV
//    read; the multigrid solve is a CUDA graph while-loop over device-gated
//    units (mg_enqueue_loop) that runs exactly as many units as the
//    host-driven solve, or optionally a fixed queue of units (mg_enqueue).
//    One time step of one instance is then a launch sequence with no host
//    synchronisation;
//  - one CUDA graph per step kind (with / without normalizePressure, every
//    100 steps as main.c:68-70): each instance's sequence is captured on its
//    own stream as an independent branch, so one graph launch advances every
//    instance and the GPU overlaps the small grids' kernels;
//  - a tile autotuner: for each instance the planes-per-block of the F/G/H
//    kernel are timed on that grid (CUDA events) and the fastest is captured.
// Results are those of stepping each instance alone with the mg / mg-mixed
// solvers (same kernels, same arithmetic, dt computed with the same
// expressions); steps whose solve ended above rtol (a fixed queue that ran
// out, or the mg_cycles limit) are counted.
#include <cstdio>
#include <cstring>
#include <vector>

#include "nusif_internal.h"
#include "solver_internal.h"

extern "C" {
struct NusifBatch;
}

namespace nusif {

DiscState *disc_state(const Discretization *d);

namespace {

struct BatchDev {
  StepScalars sc;
  int unconverged;  // steps whose multigrid solve ended above rtol
  int last_cycles;  // V-cycles of the last step
};

struct BatchInst {
  Parameter param;
  Discretization d;
  Solver s;
  cudaStream_t stream = nullptr;
  cudaEvent_t join = nullptr;
  BatchDev *dev = nullptr;  // device
  int fg_kb = 0;            // autotuned F/G/H planes per block (0: default rule)
};

__global__ void k_step_dt(const double *max3, BatchDev *bd, double dtBound, double dx, double dy,
    double dz, double tau, double fixed_dt)
{
  double dt = fixed_dt;
  if (tau > 0.0) {
    dt = dtBound;
    const double umax = max3[0], vmax = max3[1], wmax = max3[2];
    if (umax > 0) dt = (dt > dx / umax) ? dx / umax : dt;
    if (vmax > 0) dt = (dt > dy / vmax) ? dy / vmax : dt;
    if (wmax > 0) dt = (dt > dz / wmax) ? dz / wmax : dt;
    dt = dt * tau;
  }
  bd->sc.dt = dt;
  bd->sc.idt = 1.0 / dt;
  bd->sc.rx = (1.0 / dx) * bd->sc.idt;
  bd->sc.ry = (1.0 / dy) * bd->sc.idt;
  bd->sc.rz = (1.0 / dz) * bd->sc.idt;
  bd->sc.fx = dt / dx;
  bd->sc.fy = dt / dy;
  bd->sc.fz = dt / dz;
}

__global__ void k_step_advance(BatchDev *bd)
{
  bd->sc.t += bd->sc.dt;
  bd->sc.nt += 1;
}

}  // namespace
}  // namespace nusif

using namespace nusif;

struct NusifBatch {
  std::vector<BatchInst *> inst;
  cudaStream_t main = nullptr;
  cudaStream_t body = nullptr;  // captures the multigrid while-loop bodies
  cudaEvent_t fork = nullptr;
  cudaGraphExec_t exec[2] = { nullptr, nullptr };
  int queue = 0;  // > 0: fixed number of multigrid units per step, else a while-loop
  int nt = 0;
};

namespace {

// one time step of one instance, reference order (src/main.c:61-79), on the
// current library stream, without host synchronisation
bool enqueue_step(BatchInst *b, bool normalize, int queue, cudaStream_t body)
{
  Discretization *d = &b->d;
  DiscState *st = disc_state(d);
  SolverState *ss = solver_state(&b->s);
  const Dims &g = st->dims;
  const StepScalars *sp = &b->dev->sc;
  if (!launch_max3(g, d->u, d->v, d->w, st->red, st->d_scalars)) return false;
  k_step_dt<<<1, 1, 0, stream()>>>(st->d_scalars, b->dev, d->dtBound, d->grid.dx, d->grid.dy,
      d->grid.dz, d->tau, d->dt);
  if (!launched("k_step_dt")) return false;
  const int bc[6] = { d->bcLeft, d->bcRight, d->bcBottom, d->bcTop, d->bcFront, d->bcBack };
  if (!launch_bc(g, bc, PROBLEM_NONE, 0.0, 0.0, d->u, d->v, d->w)) return false;
  if (!launch_special(g, problem_code(d->problem), st->ext.lid, st->ext.inflow, d->u))
    return false;
  if (!launch_fgh(g, d->re, d->gamma, d->gx, d->gy, d->gz, 0.0, d->grid.dx, d->grid.dy,
          d->grid.dz, d->u, d->v, d->w, d->f, d->g, d->h, sp, b->fg_kb, st->ext.fg_fp64 != 0))
    return false;
  if (!launch_rhs(g, 0.0, d->grid.dx, d->grid.dy, d->grid.dz, d->f, d->g, d->h, d->rhs, sp))
    return false;
  if (normalize) {
    if (!launch_interior_sum(g, d->p, st->red, st->d_scalars + 3)) return false;
    if (!launch_subtract_mean(g, d->p, st->d_scalars + 4)) return false;
  }
  const bool solved = queue > 0 ? mg_enqueue(ss, d->p, d->rhs, queue, &b->dev->unconverged,
                                      &b->dev->last_cycles)
                                : mg_enqueue_loop(ss, d->p, d->rhs, body, &b->dev->unconverged,
                                      &b->dev->last_cycles);
  if (!solved) return false;
  if (!launch_adapt_uv(g, 0.0, d->grid.dx, d->grid.dy, d->grid.dz, d->f, d->g, d->h, d->p, d->u,
          d->v, d->w, sp))
    return false;
  k_step_advance<<<1, 1, 0, stream()>>>(b->dev);
  return launched("k_step_advance");
}

bool capture(NusifBatch *B, bool normalize, cudaGraphExec_t *out)
{
  cudaStream_t saved = stream();
  cudaGraph_t graph = nullptr;
  if (!cuda_ok(cudaStreamBeginCapture(B->main, cudaStreamCaptureModeThreadLocal), "begin capture"))
    return false;
  bool ok = cuda_ok(cudaEventRecord(B->fork, B->main), "fork");
  for (BatchInst *b : B->inst) {
    if (!ok) break;
    ok = cuda_ok(cudaStreamWaitEvent(b->stream, B->fork, 0), "branch wait");
    nusifSetStream(b->stream);
    ok = ok && enqueue_step(b, normalize, B->queue, B->body);
    ok = ok && cuda_ok(cudaEventRecord(b->join, b->stream), "join record") &&
         cuda_ok(cudaStreamWaitEvent(B->main, b->join, 0), "join wait");
  }
  nusifSetStream(saved);
  const bool ended = cuda_ok(cudaStreamEndCapture(B->main, &graph), "end capture");
  ok = ok && ended && cuda_ok(cudaGraphInstantiate(out, graph, 0), "graph instantiate");
  if (graph) cudaGraphDestroy(graph);
  return ok;
}

// planes per block of the F/G/H kernel: time the candidates on this grid
void autotune(BatchInst *b, cudaStream_t s)
{
  Discretization *d = &b->d;
  DiscState *st = disc_state(d);
  const int cand[5] = { 2, 4, 8, 16, 32 };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaStream_t saved = stream();
  nusifSetStream(s);
  float best = 1e30f;
  int best_kb = 0;
  for (int c : cand) {
    if (c > st->dims.kmax) continue;
    launch_fgh(st->dims, d->re, d->gamma, d->gx, d->gy, d->gz, d->dt, d->grid.dx, d->grid.dy,
        d->grid.dz, d->u, d->v, d->w, d->f, d->g, d->h, nullptr, c, st->ext.fg_fp64 != 0);
    cudaEventRecord(e0, s);
    for (int r = 0; r < 3; r++)
      launch_fgh(st->dims, d->re, d->gamma, d->gx, d->gy, d->gz, d->dt, d->grid.dx, d->grid.dy,
          d->grid.dz, d->u, d->v, d->w, d->f, d->g, d->h, nullptr, c, st->ext.fg_fp64 != 0);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      best_kb = c;
    }
  }
  nusifSetStream(saved);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->fg_kb = best_kb;
}

void batch_free(NusifBatch *B)
{
  if (!B) return;
  cudaDeviceSynchronize();
  for (int q = 0; q < 2; q++)
    if (B->exec[q]) cudaGraphExecDestroy(B->exec[q]);
  for (BatchInst *b : B->inst) {
    nusifFreeSolver(&b->s);
    nusifFreeDiscretization(&b->d);
    if (b->dev) cudaFree(b->dev);
    if (b->join) cudaEventDestroy(b->join);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
  }
  if (B->fork) cudaEventDestroy(B->fork);
  if (B->body) cudaStreamDestroy(B->body);
  if (B->main) cudaStreamDestroy(B->main);
  delete B;
}

}  // namespace

extern "C" {

NusifBatch *nusifBatchCreate(int n, const char *const *parfiles, int queue, int tune)
{
  if (n < 1 || !parfiles) {
    fail(NUSIF_ERR_ARG, "nusifBatchCreate: need at least one parameter file");
    return nullptr;
  }
  NusifBatch *B = new NusifBatch();
  B->queue = queue;
  cudaStream_t saved = stream();
  bool ok = cuda_ok(cudaStreamCreateWithFlags(&B->main, cudaStreamNonBlocking), "stream") &&
            cuda_ok(cudaStreamCreateWithFlags(&B->body, cudaStreamNonBlocking), "stream") &&
            cuda_ok(cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming), "event");
  for (int q = 0; q < n && ok; q++) {
    BatchInst *b = new BatchInst();
    B->inst.push_back(b);
    memset(&b->param, 0, sizeof(b->param));
    memset(&b->d, 0, sizeof(b->d));
    memset(&b->s, 0, sizeof(b->s));
    ok = cuda_ok(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream") &&
         cuda_ok(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming), "event");
    if (!ok) break;
    nusifSetStream(b->stream);
    initParameter(&b->param);
    readParameter(&b->param, parfiles[q]);
    if (has_error()) ok = false;
    if (ok) initDiscretization(&b->d, &b->param);
    if (ok && !has_error()) initSolver(&b->s, &b->d, &b->param);
    if (has_error()) ok = false;
    SolverState *ss = ok ? solver_state(&b->s) : nullptr;
    if (ok && (!ss || !ss->mg || !mg_capture_ok(ss))) {
      fail(NUSIF_ERR_ARG,
          "nusifBatchCreate: %s needs the mg or mg-mixed solver with even mg_pre/mg_post",
          parfiles[q]);
      ok = false;
    }
    if (!ok) break;
    DiscState *st = disc_state(&b->d);
    // scratch the captured launches use must exist before capture
    ok = reduce_scratch_alloc(st->red, 3 * 4 * 152 * 2) &&
         cuda_ok(cudaMalloc(&b->dev, sizeof(BatchDev)), "cudaMalloc(batch dev)") &&
         cuda_ok(cudaMemsetAsync(b->dev, 0, sizeof(BatchDev), b->stream), "zero batch dev");
    if (ok && tune) autotune(b, b->stream);
  }
  nusifSetStream(saved);
  ok = ok && cuda_ok(cudaDeviceSynchronize(), "batch setup");
  ok = ok && capture(B, false, &B->exec[0]) && capture(B, true, &B->exec[1]);
  if (!ok) {
    batch_free(B);
    return nullptr;
  }
  return B;
}

int nusifBatchStep(NusifBatch *B, int steps)
{
  if (!B) {
    fail(NUSIF_ERR_ARG, "nusifBatchStep: null batch");
    return NUSIF_ERR_ARG;
  }
  // the batch runs on its own streams: queued field copies end first
  if (nusifWaitCopies() != NUSIF_OK) return NUSIF_ERR_CUDA;
  for (auto &in : B->inst) velocity_written(disc_state(&in->d));
  for (int q = 0; q < steps; q++) {
    cudaGraphExec_t ex = B->exec[B->nt % 100 == 0 ? 1 : 0];
    if (!cuda_ok(cudaGraphLaunch(ex, B->main), "graph launch")) return NUSIF_ERR_CUDA;
    B->nt++;
  }
  if (!cuda_ok(cudaStreamSynchronize(B->main), "batch step sync")) return NUSIF_ERR_CUDA;
  return NUSIF_OK;
}

int nusifBatchSize(const NusifBatch *B) { return B ? (int)B->inst.size() : 0; }

int nusifBatchInstance(NusifBatch *B, int idx, Discretization **d, Solver **s)
{
  if (!B || idx < 0 || idx >= (int)B->inst.size()) {
    fail(NUSIF_ERR_ARG, "nusifBatchInstance: index %d out of range", idx);
    return NUSIF_ERR_ARG;
  }
  if (d) *d = &B->inst[idx]->d;
  if (s) *s = &B->inst[idx]->s;
  return NUSIF_OK;
}

int nusifBatchStats(NusifBatch *B, int idx, double *t, double *dt, int *nt, int *cycles,
    int *unconverged, int *fg_planes)
{
  if (!B || idx < 0 || idx >= (int)B->inst.size()) {
    fail(NUSIF_ERR_ARG, "nusifBatchStats: index %d out of range", idx);
    return NUSIF_ERR_ARG;
  }
  BatchInst *b = B->inst[idx];
  BatchDev h;
  if (!cuda_ok(cudaMemcpy(&h, b->dev, sizeof(h), cudaMemcpyDeviceToHost), "batch stats"))
    return NUSIF_ERR_CUDA;
  if (t) *t = h.sc.t;
  if (dt) *dt = h.sc.dt;
  if (nt) *nt = h.sc.nt;
  if (cycles) *cycles = h.last_cycles;
  if (unconverged) *unconverged = h.unconverged;
  if (fg_planes) *fg_planes = b->fg_kb;
  return NUSIF_OK;
}

void nusifBatchFree(NusifBatch *B) { batch_free(B); }

}  // extern "C"
