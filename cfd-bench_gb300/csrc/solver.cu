// Pressure solvers of the NuSiF time step and the reference entry points
// initSolver / solve (src/solver.h:35-36).
//
//  rb      red-black SOR with the reference's exact iteration semantics
//          (src/solver-rb.c:27-172)
//  mg-ref  the reference multigrid as it behaves (src/solver-mg.c:299-402)
//  mg, mg-mixed  geometric V-cycles (multigrid.cu)
//
// One red-black iteration is two launches of one kernel, one per colour. A
// thread owns the cell pair (2t+1, 2t+2) of a row and relaxes the one of the
// pass's colour, so both passes use the same coalesced mapping. The second
// pass also writes the Neumann ghost layer: a ghost is read only by its own
// boundary cell, so the reference's "copy after both passes" is reproduced
// exactly (stale ghosts during the sweep, fresh ones after it).
//
// The residual recurrence of the reference (res starts at 1, each iteration
// res = (res + sum r^2) / N) and the stopping test run on the device: the last
// block of the second pass folds the per-block partial sums in a fixed order,
// advances the iteration counter and raises a done flag. Kernels launched
// after the flag is up return at once, so the host can queue iterations in
// chunks and the iteration count stays exact.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <unordered_map>

#include "df32.cuh"
#include "nusif_internal.h"
#include "reduce.cuh"
#include "solver_internal.h"
#include "unet_internal.h"

namespace nusif {

namespace {

constexpr int kBX = 32;  // pairs per block row (64 cells)
constexpr int kBY = 8;   // rows per block
constexpr int kNT = kBX * kBY;

__device__ __forceinline__ bool solve_done(const SolveState *st)
{
  return st != nullptr && *reinterpret_cast<const volatile int *>(&st->done) != 0;
}

// Relax one colour (ACCUM: collect r^2; GHOSTS: write the six-face Neumann
// ghosts of both cells of the pair after the update). When fold_n > 0 the
// last block folds partials[0..fold_n) and advances the solve state.
//
// DF: the residual r = rhs - lap in double-float arithmetic (df32.cuh: pairs
// of FP32 numbers on the FP32 pipe, about 2^-47 of diag |p|) instead of ten
// FP64 instructions per update, which bound the pass on GB300's FP64 pipe.
// The update p - factor r adds the pair factor r to the exact p in two FP64
// additions, so p itself is carried in binary64 as in the reference; r^2 is
// accumulated as a pair and folded in FP64. At the benchmark size (diag
// 3.9e5, eps 1e-6 on the RMS residual) the pair error of r is about 3e-3 of
// eps: the stop test and the iteration count do not see it.
template <bool ACCUM, bool GHOSTS, bool DF>
__global__ void __launch_bounds__(kNT) k_sor_pass(SorArgs A, int colour, double *__restrict__ p,
    const double *__restrict__ rhs, SolveState *st, double *__restrict__ partials, int slot0,
    unsigned *ticket, int fold_n)
{
  if (solve_done(st)) return;
  const Dims &g = A.g;
  const int t = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y + 1;
  const int k0 = blockIdx.z * A.kb + 1;
  const int k1 = min(k0 + A.kb - 1, g.kmax);
  const int sj = g.sj, sk = g.sk;
  double acc = 0.0;
  df::f2 acc2{ 0.0f, 0.0f };
  // The eight values a plane's update reads, loaded one plane ahead: none of
  // them is written by this pass before it is used (they are the other colour,
  // or this thread's own cell of the next plane, or ghosts that only their
  // own boundary cell reads), so the loads of plane k + 1 overlap the
  // arithmetic and the store of plane k.
  struct Stencil {
    double c, w, e, s, n, b, t, r;
  };
  const auto load = [&](int k, Stencil &v) {
    const int i = 2 * t + 1 + ((1 + j + k + colour) & 1);
    if (i > g.imax) return;
    const int64_t c = (int64_t)k * sk + (int64_t)j * sj + i;
    v.c = p[c];
    v.w = p[c - 1];
    v.e = p[c + 1];
    v.s = p[c - sj];
    v.n = p[c + sj];
    v.b = p[c - sk];
    v.t = p[c + sk];
    v.r = rhs[c];
  };
  if (j <= g.jmax && k0 <= k1) {
    Stencil cur{}, nxt{};
    load(k0, cur);
    for (int k = k0; k <= k1; k++) {
      if (k < k1) load(k + 1, nxt);
      const int i = 2 * t + 1 + ((1 + j + k + colour) & 1);
      const int64_t row = (int64_t)k * sk + (int64_t)j * sj;
      if (i <= g.imax) {
        const int64_t c = row + i;
        const double pc = cur.c;
        if constexpr (DF) {
          using namespace df;
          // unnormalised pairs inside the stencil, r renormalised
          f2 lap = mul_u(A.pmdiag, split(pc));
          lap = fma_u(add_u(split(cur.w), split(cur.e)), A.pidx2, lap);
          lap = fma_u(add_u(split(cur.s), split(cur.n)), A.pidy2, lap);
          lap = fma_u(add_u(split(cur.b), split(cur.t)), A.pidz2, lap);
          const f2 r = sub(split(cur.r), lap);
          const f2 d = mul_u(A.pmfactor, r);
          p[c] = (pc + widen(d.hi)) + widen(d.lo);
          if (ACCUM) acc2 = add(acc2, mul_u(r, r));
        } else {
          const double lap = (cur.w + cur.e) * A.idx2 + (cur.s + cur.n) * A.idy2 +
                             (cur.b + cur.t) * A.idz2 - A.diag * pc;
          const double r = cur.r - lap;
          p[c] = pc - A.factor * r;
          if (ACCUM) acc += r * r;
        }
      }
      if (GHOSTS) {
#pragma unroll
        for (int e = 1; e <= 2; e++) {
          const int ii = 2 * t + e;
          if (ii > g.imax) continue;
          const int64_t c = row + ii;
          const bool edge = ii == 1 || ii == g.imax || j == 1 || j == g.jmax || k == 1 || k == g.kmax;
          if (!edge) continue;
          const double val = p[c];
          if (ii == 1) p[c - 1] = val;
          if (ii == g.imax) p[c + 1] = val;
          if (j == 1) p[c - sj] = val;
          if (j == g.jmax) p[c + sj] = val;
          if (k == 1) p[c - sk] = val;
          if (k == g.kmax) p[c + sk] = val;
        }
      }
      cur = nxt;
    }
  }
  if (!ACCUM) return;
  if (DF) acc = df::to_double(acc2);
  __shared__ double sm[kNT / 32];
  acc = block_reduce_sum<kNT>(acc, sm);
  __shared__ bool last;
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (flat_tid() == 0) {
    partials[slot0 + bid] = acc;
    last = fold_n > 0 ? ticket_is_last(ticket) : false;
  }
  __syncthreads();
  if (!last) return;
  const double total = fold_partials<kNT>(partials, fold_n, sm);
  if (flat_tid() == 0) {
    const double res = (st->res + total) / st->ncell;
    const int it = st->it + 1;
    st->res = res;
    st->it = it;
    st->done = !((res >= st->epssq) && (it < st->itermax));
    *ticket = 0;
  }
}

// Mean-square residual of the whole interior, seeded like the reference's
// calculateResidual (res = 1, src/solver-mg.c:252,280-282): res = (1 + sum r^2)/N.
__global__ void __launch_bounds__(kNT) k_residual_ref(SorArgs A, const double *__restrict__ p,
    const double *__restrict__ rhs, SolveState *st, double *__restrict__ partials,
    unsigned *ticket)
{
  const Dims &g = A.g;
  const int t = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y + 1;
  const int k0 = blockIdx.z * A.kb + 1;
  const int k1 = min(k0 + A.kb - 1, g.kmax);
  const int sj = g.sj, sk = g.sk;
  double acc = 0.0;
  if (j <= g.jmax) {
    for (int k = k0; k <= k1; k++) {
#pragma unroll
      for (int e = 1; e <= 2; e++) {
        const int i = 2 * t + e;
        if (i > g.imax) continue;
        const int64_t c = (int64_t)k * sk + (int64_t)j * sj + i;
        const double lap = (p[c - 1] + p[c + 1]) * A.idx2 + (p[c - sj] + p[c + sj]) * A.idy2 +
                           (p[c - sk] + p[c + sk]) * A.idz2 - A.diag * p[c];
        const double r = rhs[c] - lap;
        acc += r * r;
      }
    }
  }
  __shared__ double sm[kNT / 32];
  acc = block_reduce_sum<kNT>(acc, sm);
  __shared__ bool last;
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (flat_tid() == 0) {
    partials[bid] = acc;
    last = ticket_is_last(ticket);
  }
  __syncthreads();
  if (!last) return;
  const int n = gridDim.x * gridDim.y * gridDim.z;
  const double total = fold_partials<kNT>(partials, n, sm);
  if (flat_tid() == 0) {
    st->res = (1.0 + total) / st->ncell;
    *ticket = 0;
  }
}

// Six-face Neumann ghost copy, no edges or corners (src/solver-mg.c:153-174);
// blockIdx.z selects the face.
__global__ void k_pressure_ghosts(Dims g, double *__restrict__ p)
{
  const int face = blockIdx.z;
  const int ax = face >> 1, high = face & 1;
  const int a1 = (ax == 0) ? 1 : 0, a2 = (ax == 2) ? 1 : 2;
  const int n[3] = { g.imax, g.jmax, g.kmax };
  const int a = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int b = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (a > n[a1] || b > n[a2]) return;
  const int s[3] = { 1, g.sj, g.sk };
  const int64_t base = (int64_t)a * s[a1] + (int64_t)b * s[a2];
  const int inner = high ? n[ax] : 1, ghost = high ? n[ax] + 1 : 0;
  p[base + (int64_t)ghost * s[ax]] = p[base + (int64_t)inner * s[ax]];
}

}  // namespace

SorArgs make_sor_args(const Dims &g, double dx, double dy, double dz, double omega)
{
  SorArgs A;
  A.g = g;
  const double dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
  A.idx2 = 1.0 / dx2;
  A.idy2 = 1.0 / dy2;
  A.idz2 = 1.0 / dz2;
  A.diag = 2.0 * (A.idx2 + A.idy2 + A.idz2);
  // src/solver-rb.c:46-47
  A.factor = omega * 0.5 * (dx2 * dy2 * dz2) / (dy2 * dz2 + dx2 * dz2 + dx2 * dy2);
  A.pidx2 = df::from_double_rn(A.idx2);
  A.pidy2 = df::from_double_rn(A.idy2);
  A.pidz2 = df::from_double_rn(A.idz2);
  A.pmdiag = df::from_double_rn(-A.diag);
  A.pmfactor = df::from_double_rn(-A.factor);
  // planes per block: the largest power of two <= 16 that still gives >= 4 waves of blocks
  int sms = 152;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int gx = ((g.imax + 1) / 2 + kBX - 1) / kBX, gy = (g.jmax + kBY - 1) / kBY;
  int kb = 16;
  while (kb > 1 && (int64_t)gx * gy * ((g.kmax + kb - 1) / kb) < 4 * sms) kb >>= 1;
  A.kb = kb;
  return A;
}

dim3 sor_grid(const SorArgs &A)
{
  const Dims &g = A.g;
  return dim3(((g.imax + 1) / 2 + kBX - 1) / kBX, (g.jmax + kBY - 1) / kBY,
      (g.kmax + A.kb - 1) / A.kb);
}

int sor_blocks(const SorArgs &A)
{
  dim3 gr = sor_grid(A);
  return (int)(gr.x * gr.y * gr.z);
}

template <bool DF>
bool rb_iteration(const SorArgs &A, double *p, const double *rhs, SolveState *st,
    ReduceScratch &red)
{
  const dim3 grid = sor_grid(A), blk(kBX, kBY);
  const int nb = sor_blocks(A);
  k_sor_pass<true, false, DF><<<grid, blk, 0, stream()>>>(A, 1, p, rhs, st, red.partials, 0,
      red.ticket, 0);
  if (!launched("k_sor_pass(odd)")) return false;
  k_sor_pass<true, true, DF><<<grid, blk, 0, stream()>>>(A, 0, p, rhs, st, red.partials, nb,
      red.ticket, 2 * nb);
  return launched("k_sor_pass(even)");
}

bool launch_rb_iteration(const SorArgs &A, double *p, const double *rhs, SolveState *st,
    ReduceScratch &red, bool df)
{
  return df ? rb_iteration<true>(A, p, rhs, st, red) : rb_iteration<false>(A, p, rhs, st, red);
}

bool launch_sor_sweep(const SorArgs &A, double *p, const double *rhs, bool ghosts)
{
  const dim3 grid = sor_grid(A), blk(kBX, kBY);
  k_sor_pass<false, false, false><<<grid, blk, 0, stream()>>>(A, 1, p, rhs, nullptr, nullptr, 0,
      nullptr, 0);
  if (!launched("k_sor_pass(odd)")) return false;
  if (ghosts)
    k_sor_pass<false, true, false><<<grid, blk, 0, stream()>>>(A, 0, p, rhs, nullptr, nullptr,
        0, nullptr, 0);
  else
    k_sor_pass<false, false, false><<<grid, blk, 0, stream()>>>(A, 0, p, rhs, nullptr, nullptr,
        0, nullptr, 0);
  return launched("k_sor_pass(even)");
}

bool launch_residual_ref(const SorArgs &A, const double *p, const double *rhs, SolveState *st,
    ReduceScratch &red)
{
  k_residual_ref<<<sor_grid(A), dim3(kBX, kBY), 0, stream()>>>(A, p, rhs, st, red.partials,
      red.ticket);
  return launched("k_residual_ref");
}

bool launch_pressure_ghosts(const Dims &g, double *p)
{
  const int m = g.imax > g.jmax ? g.imax : g.jmax;
  const int mm = g.jmax > g.kmax ? g.jmax : g.kmax;
  dim3 blk(32, 8);
  dim3 grid((m + 31) / 32, (mm + 7) / 8, 6);
  k_pressure_ghosts<<<grid, blk, 0, stream()>>>(g, p);
  return launched("k_pressure_ghosts");
}

// ---- solver side table ----
static std::unordered_map<const Solver *, SolverState *> &solver_table()
{
  static std::unordered_map<const Solver *, SolverState *> t;
  return t;
}

SolverState *solver_state(const Solver *s)
{
  auto &t = solver_table();
  auto it = t.find(s);
  return it == t.end() ? nullptr : it->second;
}

static SolverState *solver_state_create(const Solver *s)
{
  auto &t = solver_table();
  auto it = t.find(s);
  if (it != t.end()) return it->second;
  SolverState *st = new SolverState();
  t[s] = st;
  return st;
}

static void solver_state_erase(const Solver *s)
{
  auto &t = solver_table();
  auto it = t.find(s);
  if (it == t.end()) return;
  delete it->second;
  t.erase(it);
}

static bool verbose()
{
  const char *v = getenv("NUSIF_VERBOSE");
  return v && v[0] && v[0] != '0';
}

// solve for kind rb: src/solver-rb.c:27-172
static double solve_rb(Solver *s, SolverState *ss, double *p, const double *rhs)
{
  const Grid *gr = s->grid;
  const Dims g = make_dims(gr->imax, gr->jmax, gr->kmax);
  const SorArgs A = make_sor_args(g, gr->dx, gr->dy, gr->dz, s->omega);
  const int nb = sor_blocks(A);
  if (!reduce_scratch_alloc(ss->red, 2 * nb)) return NAN;
  SolveState *h = ss->h_state;
  h->res = 1.0;
  h->it = 0;
  h->epssq = s->eps * s->eps;
  h->itermax = s->itermax;
  h->ncell = (double)(gr->imax * gr->jmax * gr->kmax);
  h->done = !((h->res >= h->epssq) && (h->it < h->itermax));
  if (!cuda_ok(cudaMemcpyAsync(ss->d_state, h, sizeof(SolveState), cudaMemcpyHostToDevice,
                   stream()),
          "solve state upload"))
    return NAN;
  // queue iterations in chunks; the first chunk matches the previous solve's count
  int chunk = ss->last_iterations > 0 ? ss->last_iterations : 16;
  if (chunk > s->itermax) chunk = s->itermax;
  while (!h->done) {
    for (int q = 0; q < chunk; q++)
      if (!launch_rb_iteration(A, p, rhs, ss->d_state, ss->red, !ss->ext.arith_fp64))
        return NAN;
    if (!cuda_ok(cudaMemcpyAsync(h, ss->d_state, sizeof(SolveState), cudaMemcpyDeviceToHost,
                     stream()),
            "solve state download"))
      return NAN;
    if (!cuda_ok(cudaStreamSynchronize(stream()), "solve sync")) return NAN;
    chunk = ss->last_iterations > 64 ? ss->last_iterations / 8 : 8;
  }
  ss->last_iterations = h->it;
  if (verbose()) printf("Solver took %d iterations to reach %f\n", h->it, sqrt(h->res));
  return h->res;
}

// solve for kind mg-ref: the observable part of src/solver-mg.c:299-402
static double solve_mg_ref(Solver *s, SolverState *ss, double *p, const double *rhs)
{
  const Grid *gr = s->grid;
  const Dims g = make_dims(gr->imax, gr->jmax, gr->kmax);
  const SorArgs A = make_sor_args(g, gr->dx, gr->dy, gr->dz, s->omega);
  if (!reduce_scratch_alloc(ss->red, sor_blocks(A))) return NAN;
  SolveState *h = ss->h_state;
  h->ncell = (double)(gr->imax * gr->jmax * gr->kmax);
  if (!cuda_ok(cudaMemcpyAsync(ss->d_state, h, sizeof(SolveState), cudaMemcpyHostToDevice,
                   stream()),
          "solve state upload"))
    return NAN;
  const bool coarsest = (s->levels - 1 == 0) || gr->imax < 2 || gr->jmax < 2 || gr->kmax < 2;
  for (int q = 0; q < s->presmooth; q++)
    if (!launch_sor_sweep(A, p, rhs, !coarsest)) return NAN;
  if (!launch_residual_ref(A, p, rhs, ss->d_state, ss->red)) return NAN;
  if (!coarsest) {
    // coarse levels cannot change p (their correction never reaches it); the
    // ghost copy after the (null) correction and the post-smoothing remain
    if (!launch_pressure_ghosts(g, p)) return NAN;
    for (int q = 0; q < s->postsmooth; q++)
      if (!launch_sor_sweep(A, p, rhs, true)) return NAN;
  }
  if (!cuda_ok(cudaMemcpyAsync(h, ss->d_state, sizeof(SolveState), cudaMemcpyDeviceToHost,
                   stream()),
          "solve state download"))
    return NAN;
  if (!cuda_ok(cudaStreamSynchronize(stream()), "solve sync")) return NAN;
  ss->last_iterations = 0;
  if (verbose()) printf("Residuum: %.6f\n", h->res);
  return h->res;
}

}  // namespace nusif

using namespace nusif;

extern "C" {

// initSolver, reference src/solver-rb.c:17-25 and src/solver-mg.c:356-389
void initSolver(Solver *s, Discretization *d, Parameter *p)
{
  if (!s || !d || !p) {
    fail(NUSIF_ERR_ARG, "initSolver: null argument");
    return;
  }
  if (solver_state(s)) nusifFreeSolver(s);
  s->eps = p->eps;
  s->omega = p->omg;
  s->itermax = p->itermax;
  s->levels = p->levels;
  s->presmooth = p->presmooth;
  s->postsmooth = p->postsmooth;
  s->grid = &d->grid;
  s->comm = &d->comm;
  s->problem = p->name;
  s->r = nullptr;
  s->e = nullptr;

  SolverState *ss = solver_state_create(s);
  const Extras *x = extras_for(p, false);
  ss->ext = x ? *x : Extras();
  int kind = ss->ext.solver;
  if (kind < 0) {
    const char *env = getenv("NUSIF_SOLVER");
    kind = SOLVER_RB;
    if (env && env[0]) {
      if (strcmp(env, "mg-ref") == 0) kind = SOLVER_MG_REF;
      else if (strcmp(env, "mg") == 0) kind = SOLVER_MG;
      else if (strcmp(env, "mg-mixed") == 0) kind = SOLVER_MG_MIXED;
      else if (strcmp(env, "rb") != 0) {
        fail(NUSIF_ERR_ARG, "NUSIF_SOLVER=%s is not rb, mg-ref, mg or mg-mixed", env);
        return;
      }
    }
  }
  ss->kind = kind;
  if (!cuda_ok(cudaMalloc(&ss->d_state, sizeof(SolveState)), "cudaMalloc(solve state)")) return;
  if (!cuda_ok(cudaMallocHost(&ss->h_state, sizeof(SolveState)), "cudaMallocHost(solve state)"))
    return;
  memset(ss->h_state, 0, sizeof(SolveState));
  if (kind == SOLVER_MG || kind == SOLVER_MG_MIXED) {
    if (!mg_setup(s, d, ss)) return;
  } else if (kind == SOLVER_MG_REF) {
    if (verbose()) printf("Using Multigrid solver with %d levels\n", s->levels);
  }
}

// solve, reference src/solver.h:36
double solve(Solver *s, double *p, const double *rhs)
{
  SolverState *ss = solver_state(s);
  if (!ss) {
    fail(NUSIF_ERR_STATE, "solve: solver not initialised by initSolver");
    return NAN;
  }
  const void *pf = p, *rf = rhs;
  if (!await_uploads(&rf, 1) || !await_copies(&pf, 1)) return NAN;
  switch (ss->kind) {
  case SOLVER_RB: return solve_rb(s, ss, p, rhs);
  case SOLVER_MG_REF: return solve_mg_ref(s, ss, p, rhs);
  default: return mg_solve(s, ss, p, rhs);
  }
}

int nusifSolverIterations(const Solver *s)
{
  SolverState *ss = solver_state(s);
  return ss ? ss->last_iterations : -1;
}

int nusifTimeKernel(Solver *s, const double *p, const double *rhs, int which, int reps,
    double *ms_out)
{
  SolverState *ss = solver_state(s);
  if (!ss || !ms_out || reps < 1) {
    fail(NUSIF_ERR_ARG, "nusifTimeKernel: unknown solver or bad arguments");
    return NUSIF_ERR_ARG;
  }
  if (ss->kind != SOLVER_MG && ss->kind != SOLVER_MG_MIXED) {
    fail(NUSIF_ERR_ARG, "nusifTimeKernel: only the mg and mg-mixed solvers have timing hooks");
    return NUSIF_ERR_ARG;
  }
  return mg_time_kernel(ss, p, rhs, which, reps, ms_out) ? NUSIF_OK : NUSIF_ERR_CUDA;
}

void nusifFreeSolver(Solver *s)
{
  SolverState *ss = solver_state(s);
  if (!ss) return;
  cudaStreamSynchronize(stream());
  guess_free(ss->guess);
  ss->guess = nullptr;
  mg_free(s, ss);
  if (ss->d_state) cudaFree(ss->d_state);
  if (ss->h_state) cudaFreeHost(ss->h_state);
  reduce_scratch_free(ss->red);
  solver_state_erase(s);
}

}  // extern "C"
