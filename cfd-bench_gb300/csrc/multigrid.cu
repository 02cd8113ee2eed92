// Geometric multigrid pressure solvers (solver kinds "mg" and "mg-mixed").
//
// The reference's multigrid (src/solver-mg.c:299-402) never applies its
// coarse-grid correction and, sequentially, never coarsens; these solvers are
// the corrected algorithm (its CPU restatement: oracle/nusif_oracle_mg.c):
//  - levels: an axis is halved while its size is even and >= 16;
//  - operator: 7-point Laplacian, homogeneous Neumann walls applied without
//    ghost cells (a neighbour outside the domain is the cell itself);
//  - smoother: red-black, first colour (i + j + k) even (0-based),
//    x -= omega r / diag (omega = mg_omega; 1 is Gauss-Seidel);
//  - restriction: average of the children of the residual; prolongation:
//    trilinear (3/4, 1/4 per coarsened axis), added to x;
//  - V(pre, post) cycles; coarsest level solved exactly by a dense inverse
//    when it has at most kMaxDirect cells, else by fixed sweeps from zero;
//  - right-hand side made mean-free; stop at ||b - Ap|| <= rtol ||b||.
//  mg:       all FP64, p itself is the fine-level unknown; the residual norm
//            is folded in the fine restriction after pre-smoothing.
//  mg-mixed: FP64 residual of p (norm, mean shift) -> FP32 V-cycles for the
//            correction until ||r - A e|| <= theta rtol ||b|| (theta =
//            mg_theta, at most mg_inner cycles) -> p += e in FP64
//            (iterative refinement; the FP64 residual decides the stop).
// Every kernel returns at once when the device-side done flag is up. By
// default each solve is one CUDA graph whose device while-loops run the
// V-cycles; the host-driven path queues whole cycles in chunks and reads the
// state once per chunk.
#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

#include "df32.cuh"
#include "fp_bits.cuh"
#include "nusif_internal.h"
#include "reduce.cuh"
#include "solver_internal.h"
#include "unet_internal.h"

namespace nusif {

constexpr int kMaxLevels = 16;
constexpr int kMaxDirect = 1024;  // largest coarsest level solved exactly (dense inverse)

struct MgState {
  double shift;      // mean of the right-hand side
  double nb2;        // ||rhs - shift||^2
  double res2;       // last FP64 ||b - Ap||^2
  double tol2;       // rtol^2 * nb2
  double rtol2;
  double theta2;     // mg-mixed: (target of the FP32 correction / rtol)^2
  double tol_inner;  // mg-mixed: theta2 * rtol^2 * nb2, target of the FP32 correction
  double res2_inner; // mg-mixed: last ||r32 - A e||^2
  int cycles;        // V-cycles done
  int outer;         // mg-mixed: FP64 residual evaluations that found work to do
  int maxcycles;
  int done;          // the solve is finished: every kernel returns at once
  int inner_done;    // mg-mixed: this outer iteration's correction is good enough
  int loops;         // units run by a graph while-loop (its independent stop)
  int inner_it;      // mg-mixed: FP32 V-cycles of the current correction (graph inner loop)
  int need_norm;     // the one-pass norm of the right-hand side was not trusted
};

// what the fold of a fine-level restriction decides
enum { FOLD_NONE = 0, FOLD_OUTER = 1, FOLD_INNER = 2 };

struct MgLevelDesc {
  int n[3];
  int r[3];  // coarsening ratio from the finer level
  double ih2[3];
  double relax = 1.0;  // smoother: x -= relax * r / diag (Gauss-Seidel at 1)
};

// A level's array view: interior cell (i,j,k), 0-based, lives at
// off + i + j*sy + k*sz (padded reference layout for p/rhs, compact otherwise).
template <typename T>
struct View {
  T *x;
  const T *b;
  int nx, ny, nz;
  int sy, sz, off;
  T ex, ey, ez, diag, inv_diag;
};

struct MgHierarchy {
  int nl = 0;
  int mode = 0;  // 0 mg, 1 mg-mixed
  MgLevelDesc lv[kMaxLevels];
  double *x64[kMaxLevels] = {};
  double *b64[kMaxLevels] = {};
  float *x32[kMaxLevels] = {};   // current FP32 unknown of each level
  float *x32b[kMaxLevels] = {};  // its ping-pong partner for the one-kernel sweep
  float *b32[kMaxLevels] = {};
  MgState *d_state = nullptr;
  MgState *h_state = nullptr;
  ReduceScratch red;
  int pre = 2, post = 2, coarse_sweeps = 0, maxcycles = 100;
  double *minv64 = nullptr;  // exact coarsest solve (device), mg
  float *minv32 = nullptr;   // the same in FP32, mg-mixed
  double rtol = 1e-6;
  int last_cycles = 0;  // queue size of the previous solve (cycles, or outer iterations)
  int inner = 4;        // mg-mixed: most FP32 V-cycles per FP64 residual
  double theta = 0.9;   // mg-mixed: FP32 correction target as a fraction of rtol
  int guess = 0;        // 1: start from 2 p(n-1) - p(n-2)
  double *p_prev = nullptr;   // padded copy of the previous solve's result (guess >= 1)
  double *p_prev2 = nullptr;  // and of the one before (guess >= 2)
  double *p_prev3 = nullptr;  // and of the one before that (guess 3)
  int *d_hist = nullptr;      // device: earlier solutions kept (0, 1, 2)
  // the solve as one CUDA graph (head, while-loops, tail) for fixed p / rhs
  cudaGraphExec_t graph = nullptr;
  const double *graph_p = nullptr, *graph_rhs = nullptr;
  cudaStream_t cap[3] = {};  // capture streams: graph, outer body, inner body
  bool use_graph = true;     // mg_graph: the host-driven solve runs as one graph
  int tail_l0 = 0;           // first level of the one-kernel coarse tail (0: none)
  int kc[kMaxLevels] = {};   // planes per block of each level's one-kernel sweep (0: by rule)
  // FP32 sweeps skipped inside a V-cycle copy x along (odd pre- or post-sweep counts)
  int keep_on_skip = 0;
  double *stats2 = nullptr;  // per-block sums of squares of the right-hand side
  // kernels per part of the graph (counted at capture): head, one outer unit
  // without its inner loop, one inner V-cycle, tail
  int n_head = 0, n_outer = 0, n_inner = 0, n_tail = 0;
  // mg-mixed graph without nested loops: kernels of the unrolled prefix (always
  // launched) and of one iteration of the loop that follows it
  int n_prefix = 0, n_body = 0;
  bool unrolled = false;
  int n_inner_capture = 0;  // scratch while capturing
  bool mx_df = true;  // mg-mixed: fine residual in double-float arithmetic (key arith)
  double *h_ptrs[2 * kMaxLevels] = {};  // exposed through Solver::r / Solver::e
};

namespace {

constexpr int kBX = 32, kBY = 8, kNT = kBX * kBY;

// V-cycle kernels stop when the solve is done or (mg-mixed) when the current
// correction already meets its target; inner_done stays 0 for FP64 mg
__device__ __forceinline__ bool mg_done(const MgState *st)
{
  const volatile int *f = reinterpret_cast<const volatile int *>(&st->done);
  const volatile int *g = reinterpret_cast<const volatile int *>(&st->inner_done);
  return *f != 0 || *g != 0;
}

__device__ __forceinline__ bool solve_finished(const MgState *st)
{
  return *reinterpret_cast<const volatile int *>(&st->done) != 0;
}

// x = 0 as a kernel (a plain kernel node wherever the launch is captured)
template <typename T>
__global__ void k_zero(T *__restrict__ x, int64_t n)
{
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    x[q] = (T)0;
}

// the integer-pipe conversions of the mixed-precision kernels, element-wise
// (nusifConvertF64ToF32 / nusifConvertF32ToF64)
__global__ void k_to_f32(const double *__restrict__ x, float *__restrict__ y, int64_t n)
{
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    y[q] = to_f32_rn(x[q]);
}

__global__ void k_to_f64(const float *__restrict__ x, double *__restrict__ y, int64_t n)
{
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    y[q] = to_f64(x[q]);
}

template <typename T>
__device__ __forceinline__ T lap_at(const View<T> &v, const T *x, int i, int j, int k, int64_t c,
    T xc)
{
  const T sx = (i > 0 ? x[c - 1] : xc) + (i < v.nx - 1 ? x[c + 1] : xc);
  const T sy = (j > 0 ? x[c - v.sy] : xc) + (j < v.ny - 1 ? x[c + v.sy] : xc);
  const T sz = (k > 0 ? x[c - v.sz] : xc) + (k < v.nz - 1 ? x[c + v.sz] : xc);
  return sx * v.ex + sy * v.ey + sz * v.ez - v.diag * xc;
}

// One colour of a red-black Gauss-Seidel sweep. ZERO: the sweep starts from
// x = 0 (the centre is not read; in the odd pass neither are neighbours).
// A thread owns the cell pair (2t, 2t+1) of a row and relaxes the one of the
// pass's colour, walking kb planes.
template <typename T, bool ZERO>
__global__ void __launch_bounds__(kNT) k_mg_smooth(View<T> v, int colour, const double *shift,
    int kb, const MgState *st)
{
  if (mg_done(st)) return;
  const int t = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  const int k0 = blockIdx.z * kb;
  if (j >= v.ny) return;
  const T sh = shift ? (T)(*shift) : (T)0;
  const int k1 = min(k0 + kb, v.nz);
  for (int k = k0; k < k1; k++) {
    const int i = 2 * t + (((j + k + 1) & 1) == colour ? 0 : 1);
    if (i >= v.nx) continue;
    const int64_t c = v.off + (int64_t)k * v.sz + (int64_t)j * v.sy + i;
    if (ZERO && colour == 1) {
      v.x[c] = -(v.b[c] - sh) * v.inv_diag;
    } else {
      const T xc = ZERO ? (T)0 : v.x[c];
      const T r = (v.b[c] - sh) - lap_at(v, v.x, i, j, k, c, xc);
      v.x[c] = xc - r * v.inv_diag;
    }
  }
}

// The FP32 pass on levels with an even row length (every coarsened level and
// even fine grids): the pair (2t, 2t+1) is read as one 8-byte vector in the
// row and in the four neighbouring rows, the far x-neighbour comes from the
// adjacent lane, so each warp reads whole 32-byte sectors. Same arithmetic
// as k_mg_smooth<float>.
template <bool ZERO>
__global__ void __launch_bounds__(kNT) k_mg_smooth_f2(View<float> v, int colour, int kb,
    const MgState *st)
{
  if (mg_done(st)) return;
  const int t = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  const int k0 = blockIdx.z * kb;
  if (j >= v.ny) return;  // whole warps: a warp is one row of 32 threads
  const int k1 = min(k0 + kb, v.nz);
  const int npair = v.nx >> 1;
  const bool live = t < npair;
  const int tt = live ? t : npair - 1;  // loads stay in the row
  for (int k = k0; k < k1; k++) {
    const int a = ((j + k + 1) & 1) == colour ? 0 : 1;  // which cell of the pair is updated
    const int i = 2 * tt + a;
    const int64_t row = (int64_t)k * v.sz + (int64_t)j * v.sy;
    const float2 pc = *reinterpret_cast<const float2 *>(v.x + row + 2 * tt);
    // neighbours across the pair boundary: lane-1's right cell, lane+1's left cell
    float left = __shfl_up_sync(0xffffffffu, pc.y, 1);
    float right = __shfl_down_sync(0xffffffffu, pc.x, 1);
    if (threadIdx.x == 0 && tt > 0) left = v.x[row + 2 * tt - 1];
    if (threadIdx.x == kBX - 1 && tt + 1 < npair) right = v.x[row + 2 * tt + 2];
    const float xc = ZERO ? 0.0f : (a ? pc.y : pc.x);
    float xw = a ? pc.x : left;    // x(i-1)
    float xe = a ? right : pc.y;   // x(i+1)
    if (i == 0) xw = xc;
    if (i == v.nx - 1) xe = xc;
    const int64_t c = row + i;
    const int64_t pair = row + 2 * tt;
    auto pick = [a](float2 q) { return a ? q.y : q.x; };
    const float bc = pick(*reinterpret_cast<const float2 *>(v.b + pair));
    if (ZERO && colour == 1) {
      if (live) v.x[c] = -bc * v.inv_diag;
      continue;
    }
    const float ys = j > 0 ? pick(*reinterpret_cast<const float2 *>(v.x + pair - v.sy)) : xc;
    const float yn = j < v.ny - 1 ? pick(*reinterpret_cast<const float2 *>(v.x + pair + v.sy)) : xc;
    const float zb = k > 0 ? pick(*reinterpret_cast<const float2 *>(v.x + pair - v.sz)) : xc;
    const float zt = k < v.nz - 1 ? pick(*reinterpret_cast<const float2 *>(v.x + pair + v.sz)) : xc;
    const float lap = (xw + xe) * v.ex + (ys + yn) * v.ey + (zb + zt) * v.ez - v.diag * xc;
    const float r = bc - lap;
    if (live) v.x[c] = xc - r * v.inv_diag;
  }
}

// Residual of the fine level averaged into the coarse right-hand side. One
// thread per coarse cell. FOLD != FOLD_NONE: also sum r^2 (FP64) and let the
// last block fold the partials and decide: FOLD_OUTER (FP64 mg) counts the
// cycle and stops the solve at rtol; FOLD_INNER (mg-mixed) counts the FP32
// V-cycle and ends this correction once it meets its target.
template <typename T, int FOLD>
__global__ void __launch_bounds__(kNT) k_mg_restrict(View<T> f, T *bc, int cnx, int cny, int cnz,
    int rx, int ry, int rz, T inv_count, const double *shift, MgState *st,
    double *partials, unsigned *ticket)
{
  constexpr bool ACCUM = FOLD != FOLD_NONE;
  if (mg_done(st)) return;
  const int64_t ncoarse = (int64_t)cnx * cny * cnz;
  const T sh = shift ? (T)(*shift) : (T)0;
  double acc = 0.0;
  for (int64_t q = blockIdx.x * (int64_t)kNT + threadIdx.x; q < ncoarse;
       q += (int64_t)gridDim.x * kNT) {
    const int I = (int)(q % cnx);
    const int64_t rest = q / cnx;
    const int J = (int)(rest % cny);
    const int K = (int)(rest / cny);
    T sum = 0;
    for (int dk = 0; dk < rz; dk++)
      for (int dj = 0; dj < ry; dj++)
        for (int di = 0; di < rx; di++) {
          const int i = I * rx + di, j = J * ry + dj, k = K * rz + dk;
          const int64_t c = f.off + (int64_t)k * f.sz + (int64_t)j * f.sy + i;
          const T r = (f.b[c] - sh) - lap_at(f, f.x, i, j, k, c, f.x[c]);
          sum += r;
          if (ACCUM) acc += (double)r * (double)r;
        }
    if (bc) bc[q] = sum * inv_count;
  }
  if (!ACCUM) return;
  __shared__ double sm[kNT / 32];
  acc = block_reduce_sum<kNT>(acc, sm);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = acc;
    last = ticket_is_last(ticket);
  }
  __syncthreads();
  if (!last) return;
  const double total = fold_partials<kNT>(partials, gridDim.x, sm);
  if (threadIdx.x == 0) {
    const int c = st->cycles + 1;
    st->cycles = c;
    if (FOLD == FOLD_OUTER) {
      st->res2 = total;
      st->done = (total <= st->tol2) || (c >= st->maxcycles);
    } else {
      st->res2_inner = total;
      st->inner_done = total <= st->tol_inner;
    }
    *ticket = 0;
  }
}

// The same restriction when x is halved (rx == 2), one thread per coarse cell
// on a 3-D grid (32 x 8 coarse (I, J) per block, planes K strided by the
// grid): no index division, children in the same order as k_mg_restrict.
template <typename T, int FOLD>
__global__ void __launch_bounds__(kNT) k_mg_restrict_x2(View<T> f, T *bc, int cnx, int cny,
    int cnz, int ry, int rz, T inv_count, const double *shift, MgState *st, double *partials,
    unsigned *ticket)
{
  constexpr bool ACCUM = FOLD != FOLD_NONE;
  if (mg_done(st)) return;
  const T sh = shift ? (T)(*shift) : (T)0;
  const int I = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y * 8 + threadIdx.y;
  double acc = 0.0;
  if (I < cnx && J < cny) {
    for (int K = blockIdx.z; K < cnz; K += gridDim.z) {
      T sum = 0, sq = 0;
      for (int dk = 0; dk < rz; dk++)
        for (int dj = 0; dj < ry; dj++)
#pragma unroll
          for (int di = 0; di < 2; di++) {
            const int i = 2 * I + di, j = J * ry + dj, k = K * rz + dk;
            const int64_t c = f.off + (int64_t)k * f.sz + (int64_t)j * f.sy + i;
            const T r = (f.b[c] - sh) - lap_at(f, f.x, i, j, k, c, f.x[c]);
            sum += r;
            // FP32 levels: a coarse cell's (at most 8) squares summed in FP32,
            // then one FP64 add (the FP64 pipe would bound this kernel)
            if constexpr (sizeof(T) == sizeof(float)) {
              if (ACCUM) sq += r * r;
            } else {
              if (ACCUM) acc += (double)r * (double)r;
            }
          }
      if constexpr (sizeof(T) == sizeof(float)) {
        if (ACCUM) acc += (double)sq;
      }
      if (bc) bc[((int64_t)K * cny + J) * cnx + I] = sum * inv_count;
    }
  }
  if (!ACCUM) return;
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
  const double total = fold_partials<kNT>(partials, gridDim.x * gridDim.y * gridDim.z, sm);
  if (flat_tid() == 0) {
    const int c = st->cycles + 1;
    st->cycles = c;
    if (FOLD == FOLD_OUTER) {
      st->res2 = total;
      st->done = (total <= st->tol2) || (c >= st->maxcycles);
    } else {
      st->res2_inner = total;
      st->inner_done = total <= st->tol_inner;
    }
    *ticket = 0;
  }
}

// FP32 levels halved on every axis (rows of even length, no shift): one
// thread per coarse column (I, J) walks a contiguous chunk of coarse planes.
// A fine plane is held as 4 rows x 4 columns (rows 2J-1 .. 2J+2, columns
// 2I-1 .. 2I+2; a neighbour beyond a wall is the cell itself, so the clamped
// index gives it): each row comes as one 8-byte load and its outer columns
// from the neighbouring lanes, and the planes shared by consecutive fine
// planes stay in registers. Same arithmetic and summation order as
// k_mg_restrict_x2<float>, with 12 vector loads per coarse cell instead of 64
// scalar ones.
template <int FOLD>
__global__ void __launch_bounds__(kNT) k_mg_restrict_f32(View<float> f, float *bc, int cnx,
    int cny, int cnz, int kcz, float inv_count, MgState *st, double *partials, unsigned *ticket)
{
  constexpr bool ACCUM = FOLD != FOLD_NONE;
  if (mg_done(st)) return;
  const int lane = threadIdx.x;  // blockDim.x == 32: a warp is one coarse row
  const int I = blockIdx.x * 32 + lane, J = blockIdx.y * 8 + threadIdx.y;
  const bool in = I < cnx && J < cny;
  const int i0 = 2 * min(I, cnx - 1), j0 = 2 * min(J, cny - 1);  // loads stay in bounds
  const bool has_l = i0 > 0, has_r = i0 + 2 < f.nx;
  int64_t roff[4];
#pragma unroll
  for (int r = 0; r < 4; r++) roff[r] = (int64_t)min(max(j0 - 1 + r, 0), f.ny - 1) * f.sy + i0;
  const float *__restrict__ x = f.x;
  const float *__restrict__ b = f.b;
  const float ex = f.ex, ey = f.ey, ez = f.ez, dg = f.diag;
  auto load_plane = [&](float(&v)[4][4], int k) {
    const int64_t ko = f.off + (int64_t)min(max(k, 0), f.nz - 1) * f.sz;
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const float2 a = *reinterpret_cast<const float2 *>(x + ko + roff[r]);
      float lv = __shfl_up_sync(0xffffffffu, a.y, 1);
      float rv = __shfl_down_sync(0xffffffffu, a.x, 1);
      if (lane == 0 && has_l) lv = x[ko + roff[r] - 1];
      if (lane == 31 && has_r) rv = x[ko + roff[r] + 2];
      v[r][0] = has_l ? lv : a.x;
      v[r][1] = a.x;
      v[r][2] = a.y;
      v[r][3] = has_r ? rv : a.y;
    }
  };
  auto resid = [&](const float(&vm)[4][4], const float(&vc)[4][4], const float(&vp)[4][4],
                   int kf, float &sum, float &sq) {
    const int64_t kb = f.off + (int64_t)kf * f.sz;
#pragma unroll
    for (int dj = 0; dj < 2; dj++) {
      const float2 bb = *reinterpret_cast<const float2 *>(b + kb + roff[1 + dj]);
#pragma unroll
      for (int di = 0; di < 2; di++) {
        const int rj = 1 + dj, ci = 1 + di;
        const float xc = vc[rj][ci];
        const float sx = vc[rj][ci - 1] + vc[rj][ci + 1];
        const float sy = vc[rj - 1][ci] + vc[rj + 1][ci];
        const float sz = vm[rj][ci] + vp[rj][ci];
        const float lap = sx * ex + sy * ey + sz * ez - dg * xc;
        const float r = (di ? bb.y : bb.x) - lap;
        sum += r;
        if (ACCUM) sq += r * r;
      }
    }
  };
  double acc = 0.0;
  const int K0 = blockIdx.z * kcz, K1 = min(K0 + kcz, cnz);
  if (K0 < K1) {
    float p0[4][4], p1[4][4], p2[4][4], p3[4][4];
    load_plane(p0, 2 * K0 - 1);
    load_plane(p1, 2 * K0);
    for (int K = K0; K < K1; K++) {
      float sum = 0.0f, sq = 0.0f;
      load_plane(p2, 2 * K + 1);
      resid(p0, p1, p2, 2 * K, sum, sq);
      load_plane(p3, 2 * K + 2);
      resid(p1, p2, p3, 2 * K + 1, sum, sq);
      if (in) {
        bc[((int64_t)K * cny + J) * cnx + I] = sum * inv_count;
        if (ACCUM) acc += to_f64(sq);
      }
#pragma unroll
      for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
          p0[r][c] = p2[r][c];
          p1[r][c] = p3[r][c];
        }
    }
  }
  if (!ACCUM) return;
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
  const double total = fold_partials<kNT>(partials, gridDim.x * gridDim.y * gridDim.z, sm);
  if (flat_tid() == 0) {
    const int c = st->cycles + 1;
    st->cycles = c;
    if (FOLD == FOLD_OUTER) {
      st->res2 = total;
      st->done = (total <= st->tol2) || (c >= st->maxcycles);
    } else {
      st->res2_inner = total;
      st->inner_done = total <= st->tol_inner;
    }
    *ticket = 0;
  }
}

// FP64 residual of p (padded layout) into the FP32 fine right-hand side, with
// its FP64 norm folded by the last block: the mixed-precision stop test. It
// also opens the next correction (inner_done = 0). count_cycles: one FP32
// V-cycle per outer iteration is counted here (single-level grids, where no
// fine restriction counts them). e_zero (may be null): the FP32 correction,
// set to zero for the V-cycles that follow (the graph's inner loop, whose
// V-cycles all start from the current correction).
__global__ void __launch_bounds__(kNT) k_mx_residual(View<double> f, float *r32, MgState *st,
    double *partials, unsigned *ticket, int count_cycles, float *e_zero)
{
  if (solve_finished(st)) return;
  const int64_t n = (int64_t)f.nx * f.ny * f.nz;
  const double sh = st->shift;
  double acc = 0.0;
  const int64_t q0 = blockIdx.x * (int64_t)kNT + threadIdx.x, stride = (int64_t)gridDim.x * kNT;
  FlatWalk w(q0, stride, f.nx, f.ny);
  for (int64_t q = q0; q < n; q += stride, w.advance(f.nx, f.ny)) {
    const int i = w.i, j = w.j, k = w.k;
    const int64_t c = f.off + (int64_t)k * f.sz + (int64_t)j * f.sy + i;
    const double *x = f.x;
    const double xc = x[c];
    const double sx = (i > 0 ? x[c - 1] : xc) + (i < f.nx - 1 ? x[c + 1] : xc);
    const double sy = (j > 0 ? x[c - f.sy] : xc) + (j < f.ny - 1 ? x[c + f.sy] : xc);
    const double sz = (k > 0 ? x[c - f.sz] : xc) + (k < f.nz - 1 ? x[c + f.sz] : xc);
    // r = (b - shift) - A x with the shift folded into the first FMA: eight
    // FP64 instructions, the norm's FMA the ninth, the FP32 copy on the
    // integer pipe
    double t = fma(-f.diag, xc, sh);
    t = fma(sx, f.ex, t);
    t = fma(sy, f.ey, t);
    t = fma(sz, f.ez, t);
    const double r = f.b[c] - t;
    r32[q] = to_f32_rn(r);
    if (e_zero) e_zero[q] = 0.0f;
    acc = fma(r, r, acc);
  }
  __shared__ double sm[kNT / 32];
  acc = block_reduce_sum<kNT>(acc, sm);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = acc;
    last = ticket_is_last(ticket);
  }
  __syncthreads();
  if (!last) return;
  const double total = fold_partials<kNT>(partials, gridDim.x, sm);
  if (threadIdx.x == 0) {
    st->res2 = total;
    const int m = st->outer;  // corrections applied before this residual
    st->done = (total <= st->tol2) || (m >= st->maxcycles);
    if (!st->done) {
      st->outer = m + 1;
      st->inner_done = 0;
      st->inner_it = 0;
      if (count_cycles) st->cycles += 1;
    }
    *ticket = 0;
  }
}

// The same residual, stop test and side effects as k_mx_residual, with the
// stencil carried in double-float arithmetic (df32.cuh: pairs of FP32
// numbers on the FP32 pipe, about 2^-47 of the operands) instead of nine FP64
// instructions per cell, which bound that kernel at 256^3 (FP64 issue, not
// HBM). The residual's error is then a few units of 2^-47 of diag |x|, which
// near convergence is the scale of the cancellation b - A x; the stop test
// compares it with rtol ||b||, 1e-6 to 1e-8 here, far above that error.
// The norm is accumulated as a pair and folded in FP64.
//
// Mapping: a 32 x 8 tile of columns marching over kb planes. Plane k's pairs
// (the tile and a one-cell ring) sit in shared memory, double-buffered so a
// plane needs one barrier; the column's k-1 and k+1 pairs stay in registers.
// Indices outside the grid are clamped to it, which is the Neumann rule
// itself (a missing neighbour is the cell). Each value is split into its pair
// once per block (ring cells once more by the neighbouring block).
// the operator's constants as pairs, formed on the host (GB300 runs double
// <-> float conversions on its FP64 pipe)
struct DfStencil {
  df::f2 ex, ey, ez, mdiag;
};

__global__ void __launch_bounds__(kNT, 4) k_mx_residual_df(View<double> f, DfStencil cs, float *r32,
    MgState *st, double *partials, unsigned *ticket, int count_cycles, float *e_zero, int kb)
{
  using namespace df;
  if (solve_finished(st)) return;
  __shared__ f2 pl[2][kBY + 2][kBX + 2];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kBX + tx;
  const int i0 = blockIdx.x * kBX, j0 = blockIdx.y * kBY;
  const bool active = i0 + tx < f.nx && j0 + ty < f.ny;
  const int i = min(i0 + tx, f.nx - 1), j = min(j0 + ty, f.ny - 1);
  const int k0 = blockIdx.z * kb, k1 = min(k0 + kb, f.nz);
  const double *x = f.x;
  // ring cell of this thread (threads 0..79): rows j0-1 and j0+8, columns i0-1 and i0+32
  const bool ring = tid < 2 * kBX + 2 * kBY;
  int rr = 0, rc = 0, roff = 0;
  if (ring) {
    if (tid < 2 * kBX) {
      rc = (tid & (kBX - 1)) + 1;
      rr = tid < kBX ? 0 : kBY + 1;
    } else {
      const int q = tid - 2 * kBX;
      rr = (q & (kBY - 1)) + 1;
      rc = q < kBY ? 0 : kBX + 1;
    }
    const int ri = min(max(i0 - 1 + rc, 0), f.nx - 1), rj = min(max(j0 - 1 + rr, 0), f.ny - 1);
    roff = f.off + rj * f.sy + ri;
  }
  const int coff = f.off + j * f.sy + i;
  double acc_d = 0.0;
  if (k0 < k1) {
    const f2 ex = cs.ex, ey = cs.ey, ez = cs.ez, mdiag = cs.mdiag, sh = split(st->shift);
    const auto plane = [&](int k) { return (int64_t)min(max(k, 0), f.nz - 1) * f.sz; };
    f2 zb = split(x[plane(k0 - 1) + coff]);
    f2 zc = split(x[plane(k0) + coff]);
    double xn = x[plane(k0 + 1) + coff];           // the column's next plane (raw)
    double rn = ring ? x[plane(k0) + roff] : 0.0;  // this thread's ring cell of the next plane
    f2 acc{ 0.0f, 0.0f };
    int buf = 0;
    for (int k = k0; k < k1; k++) {
      const int64_t pk = (int64_t)k * f.sz;
      const double bv = f.b[pk + coff];
      pl[buf][ty + 1][tx + 1] = zc;
      if (ring) pl[buf][rr][rc] = split(rn);
      const f2 zt = split(xn);
      if (k + 1 < k1) {
        xn = x[plane(k + 2) + coff];
        if (ring) rn = x[pk + f.sz + roff];
      }
      __syncthreads();
      // unnormalised pairs inside the stencil (only pair arithmetic follows),
      // the residual itself renormalised (its hi is the FP32 copy)
      const f2 sx = add_u(pl[buf][ty + 1][tx], pl[buf][ty + 1][tx + 2]);
      const f2 sy = add_u(pl[buf][ty][tx + 1], pl[buf][ty + 2][tx + 1]);
      const f2 sz = add_u(zb, zt);
      f2 t = fma_u(mdiag, zc, sh);
      t = fma_u(sx, ex, t);
      t = fma_u(sy, ey, t);
      t = fma_u(sz, ez, t);
      const f2 r = sub(split(bv), t);
      if (active) {
        const int64_t q = ((int64_t)k * f.ny + j) * f.nx + i;
        r32[q] = r.hi;  // the pair is renormalised: hi is its value rounded to FP32
        if (e_zero) e_zero[q] = 0.0f;
        acc = add(acc, mul_u(r, r));
      }
      zb = zc;
      zc = zt;
      buf ^= 1;
    }
    acc_d = to_double(acc);
  }
  __shared__ double sm[kNT / 32];
  acc_d = block_reduce_sum<kNT>(acc_d, sm);
  __shared__ bool last;
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (tid == 0) {
    partials[bid] = acc_d;
    last = ticket_is_last(ticket);
  }
  __syncthreads();
  if (!last) return;
  const double total = fold_partials<kNT>(partials, gridDim.x * gridDim.y * gridDim.z, sm);
  if (tid == 0) {
    st->res2 = total;
    const int m = st->outer;  // corrections applied before this residual
    st->done = (total <= st->tol2) || (m >= st->maxcycles);
    if (!st->done) {
      st->outer = m + 1;
      st->inner_done = 0;
      st->inner_it = 0;
      if (count_cycles) st->cycles += 1;
    }
    *ticket = 0;
  }
}

// x_f += trilinear interpolation of x_c; one thread per fine cell
template <typename T>
__global__ void __launch_bounds__(kNT) k_mg_prolong(View<T> f, const T *xc, int cnx, int cny,
    int cnz, int rx, int ry, int rz, const MgState *st)
{
  if (mg_done(st)) return;
  const int64_t n = (int64_t)f.nx * f.ny * f.nz;
  for (int64_t q = blockIdx.x * (int64_t)kNT + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * kNT) {
    const int fi[3] = { (int)(q % f.nx), (int)((q / f.nx) % f.ny), (int)(q / ((int64_t)f.nx * f.ny)) };
    const int cn[3] = { cnx, cny, cnz };
    const int rr[3] = { rx, ry, rz };
    int P[3], Q[3];
    T w[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      if (rr[a] == 2) {
        P[a] = fi[a] >> 1;
        const int nb = (fi[a] & 1) ? P[a] + 1 : P[a] - 1;
        Q[a] = (nb < 0 || nb >= cn[a]) ? P[a] : nb;
        w[a] = (T)0.25;
      } else {
        P[a] = fi[a];
        Q[a] = fi[a];
        w[a] = (T)0;
      }
    }
    const int64_t sy = cnx, sz = (int64_t)cnx * cny;
    T v[2][2];
#pragma unroll
    for (int dz = 0; dz < 2; dz++)
#pragma unroll
      for (int dy = 0; dy < 2; dy++) {
        const int64_t base = (int64_t)(dz ? Q[2] : P[2]) * sz + (int64_t)(dy ? Q[1] : P[1]) * sy;
        const T a0 = xc[base + P[0]], a1 = xc[base + Q[0]];
        v[dz][dy] = a0 + w[0] * (a1 - a0);
      }
    const T y0 = v[0][0] + w[1] * (v[0][1] - v[0][0]);
    const T y1 = v[1][0] + w[1] * (v[1][1] - v[1][0]);
    const int64_t c = f.off + (int64_t)fi[2] * f.sz + (int64_t)fi[1] * f.sy + fi[0];
    f.x[c] += y0 + w[2] * (y1 - y0);
  }
}

// x_f += trilinear interpolation of x_c when x was coarsened (rx == 2) and
// the fine rows hold a multiple of four cells: one thread per four
// consecutive fine cells (two coarse x-positions), so the four coarse values
// of each (y, z) line are loaded once for four cells, and (VEC, FP32 compact
// rows) the fine cells move as one 16-byte vector. Same interpolation order
// as k_mg_prolong_x2 (x, then y, then z).
template <typename T, bool VEC>
__global__ void __launch_bounds__(kNT) k_mg_prolong_x4(View<T> f, const T *__restrict__ xc,
    int cnx, int cny, int cnz, int ry, int rz, const MgState *st)
{
  if (mg_done(st)) return;
  const int Q = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (4 * Q >= f.nx || j >= f.ny) return;
  int Py, Qy;
  T wy;
  if (ry == 2) {
    Py = j >> 1;
    const int nb = (j & 1) ? Py + 1 : Py - 1;
    Qy = (nb < 0 || nb >= cny) ? Py : nb;
    wy = (T)0.25;
  } else {
    Py = Qy = j;
    wy = (T)0;
  }
  // planes strided by the grid: a few blocks per SM, each over several planes
  for (int k = blockIdx.z; k < f.nz; k += gridDim.z) {
  int Pz, Qz;
  T wz;
  if (rz == 2) {
    Pz = k >> 1;
    const int nb = (k & 1) ? Pz + 1 : Pz - 1;
    Qz = (nb < 0 || nb >= cnz) ? Pz : nb;
    wz = (T)0.25;
  } else {
    Pz = Qz = k;
    wz = (T)0;
  }
  const int X0 = 2 * Q, X1 = X0 + 1;
  const int Xm = X0 > 0 ? X0 - 1 : X0, Xp = X1 < cnx - 1 ? X1 + 1 : X1;
  const int64_t sy = cnx, sz = (int64_t)cnx * cny;
  T o[4][2][2];  // per fine cell, per (z, y) line: the x-interpolated value
#pragma unroll
  for (int dz = 0; dz < 2; dz++)
#pragma unroll
    for (int dy = 0; dy < 2; dy++) {
      const int64_t base = (int64_t)(dz ? Qz : Pz) * sz + (int64_t)(dy ? Qy : Py) * sy;
      const T am = xc[base + Xm], a0 = xc[base + X0], a1 = xc[base + X1], ap = xc[base + Xp];
      o[0][dz][dy] = a0 + (T)0.25 * (am - a0);
      o[1][dz][dy] = a0 + (T)0.25 * (a1 - a0);
      o[2][dz][dy] = a1 + (T)0.25 * (a0 - a1);
      o[3][dz][dy] = a1 + (T)0.25 * (ap - a1);
    }
  T add[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const T y0 = o[q][0][0] + wy * (o[q][0][1] - o[q][0][0]);
    const T y1 = o[q][1][0] + wy * (o[q][1][1] - o[q][1][0]);
    add[q] = y0 + wz * (y1 - y0);
  }
  const int64_t c = f.off + (int64_t)k * f.sz + (int64_t)j * f.sy + 4 * Q;
  if constexpr (VEC) {
    float4 v = *reinterpret_cast<const float4 *>(f.x + c);
    v.x += add[0];
    v.y += add[1];
    v.z += add[2];
    v.w += add[3];
    *reinterpret_cast<float4 *>(f.x + c) = v;
  } else {
#pragma unroll
    for (int q = 0; q < 4; q++) f.x[c + q] += add[q];
  }
  }
}

// One red-black sweep from x = 0 (the first pre-sweep of a V-cycle level),
// FP32 rows of a multiple of four cells. From zero, a first-colour cell
// ((i+j+k) even) relaxes to -b/diag (times the relaxation), and a
// second-colour cell relaxes against those values: its other neighbours are
// second-colour cells, still 0, as is a missing neighbour beyond a wall (the
// cell itself). So the whole sweep is one stencil pass over b, one thread per
// four consecutive cells of a row, writing x_new (the buffer the host swaps
// in), with the arithmetic of the general sweep (k_rbgs_sweep) on x = 0.
__global__ void __launch_bounds__(kNT) k_rb_zero_sweep(View<float> v, float *__restrict__ xnew,
    const MgState *st, int keep)
{
  const int Q = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = v.nx, ny = v.ny, nz = v.nz;
  const int i0 = 4 * Q;
  if (i0 >= nx || j >= ny) return;
  if (mg_done(st)) {
    // skipped inside a V-cycle: leave the zero it would have started from
    if (keep && !solve_finished(st))
      for (int k = blockIdx.z; k < nz; k += gridDim.z)
        *reinterpret_cast<float4 *>(xnew + (int64_t)k * v.sz + (int64_t)j * v.sy + i0) =
            make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const float ex = v.ex, ey = v.ey, ez = v.ez, dg = v.diag, idg = v.inv_diag;
  const float *__restrict__ b = v.b;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int k = blockIdx.z; k < nz; k += gridDim.z) {
    const int64_t c = (int64_t)k * v.sz + (int64_t)j * v.sy + i0;
    const float4 bc = *reinterpret_cast<const float4 *>(b + c);
    const float4 bs = j > 0 ? *reinterpret_cast<const float4 *>(b + c - v.sy) : z4;
    const float4 bn = j < ny - 1 ? *reinterpret_cast<const float4 *>(b + c + v.sy) : z4;
    const float4 bd = k > 0 ? *reinterpret_cast<const float4 *>(b + c - v.sz) : z4;
    const float4 bu = k < nz - 1 ? *reinterpret_cast<const float4 *>(b + c + v.sz) : z4;
    const float brow[6] = { i0 > 0 ? b[c - 1] : 0.f, bc.x, bc.y, bc.z, bc.w,
                            i0 + 4 < nx ? b[c + 4] : 0.f };
    const float bsv[4] = { bs.x, bs.y, bs.z, bs.w }, bnv[4] = { bn.x, bn.y, bn.z, bn.w };
    const float bdv[4] = { bd.x, bd.y, bd.z, bd.w }, buv[4] = { bu.x, bu.y, bu.z, bu.w };
    // a first-colour cell's new value from its own b
    auto first = [&](float bb) { return 0.0f - (bb - 0.0f) * idg; };
    float out[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int i = i0 + q;
      if (((i + j + k) & 1) == 0) {
        out[q] = first(brow[q + 1]);
      } else {
        const float rw = i > 0 ? first(brow[q]) : 0.f, re = i < nx - 1 ? first(brow[q + 2]) : 0.f;
        const float rs = j > 0 ? first(bsv[q]) : 0.f, rn = j < ny - 1 ? first(bnv[q]) : 0.f;
        const float rd = k > 0 ? first(bdv[q]) : 0.f, ru = k < nz - 1 ? first(buv[q]) : 0.f;
        const float sx = rw + re, sy = rs + rn, sz = rd + ru;
        const float lap = sx * ex + sy * ey + sz * ez - dg * 0.0f;
        out[q] = 0.0f - (brow[q + 1] - lap) * idg;
      }
    }
    *reinterpret_cast<float4 *>(xnew + c) = make_float4(out[0], out[1], out[2], out[3]);
  }
}

// x_f += trilinear interpolation of x_c on FP32 levels halved on every axis
// with fine rows of a multiple of four cells (16-byte aligned): one thread per
// four consecutive fine cells of a row walks a chunk of coarse planes K and
// updates fine planes 2K and 2K+1. The x-interpolated values of the two
// coarse rows it needs are kept for coarse planes K-1, K, K+1, so each coarse
// plane is read once per thread, as one 8-byte load per row with the outer
// columns from the neighbouring lanes. Same interpolation order as
// k_mg_prolong_x4 (x, then y, then z).
__global__ void __launch_bounds__(kNT) k_mg_prolong_f32(View<float> f, const float *__restrict__ xc,
    int cnx, int cny, int cnz, int kcz, const MgState *st)
{
  if (mg_done(st)) return;
  const int lane = threadIdx.x;  // blockDim.x == 32: a warp is one fine row
  const int Qraw = blockIdx.x * 32 + lane, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (j >= f.ny) return;  // whole warps: a warp shares one j
  const int nq = f.nx / 4;
  const bool in = Qraw < nq;
  const int Q = min(Qraw, nq - 1);  // loads stay in bounds
  const int X0 = 2 * Q, X1 = X0 + 1;
  const bool has_m = X0 > 0, has_p = X1 < cnx - 1;
  const int Py = j >> 1;
  const int ny_ = (j & 1) ? Py + 1 : Py - 1;
  const int Qy = (ny_ < 0 || ny_ >= cny) ? Py : ny_;
  const int64_t sy = cnx, sz = (int64_t)cnx * cny;
  const float w = 0.25f;
  // y-interpolated values of the four fine cells for one coarse plane
  auto plane = [&](float(&y)[4], int K) {
    const int Kc = min(max(K, 0), cnz - 1);
    float o[2][4];
#pragma unroll
    for (int dy = 0; dy < 2; dy++) {
      const int64_t base = (int64_t)Kc * sz + (int64_t)(dy ? Qy : Py) * sy;
      const float2 a = *reinterpret_cast<const float2 *>(xc + base + X0);
      float am = __shfl_up_sync(0xffffffffu, a.y, 1);
      float ap = __shfl_down_sync(0xffffffffu, a.x, 1);
      if (lane == 0 && has_m) am = xc[base + X0 - 1];
      if (lane == 31 && has_p) ap = xc[base + X1 + 1];
      if (!has_m) am = a.x;
      if (!has_p) ap = a.y;
      o[dy][0] = a.x + w * (am - a.x);
      o[dy][1] = a.x + w * (a.y - a.x);
      o[dy][2] = a.y + w * (a.x - a.y);
      o[dy][3] = a.y + w * (ap - a.y);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) y[q] = o[0][q] + w * (o[1][q] - o[0][q]);
  };
  const int K0 = blockIdx.z * kcz, K1 = min(K0 + kcz, cnz);
  if (K0 >= K1) return;
  float ym[4], y0[4], yp[4];
  plane(ym, K0 - 1);
  plane(y0, K0);
  float *__restrict__ row = f.x + f.off + (int64_t)j * f.sy + 4 * Q;
  for (int K = K0; K < K1; K++) {
    plane(yp, K + 1);
    // fine plane 2K: coarse planes K and K - 1 (K itself at the low wall)
    // fine plane 2K + 1: coarse planes K and K + 1 (K itself at the high wall)
    const bool lo = K > 0, hi = K < cnz - 1;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      float add[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const float yq = h ? (hi ? yp[q] : y0[q]) : (lo ? ym[q] : y0[q]);
        add[q] = y0[q] + w * (yq - y0[q]);
      }
      if (in) {
        float4 *px = reinterpret_cast<float4 *>(row + (int64_t)(2 * K + h) * f.sz);
        float4 v = *px;
        v.x += add[0];
        v.y += add[1];
        v.z += add[2];
        v.w += add[3];
        *px = v;
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      ym[q] = y0[q];
      y0[q] = yp[q];
    }
  }
}

// One whole red-black Gauss-Seidel sweep in one kernel, exact: reads x_old,
// writes x_new (ping-pong), so no block ever reads a value another block
// writes. A block owns a 64 x 8 tile of (i, j) columns and a chunk of planes;
// per plane it relaxes the odd ("red") cells on the tile plus a one-cell ring
// (from old even values: exactly what the first pass of a two-pass sweep
// computes there), then the even cells of the previous plane on the tile
// (from the new odd values and their own old value), and writes both colours
// of that plane. Planes walk with a one-plane lag (odd at k, even at k-1); the
// odd planes just outside the chunk are recomputed, so chunks are
// independent. x_old (tile + two-cell ring) and b (tile + one-cell ring) are
// staged in shared memory by asynchronous copies issued one plane ahead
// (cp.async, completed by cp.async.wait_group), so global latency overlaps
// the arithmetic of the plane before. One sweep reads x and b once and
// writes x once. (A sweep from x = 0 is k_rb_zero_sweep.)
constexpr int kSX = 64, kSY = 8;  // tile (cells)
constexpr int kWX = kSX + 8;      // staged row: tile + 4 cells each side (16-byte chunks)
constexpr int kRY = kSY + 4;      // staged x_old rows: tile + 2-row ring
constexpr int kBYr = kSY + 2;     // staged b rows and odd values: tile + 1-row ring
constexpr int kQX = kSX + 2;      // odd values: tile + 1-cell ring

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// FP32 levels with nx % 4 == 0 (rows start on 16-byte boundaries): every
// staged row is 18 chunks of four cells starting 4 cells left of the tile,
// one chunk per thread per array per plane.
//
// Walls cost no tests per neighbour: the Neumann operator replaces a missing
// neighbour by the cell itself, and the staged x_old already holds that value
// outside the domain (planes beyond a wall are staged as the wall plane, rows
// beyond a wall as the wall row, and the column beyond a wall is patched to
// the wall column); a first-colour ring cell outside the domain stores that
// mirrored old value instead of a relaxed one, which is exactly what its
// second-colour neighbour inside the domain must see there.
__global__ void __launch_bounds__(256) k_rbgs_sweep(View<float> v, float *__restrict__ xnew,
    int kc, const MgState *st, int keep)
{
  if (mg_done(st)) {
    // The host swaps the two buffers after every sweep it launches. A sweep
    // skipped because the correction met its target inside this V-cycle must
    // still leave x where the next kernels look (keep: set when a level's
    // sweeps per V-cycle could be skipped in odd numbers): it copies its chunk.
    if (keep && !solve_finished(st)) {
      const int i0 = blockIdx.x * kSX, j0 = blockIdx.y * kSY, k0 = blockIdx.z * kc;
      const int k1 = min(k0 + kc, v.nz);
      constexpr int kRowChunks = kSX / 4, kPlane = kSY * kRowChunks;
      for (int q = threadIdx.x; q < (k1 - k0) * kPlane; q += 256) {
        const int k = k0 + q / kPlane, rem = q % kPlane;
        const int j = j0 + rem / kRowChunks, i = i0 + 4 * (rem % kRowChunks);
        if (j >= v.ny || i >= v.nx) continue;
        const int64_t c = (int64_t)k * v.sz + (int64_t)j * v.sy + i;
        *reinterpret_cast<float4 *>(xnew + c) = *reinterpret_cast<const float4 *>(v.x + c);
      }
    }
    return;
  }
  constexpr int PX = kRY * kWX, PB = kBYr * kWX, PR = kBYr * kQX;  // floats per staged plane
  // Five x_old slots and four b and first-colour slots: the copies a thread
  // issues for plane k + 3 never land in a slot that a slower warp may still
  // read for the second colour of plane k - 1, so each plane needs two
  // barriers, not three.
  __shared__ __align__(16) float xo[5 * PX];  // x_old planes, slot = plane mod 5
  __shared__ __align__(16) float bs[4 * PB];  // b planes, slot = plane & 3
  __shared__ float xr[4 * PR];                // new first-colour values, slot = plane & 3
  const int nx = v.nx, ny = v.ny, nz = v.nz;
  const int i0 = blockIdx.x * kSX, j0 = blockIdx.y * kSY;
  const int k0 = blockIdx.z * kc, k1 = min(k0 + kc, nz);
  const int tid = threadIdx.x;
  // staging: this thread's 16-byte chunk (row cr, chunk cc) of a staged plane
  constexpr int kChunks = kWX / 4;  // 18 per row
  const int cr = tid / kChunks, cc = tid - cr * kChunks;
  const int gic = min(max(i0 - 4 + 4 * cc, 0), nx - 4);
  const bool x_lane = cr < kRY, b_lane = cr < kBYr;
  const int gjx = min(max(j0 - 2 + cr, 0), ny - 1), gjb = min(max(j0 - 1 + cr, 0), ny - 1);
  const float *__restrict__ gxs = v.x + (int64_t)gjx * v.sy + gic;
  const float *__restrict__ gbs = v.b + (int64_t)gjb * v.sy + gic;
  const int so = cr * kWX + 4 * cc;  // the chunk's offset in a staged plane (x and b rows alike)
  const int64_t sz = v.sz;
  // staged columns of the ghosts beyond the x walls, when inside this window
  const bool wl = i0 == 0;             // gi = -1 at column 3, wall column 4
  const int wr = nx - (i0 - 4);        // column of gi = nx
  const bool patch = wl || wr < kWX;
  // first-colour items (two at most per plane): offsets in a plane with the
  // colour bit lsb = 0, the colour bit at even k, and in-domain flags per bit
  constexpr int kRow = kQX / 2;      // 33 pairs per row
  constexpr int kOdd = kRow * kBYr;  // 330 per plane
  int ox[2], orr[2], par[2];
  bool ok0[2], ok1[2];
#pragma unroll
  for (int s = 0; s < 2; s++) {
    const int q = tid + 256 * s;
    const int lj = q / kRow, pi = q - lj * kRow;
    const int gj = j0 - 1 + lj, gi = i0 - 1 + 2 * pi;
    const bool row = q < kOdd && gj >= 0 && gj < ny;
    ox[s] = (lj + 1) * kWX + 2 * pi + 3;  // x_old column li + 3, row lj + 1 (b: row lj)
    orr[s] = lj * kQX + 2 * pi;
    par[s] = ((i0 + gj) & 1) ^ 1;
    ok0[s] = row && gi >= 0 && gi < nx;
    ok1[s] = row && gi + 1 >= 0 && gi + 1 < nx;
  }
  const bool has_b = tid + 256 < kOdd;
  // second-colour item: the cell pair (2 ep, 2 ep + 1) of tile row tj
  const int tj = tid >> 5, ep = tid & 31;
  const int gje = j0 + tj;
  const bool even_ok = gje < ny && i0 + 2 * ep < nx;
  const int epar = (i0 + gje + 1) & 1;         // its position in the pair at even planes
  const int oxe = (tj + 2) * kWX + 2 * ep + 4;  // x_old of the pair's first cell
  const int obe = (tj + 1) * kWX + 2 * ep + 4;  // b of the pair's first cell
  const int ore = (tj + 1) * kQX + 2 * ep + 1;  // new first-colour values around it
  float *__restrict__ gout = xnew + (int64_t)min(gje, ny - 1) * v.sy + i0 + 2 * ep;
  const float ex = v.ex, ey = v.ey, ez = v.ez, dg = v.diag, idg = v.inv_diag;

  int m5 = (k0 + 9) % 5;  // x_old slot of plane k0 - 1 (k0 - 1 >= -1)
  if (x_lane) {
    int s5 = m5 == 0 ? 4 : m5 - 1;  // slot of plane k0 - 2
#pragma unroll
    for (int kx = k0 - 2; kx <= k0; kx++) {
      cp_async16(xo + s5 * PX + so, gxs + (int64_t)min(max(kx, 0), nz - 1) * sz);
      s5 = s5 == 4 ? 0 : s5 + 1;
    }
  }
  if (b_lane && k0 >= 1) cp_async16(bs + ((k0 - 1) & 3) * PB + so, gbs + (int64_t)(k0 - 1) * sz);
  cp_async_commit();
  for (int k = k0 - 1; k <= k1; k++, m5 = m5 == 4 ? 0 : m5 + 1) {
    // x_old slots of planes k - 1, k, k + 1, k + 2 (m5 is plane k's)
    const int sm = m5 == 0 ? 4 : m5 - 1, sp = m5 == 4 ? 0 : m5 + 1;
    const int sn = sp == 4 ? 0 : sp + 1;
    // prefetch x_old(k + 2) and b(k + 1): completes during this plane's arithmetic
    if (x_lane && k + 2 <= k1 + 1)
      cp_async16(xo + sn * PX + so, gxs + (int64_t)min(k + 2, nz - 1) * sz);
    if (b_lane && k + 1 < nz) cp_async16(bs + ((k + 1) & 3) * PB + so, gbs + (int64_t)(k + 1) * sz);
    cp_async_commit();
    cp_async_wait<1>();  // all but the prefetch: x_old(k + 1), b(k) are in
    __syncthreads();
    const float *xk = xo + m5 * PX;
    const float *xkm = xo + sm * PX;
    const float *xkp = xo + sp * PX;
    if (patch) {  // ghost columns of plane k (read as x-neighbours below)
      if (tid < kRY) {
        float *row = xo + m5 * PX + tid * kWX;
        if (wl) row[3] = row[4];
        if (wr < kWX) row[wr] = row[wr - 1];
      }
      __syncthreads();
    }
    {
      const float *bk = bs + (k & 3) * PB;
      float *rq = xr + (k & 3) * PR;
      const bool kin = k >= 0 && k < nz;
      const int kp = k & 1;
#pragma unroll
      for (int s = 0; s < 2; s++) {
        if (s == 1 && !has_b) break;
        const int lsb = par[s] ^ kp;
        const int o = ox[s] + lsb;
        const float xc = xk[o];
        const float sx = xk[o - 1] + xk[o + 1];
        const float sy = xk[o - kWX] + xk[o + kWX];
        const float sz2 = xkm[o] + xkp[o];
        const float lap = sx * ex + sy * ey + sz2 * ez - dg * xc;
        const float relaxed = xc - (bk[o - kWX] - lap) * idg;
        const bool in = kin && (lsb ? ok1[s] : ok0[s]);
        rq[orr[s] + lsb] = in ? relaxed : xc;
      }
    }
    __syncthreads();
    // second-colour cells of plane k - 1 on the tile, both cells of the pair
    // stored as one 8-byte vector
    const int ke = k - 1;
    if (ke >= k0 && ke < k1 && even_ok) {
      const float *r0 = xr + (ke & 3) * PR;        // plane ke
      const float *rm = xr + ((ke + 3) & 3) * PR;  // plane ke - 1
      const float *rp = xr + (k & 3) * PR;         // plane ke + 1
      const float *be = bs + (ke & 3) * PB;
      const int e = epar ^ (ke & 1);
      const int o = ore + e;
      const float xc = xkm[oxe + e];  // x_old(ke) sits in plane k - 1's slot
      const float sx = r0[o - 1] + r0[o + 1];
      const float sy = r0[o - kQX] + r0[o + kQX];
      const float sz2 = rm[o] + rp[o];
      const float lap = sx * ex + sy * ey + sz2 * ez - dg * xc;
      const float even = xc - (be[obe + e] - lap) * idg;
      const float odd = r0[o + 1 - 2 * e];
      const float2 pair = e ? make_float2(odd, even) : make_float2(even, odd);
      *reinterpret_cast<float2 *>(gout + (int64_t)ke * sz) = pair;
    }
    // no barrier here: the next plane's copies go to slots no warp reads now,
    // and its first barrier orders everything else
  }
  cp_async_wait<0>();
}

// The same exact red-black sweep for levels whose rows are a multiple of 128
// cells and whose columns a multiple of 8 (the finest levels of the benchmark
// grids), with the work in registers instead of shared memory: a block owns a
// 128 x 8 tile of (i, j) columns and a chunk of planes; warp w < 10 handles
// row j0 - 1 + w (rows j0 - 1 and j0 + 8 are the first-colour ring), lane l
// the four cells i0 + 4l .. i0 + 4l + 3 of that row as one float4. Each such
// thread keeps its column's x_old at k - 1, k, k + 1 and the half-updated
// planes (first colour new, second colour old) at k - 2, k - 1, k in
// registers and takes its x-neighbours from the neighbouring lanes by
// shuffle; only the y-neighbours come from shared memory (x_old of plane k
// and the half-updated plane k - 1, double-buffered), so a plane needs one
// barrier. Warp 10 carries the ring columns i0 - 1 and i0 + 128 for the ten
// rows (lanes 0-9 and 16-25), so the row warps run no per-lane ring code.
// Planes walk with the same one-plane lag as k_rbgs_sweep (first colour at k,
// second colour at k - 1) and the same expressions, so the two kernels give
// the same bits; walls are the same mirrors (a neighbour outside the domain
// holds the wall cell's old value, in x_old and in the half-updated planes).
constexpr int kVX = 128, kVY = 8;
constexpr int kVRows = kVY + 2;        // rows j0 - 1 .. j0 + 8
constexpr int kVThreads = 32 * (kVRows + 1);
constexpr int kVRow = kVX + 8;         // staged row: columns i0 - 4 .. i0 + 131 (tile at 4)
constexpr int kVL = 3, kVR = kVX + 4;  // staged columns of the ring cells i0 - 1, i0 + 128

__global__ void __launch_bounds__(kVThreads, 2) k_rbgs_sweep_v(View<float> v,
    float *__restrict__ xnew, int kc, const MgState *st, int keep)
{
  const int nx = v.nx, ny = v.ny, nz = v.nz;
  const int i0 = blockIdx.x * kVX, j0 = blockIdx.y * kVY;
  const int k0 = blockIdx.z * kc, k1 = min(k0 + kc, nz);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sy = v.sy, sz = v.sz;
  if (mg_done(st)) {
    // a sweep skipped inside a V-cycle leaves x where the next kernels look
    // (see k_rbgs_sweep): copy the tile rows of the chunk
    if (keep && !solve_finished(st) && w >= 1 && w <= kVY) {
      const int c0 = (j0 + w - 1) * sy + i0 + 4 * lane;
      for (int k = k0; k < k1; k++)
        *reinterpret_cast<float4 *>(xnew + c0 + (int64_t)k * sz) =
            *reinterpret_cast<const float4 *>(v.x + c0 + (int64_t)k * sz);
    }
    return;
  }
  __shared__ __align__(16) float sx[2][kVY + 4][kVRow];  // x_old(k): rows j0 - 2 .. j0 + 9
  __shared__ __align__(16) float sr[2][kVRows][kVRow];   // half-updated plane: rows j0 - 1 .. j0 + 8
  const float ex = v.ex, ey = v.ey, ez = v.ez, dg = v.diag, idg = v.inv_diag;
  const auto plane = [&](int k) { return min(max(k, 0), nz - 1) * sz; };  // < 2^31

  if (w == kVRows) {
    // ---------------- ring columns: lane r < 10 left, 16 <= lane < 26 right ----------------
    const int r = lane & 15;
    const bool right = lane >= 16;
    const bool act = r < kVRows;
    const int j = j0 - 1 + r;
    const int jc = min(max(j, 0), ny - 1);
    const bool wall = right ? i0 + kVX == nx : i0 == 0;
    const int col = right ? i0 + kVX : i0 - 1;       // the ring cell
    const int beyond = right ? i0 + kVX + 1 : i0 - 2;
    const int edge = right ? i0 + kVX - 1 : i0;      // the tile's edge cell beside it
    const int scol = right ? kVR : kVL;
    const bool in = act && !wall && j >= 0 && j < ny && r >= 1 && r <= kVY;
    const float *__restrict__ xr = v.x + jc * sy;
    const float *__restrict__ br = v.b + jc * sy;
    // the ring cell's x_old at k - 1, k, k + 1 (the wall cell's own value outside the domain)
    const auto ld = [&](int k) { return act ? xr[plane(k) + (wall ? edge : col)] : 0.0f; };
    float hm = ld(k0 - 2), hc = ld(k0 - 1), hp = ld(k0);
    // b and the column beyond the ring cell, one plane ahead (ring cells in the domain)
    const auto ldb2 = [&](int k) {
      return in ? make_float2(br[plane(k) + col], xr[plane(k) + beyond]) : make_float2(0.f, 0.f);
    };
    float2 bb = ldb2(k0 - 1);
    for (int k = k0 - 1; k <= k1; k++) {
      const int s = k & 1;
      if (act) sx[s][r + 1][scol] = hc;
      const bool kin = k >= 0 && k < nz;
      const float hb = bb.x, hby = bb.y;
      const float hnext = ld(k + 2);
      const float2 bbnext = ldb2(k + 1);
      __syncthreads();
      if (act) {
        float hr = hc;
        const bool first = right ? ((j + k) & 1) == 0 : ((j + k) & 1) != 0;
        if (first && in && kin) {
          const float inner = sx[s][r + 1][right ? kVR - 1 : kVL + 1];  // the tile's edge cell
          const float sxs = right ? inner + hby : hby + inner;
          const float sys = sx[s][r][scol] + sx[s][r + 2][scol];
          const float szs = hm + hp;
          const float lap = sxs * ex + sys * ey + szs * ez - dg * hc;
          hr = hc - (hb - lap) * idg;
        }
        sr[s][r][scol] = hr;
      }
      hm = hc;
      hc = hp;
      hp = hnext;
      bb = bbnext;
    }
    return;
  }

  // ---------------- row warps ----------------
  const int j = j0 - 1 + w;
  const bool row_in = j >= 0 && j < ny;
  const bool tile_row = w >= 1 && w <= kVY;
  const int jc = min(max(j, 0), ny - 1);
  const float *__restrict__ xrow = v.x + jc * sy + i0 + 4 * lane;
  const float *__restrict__ brow = v.b + jc * sy + i0 + 4 * lane;
  float *__restrict__ orow = xnew + j * sy + i0 + 4 * lane;  // used for tile rows only
  // the extra staged rows j0 - 2 (warp 0) and j0 + 9 (warp 9), x_old only
  const bool extra = w == 0 || w == kVRows - 1;
  const int je = w == 0 ? j0 - 2 : j0 + 9;
  const float *__restrict__ xext = v.x + min(max(je, 0), ny - 1) * sy + i0 + 4 * lane;
  const int srow_ext = w == 0 ? 0 : kVY + 3;
  const auto ldx = [&](int k) { return *reinterpret_cast<const float4 *>(xrow + plane(k)); };
  const auto ldb = [&](int k) { return *reinterpret_cast<const float4 *>(brow + plane(k)); };
  const auto lde = [&](int k) { return *reinterpret_cast<const float4 *>(xext + plane(k)); };

  // x_old at k - 1, k, k + 1 (k + 2 and k + 3 in flight), b at k - 1, k (k + 1 and
  // k + 2 in flight), the half-updated planes at k - 2, k - 1, k
  float4 om = ldx(k0 - 2), oc = ldx(k0 - 1), op = ldx(k0), on = ldx(k0 + 1);
  float4 bm = make_float4(0.f, 0.f, 0.f, 0.f), bc = ldb(k0 - 1), bn = ldb(k0);
  float4 rm2 = oc, rm1 = oc, rc = oc;
  float4 ec = make_float4(0.f, 0.f, 0.f, 0.f);
  if (extra) ec = lde(k0 - 1);
  for (int k = k0 - 1; k <= k1; k++) {
    const int s = k & 1;
    const bool kin = k >= 0 && k < nz;
    *reinterpret_cast<float4 *>(&sx[s][w + 1][4 + 4 * lane]) = oc;
    if (extra) *reinterpret_cast<float4 *>(&sx[s][srow_ext][4 + 4 * lane]) = ec;
    // loads for the coming planes, issued before the barrier
    const float4 onext = ldx(k + 3);
    const float4 bnext = ldb(k + 2);
    float4 enext = ec;
    if (extra) enext = lde(k + 1);
    __syncthreads();
    // ---- first colour of plane k on this row: (i + j + k) even ----
    {
      float left = __shfl_up_sync(0xffffffffu, oc.w, 1);
      float right = __shfl_down_sync(0xffffffffu, oc.x, 1);
      if (lane == 0) left = sx[s][w + 1][kVL];
      if (lane == 31) right = sx[s][w + 1][kVR];
      const float4 yn = *reinterpret_cast<const float4 *>(&sx[s][w][4 + 4 * lane]);
      const float4 ys = *reinterpret_cast<const float4 *>(&sx[s][w + 2][4 + 4 * lane]);
      rc = oc;
      if (kin && row_in) {
        if (((j + k) & 1) == 0) {  // cells 0 and 2
          {
            const float sxs = left + oc.y, sys = yn.x + ys.x, szs = om.x + op.x;
            const float lap = sxs * ex + sys * ey + szs * ez - dg * oc.x;
            rc.x = oc.x - (bc.x - lap) * idg;
          }
          {
            const float sxs = oc.y + oc.w, sys = yn.z + ys.z, szs = om.z + op.z;
            const float lap = sxs * ex + sys * ey + szs * ez - dg * oc.z;
            rc.z = oc.z - (bc.z - lap) * idg;
          }
        } else {  // cells 1 and 3
          {
            const float sxs = oc.x + oc.z, sys = yn.y + ys.y, szs = om.y + op.y;
            const float lap = sxs * ex + sys * ey + szs * ez - dg * oc.y;
            rc.y = oc.y - (bc.y - lap) * idg;
          }
          {
            const float sxs = oc.z + right, sys = yn.w + ys.w, szs = om.w + op.w;
            const float lap = sxs * ex + sys * ey + szs * ez - dg * oc.w;
            rc.w = oc.w - (bc.w - lap) * idg;
          }
        }
      }
    }
    *reinterpret_cast<float4 *>(&sr[s][w][4 + 4 * lane]) = rc;
    // ---- second colour of plane k - 1 on the tile rows: (i + j + k - 1) odd ----
    const int ke = k - 1;
    if (ke >= k0 && ke < k1 && tile_row) {
      const int se = ke & 1;
      float left = __shfl_up_sync(0xffffffffu, rm1.w, 1);
      float right = __shfl_down_sync(0xffffffffu, rm1.x, 1);
      if (lane == 0) left = sr[se][w][kVL];
      if (lane == 31) right = sr[se][w][kVR];
      const float4 yn = *reinterpret_cast<const float4 *>(&sr[se][w - 1][4 + 4 * lane]);
      const float4 ys = *reinterpret_cast<const float4 *>(&sr[se][w + 1][4 + 4 * lane]);
      float4 out = rm1;
      if (((j + k) & 1) == 0) {  // second colour of plane k - 1: cells 0 and 2
        {
          const float sxs = left + rm1.y, sys = yn.x + ys.x, szs = rm2.x + rc.x;
          const float lap = sxs * ex + sys * ey + szs * ez - dg * rm1.x;
          out.x = rm1.x - (bm.x - lap) * idg;
        }
        {
          const float sxs = rm1.y + rm1.w, sys = yn.z + ys.z, szs = rm2.z + rc.z;
          const float lap = sxs * ex + sys * ey + szs * ez - dg * rm1.z;
          out.z = rm1.z - (bm.z - lap) * idg;
        }
      } else {
        {
          const float sxs = rm1.x + rm1.z, sys = yn.y + ys.y, szs = rm2.y + rc.y;
          const float lap = sxs * ex + sys * ey + szs * ez - dg * rm1.y;
          out.y = rm1.y - (bm.y - lap) * idg;
        }
        {
          const float sxs = rm1.z + right, sys = yn.w + ys.w, szs = rm2.w + rc.w;
          const float lap = sxs * ex + sys * ey + szs * ez - dg * rm1.w;
          out.w = rm1.w - (bm.w - lap) * idg;
        }
      }
      *reinterpret_cast<float4 *>(orow + (int64_t)ke * sz) = out;
    }
    // ---- rotate ----
    rm2 = rm1;
    rm1 = rc;
    om = oc;
    oc = op;
    op = on;
    on = onext;
    bm = bc;
    bc = bn;
    bn = bnext;
    ec = enext;
  }
}

// x_f += trilinear interpolation of x_c when x was coarsened (rx == 2): one
// thread per coarse x-position and fine (j, k) produces both x-children, so
// the three coarse values of each (y, z) line are loaded once for two cells.
// Same interpolation order as k_mg_prolong (x, then y, then z).
template <typename T>
__global__ void __launch_bounds__(kNT) k_mg_prolong_x2(View<T> f, const T *xc, int cnx, int cny,
    int cnz, int ry, int rz, const MgState *st)
{
  if (mg_done(st)) return;
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z * blockDim.z + threadIdx.z;
  if (I >= cnx || j >= f.ny || k >= f.nz) return;
  int Py, Qy, Pz, Qz;
  T wy, wz;
  if (ry == 2) {
    Py = j >> 1;
    const int nb = (j & 1) ? Py + 1 : Py - 1;
    Qy = (nb < 0 || nb >= cny) ? Py : nb;
    wy = (T)0.25;
  } else {
    Py = Qy = j;
    wy = (T)0;
  }
  if (rz == 2) {
    Pz = k >> 1;
    const int nb = (k & 1) ? Pz + 1 : Pz - 1;
    Qz = (nb < 0 || nb >= cnz) ? Pz : nb;
    wz = (T)0.25;
  } else {
    Pz = Qz = k;
    wz = (T)0;
  }
  const int Im = I > 0 ? I - 1 : I, Ip = I < cnx - 1 ? I + 1 : I;
  const int64_t sy = cnx, sz = (int64_t)cnx * cny;
  T lo[2][2], hi[2][2];
#pragma unroll
  for (int dz = 0; dz < 2; dz++)
#pragma unroll
    for (int dy = 0; dy < 2; dy++) {
      const int64_t base = (int64_t)(dz ? Qz : Pz) * sz + (int64_t)(dy ? Qy : Py) * sy;
      const T a0 = xc[base + I];
      lo[dz][dy] = a0 + (T)0.25 * (xc[base + Im] - a0);
      hi[dz][dy] = a0 + (T)0.25 * (xc[base + Ip] - a0);
    }
  const T ly0 = lo[0][0] + wy * (lo[0][1] - lo[0][0]), ly1 = lo[1][0] + wy * (lo[1][1] - lo[1][0]);
  const T hy0 = hi[0][0] + wy * (hi[0][1] - hi[0][0]), hy1 = hi[1][0] + wy * (hi[1][1] - hi[1][0]);
  const int64_t c = f.off + (int64_t)k * f.sz + (int64_t)j * f.sy + 2 * I;
  f.x[c] += ly0 + wz * (ly1 - ly0);
  f.x[c + 1] += hy0 + wz * (hy1 - hy0);
}

// Coarsest level: `sweeps` red-black Gauss-Seidel sweeps from zero by one
// block, the level held in shared memory (compact layout).
template <typename T>
__global__ void __launch_bounds__(512) k_mg_coarse(View<T> v, int sweeps, const MgState *st)
{
  if (mg_done(st)) return;
  extern __shared__ unsigned char smem_raw[];
  T *xs = reinterpret_cast<T *>(smem_raw);
  T *bs = xs + (int64_t)v.nx * v.ny * v.nz;
  const int n = v.nx * v.ny * v.nz;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    xs[q] = 0;
    bs[q] = v.b[q];
  }
  __syncthreads();
  View<T> s = v;
  s.x = xs;
  s.sy = v.nx;
  s.sz = v.nx * v.ny;
  s.off = 0;
  for (int it = 0; it < sweeps; it++) {
    for (int colour = 1; colour >= 0; colour--) {
      for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int i = q % v.nx, j = (q / v.nx) % v.ny, k = q / (v.nx * v.ny);
        if (((i + j + k + 3) & 1) != colour) continue;
        const T xc = xs[q];
        const T r = bs[q] - lap_at(s, xs, i, j, k, q, xc);
        xs[q] = xc - r * s.inv_diag;
      }
      __syncthreads();
    }
  }
  for (int q = threadIdx.x; q < n; q += blockDim.x) v.x[q] = xs[q];
}

// Coarsest level, exact: x = Minv * b with Minv the inverse of the coarsest
// operator deflated by its null space (see coarse_inverse); one warp per row,
// b staged in shared memory.
template <typename T>
__global__ void __launch_bounds__(128) k_mg_direct(const T *__restrict__ minv,
    const T *__restrict__ b, T *__restrict__ x, int n, const MgState *st)
{
  if (mg_done(st)) return;
  extern __shared__ unsigned char smem_raw[];
  T *bs = reinterpret_cast<T *>(smem_raw);
  for (int q = threadIdx.x; q < n; q += blockDim.x) bs[q] = b[q];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (row >= n) return;
  const T *m = minv + (int64_t)row * n;
  T acc = 0;
  for (int q = lane; q < n; q += 32) acc += m[q] * bs[q];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) x[row] = acc;
}

// The coarse end of a V-cycle in one kernel: one block of 1024 threads
// smooths, restricts, solves the coarsest level and prolongates through every
// level from `lv[0]` down (the small levels, where a launch per step costs
// more than the work), with __syncthreads between the steps. Same operations
// and colour order as the per-level kernels: red-black Gauss-Seidel (first the
// cells with (i + j + k) even), residual restriction, exact coarsest solve
// (or sweeps), trilinear prolongation.
template <typename T>
struct TailLevel {
  int n[3];
  int r[3];  // coarsening ratio from the level above
  T ex, ey, ez, diag, inv_diag;
  T *x, *b;
};

template <typename T>
struct TailArgs {
  int count;  // levels in the tail (the last one is the coarsest)
  TailLevel<T> lv[kMaxLevels];
  const T *minv;  // exact coarsest solve, or null (coarse_sweeps sweeps)
  int pre, post, coarse_sweeps, zero_top;
  const MgState *st;
};

template <typename T>
__device__ __forceinline__ View<T> tail_view(const TailLevel<T> &L)
{
  View<T> v;
  v.x = L.x;
  v.b = L.b;
  v.nx = L.n[0];
  v.ny = L.n[1];
  v.nz = L.n[2];
  v.sy = L.n[0];
  v.sz = L.n[0] * L.n[1];
  v.off = 0;
  v.ex = L.ex;
  v.ey = L.ey;
  v.ez = L.ez;
  v.diag = L.diag;
  v.inv_diag = L.inv_diag;
  return v;
}

template <typename T>
__device__ void tail_smooth(const View<T> &v, int count, bool zero_first)
{
  const int n = v.nx * v.ny * v.nz;
  if (count == 0 && zero_first) {
    for (int q = threadIdx.x; q < n; q += blockDim.x) v.x[q] = (T)0;
    __syncthreads();
    return;
  }
  for (int s = 0; s < count; s++) {
    const bool z = zero_first && s == 0;
    for (int colour = 1; colour >= 0; colour--) {  // colour 1: (i + j + k) even
      for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int i = q % v.nx, j = (q / v.nx) % v.ny, k = q / (v.nx * v.ny);
        if (((i + j + k + 1) & 1) != colour) continue;
        if (z && colour == 1) {
          v.x[q] = -v.b[q] * v.inv_diag;
        } else {
          const T xc = z ? (T)0 : v.x[q];
          const T r = v.b[q] - lap_at(v, v.x, i, j, k, q, xc);
          v.x[q] = xc - r * v.inv_diag;
        }
      }
      __syncthreads();
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(1024) k_mg_tail(TailArgs<T> a)
{
  if (mg_done(a.st)) return;
  const int m = a.count;
  for (int l = 0; l < m - 1; l++) {
    const View<T> v = tail_view(a.lv[l]);
    tail_smooth(v, a.pre, l > 0 || a.zero_top);
    // residual restriction into the next level's right-hand side
    const TailLevel<T> &C = a.lv[l + 1];
    const int rx = C.r[0], ry = C.r[1], rz = C.r[2];
    const T inv = (T)(1.0 / (rx * ry * rz));
    const int nc = C.n[0] * C.n[1] * C.n[2];
    for (int q = threadIdx.x; q < nc; q += blockDim.x) {
      const int I = q % C.n[0], J = (q / C.n[0]) % C.n[1], K = q / (C.n[0] * C.n[1]);
      T sum = 0;
      for (int dk = 0; dk < rz; dk++)
        for (int dj = 0; dj < ry; dj++)
          for (int di = 0; di < rx; di++) {
            const int i = I * rx + di, j = J * ry + dj, k = K * rz + dk;
            const int c = (k * v.ny + j) * v.nx + i;
            sum += v.b[c] - lap_at(v, v.x, i, j, k, c, v.x[c]);
          }
      C.b[q] = sum * inv;
    }
    __syncthreads();
  }
  // coarsest level
  {
    const View<T> v = tail_view(a.lv[m - 1]);
    const int n = v.nx * v.ny * v.nz;
    if (a.minv) {
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
      for (int row = warp; row < n; row += nw) {
        const T *mrow = a.minv + (int64_t)row * n;
        T acc = 0;
        for (int q = lane; q < n; q += 32) acc += mrow[q] * v.b[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) v.x[row] = acc;
      }
      __syncthreads();
    } else {
      tail_smooth(v, a.coarse_sweeps, true);
    }
  }
  for (int l = m - 2; l >= 0; l--) {
    const View<T> f = tail_view(a.lv[l]);
    const TailLevel<T> &C = a.lv[l + 1];
    const int cn[3] = { C.n[0], C.n[1], C.n[2] };
    const int n = f.nx * f.ny * f.nz;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
      const int fi[3] = { q % f.nx, (q / f.nx) % f.ny, q / (f.nx * f.ny) };
      int P[3], Q[3];
      T w[3];
#pragma unroll
      for (int ax = 0; ax < 3; ax++) {
        if (C.r[ax] == 2) {
          P[ax] = fi[ax] >> 1;
          const int nb = (fi[ax] & 1) ? P[ax] + 1 : P[ax] - 1;
          Q[ax] = (nb < 0 || nb >= cn[ax]) ? P[ax] : nb;
          w[ax] = (T)0.25;
        } else {
          P[ax] = Q[ax] = fi[ax];
          w[ax] = (T)0;
        }
      }
      const int sy = cn[0], sz = cn[0] * cn[1];
      T vv[2][2];
#pragma unroll
      for (int dz = 0; dz < 2; dz++)
#pragma unroll
        for (int dy = 0; dy < 2; dy++) {
          const int base = (dz ? Q[2] : P[2]) * sz + (dy ? Q[1] : P[1]) * sy;
          const T a0 = C.x[base + P[0]], a1 = C.x[base + Q[0]];
          vv[dz][dy] = a0 + w[0] * (a1 - a0);
        }
      const T y0 = vv[0][0] + w[1] * (vv[0][1] - vv[0][0]);
      const T y1 = vv[1][0] + w[1] * (vv[1][1] - vv[1][0]);
      f.x[q] += y0 + w[2] * (y1 - y0);
    }
    __syncthreads();
    tail_smooth(f, a.post, false);
  }
}

// the solve state for a right-hand side whose ||b - shift||^2 is nb2
__device__ void open_solve(MgState *st, double nb2)
{
  st->nb2 = nb2;
  st->tol2 = st->rtol2 * nb2;
  st->tol_inner = st->theta2 * st->rtol2 * nb2;
  st->res2 = 0.0;
  st->res2_inner = 0.0;
  st->cycles = 0;
  st->outer = 0;
  st->inner_done = 0;
  st->loops = 0;
  st->done = (nb2 == 0.0);
}

// One pass over the right-hand side: its sum and sum of squares, folded by the
// last block into the mean (the shift) and ||b - shift||^2 = sum b^2 -
// shift * sum b; initialises the solve state. The subtraction keeps its digits
// while the mean is small against the spread (a compatible Neumann right-hand
// side has mean ~0); when shift * sum b exceeds half of sum b^2 it raises
// need_norm instead, and k_mg_rhs_norm computes the norm about the mean in a
// second pass.
// DF: the per-thread sums of b and b^2 as double-float pairs (df32.cuh) on the
// FP32 pipe instead of two FP64 instructions per cell; the block and grid folds
// stay in FP64.
template <bool DF>
__global__ void __launch_bounds__(kNT) k_mg_rhs_stats(View<double> f, MgState *st,
    double *partials, double *partials2, unsigned *ticket)
{
  const int64_t n = (int64_t)f.nx * f.ny * f.nz;
  double acc = 0.0, acc2 = 0.0;
  df::f2 s1{ 0.0f, 0.0f }, s2{ 0.0f, 0.0f };
  const int64_t q0 = blockIdx.x * (int64_t)kNT + threadIdx.x, stride = (int64_t)gridDim.x * kNT;
  FlatWalk w(q0, stride, f.nx, f.ny);
  for (int64_t q = q0; q < n; q += stride, w.advance(f.nx, f.ny)) {
    const double b = f.b[f.off + (int64_t)w.k * f.sz + (int64_t)w.j * f.sy + w.i];
    if constexpr (DF) {
      const df::f2 bp = df::split(b);
      s1 = df::add(s1, bp);
      s2 = df::add(s2, df::mul_u(bp, bp));
    } else {
      acc += b;
      acc2 = fma(b, b, acc2);
    }
  }
  if constexpr (DF) {
    acc = df::to_double(s1);
    acc2 = df::to_double(s2);
  }
  __shared__ double sm[kNT / 32];
  acc = block_reduce_sum<kNT>(acc, sm);
  acc2 = block_reduce_sum<kNT>(acc2, sm);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = acc;
    partials2[blockIdx.x] = acc2;
    last = ticket_is_last(ticket);
  }
  __syncthreads();
  if (!last) return;
  const double total = fold_partials<kNT>(partials, gridDim.x, sm);
  const double total2 = fold_partials<kNT>(partials2, gridDim.x, sm);
  if (threadIdx.x == 0) {
    const double shift = total / (double)n;
    st->shift = shift;
    const double mean_part = shift * total;  // n shift^2
    st->need_norm = mean_part > 0.5 * total2;
    if (!st->need_norm) open_solve(st, fmax(total2 - mean_part, 0.0));
    *ticket = 0;
  }
}

// ||b - shift||^2 in a second pass, when k_mg_rhs_stats did not trust its
// one-pass value (returns at once otherwise)
__global__ void __launch_bounds__(kNT) k_mg_rhs_norm(View<double> f, MgState *st,
    double *partials, unsigned *ticket)
{
  if (!*reinterpret_cast<const volatile int *>(&st->need_norm)) return;
  const int64_t n = (int64_t)f.nx * f.ny * f.nz;
  const double sh = st->shift;
  double acc = 0.0;
  const int64_t q0 = blockIdx.x * (int64_t)kNT + threadIdx.x, stride = (int64_t)gridDim.x * kNT;
  FlatWalk w(q0, stride, f.nx, f.ny);
  for (int64_t q = q0; q < n; q += stride, w.advance(f.nx, f.ny)) {
    const double b = f.b[f.off + (int64_t)w.k * f.sz + (int64_t)w.j * f.sy + w.i] - sh;
    acc += b * b;
  }
  __shared__ double sm[kNT / 32];
  acc = block_reduce_sum<kNT>(acc, sm);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = acc;
    last = ticket_is_last(ticket);
  }
  __syncthreads();
  if (!last) return;
  const double total = fold_partials<kNT>(partials, gridDim.x, sm);
  if (threadIdx.x == 0) {
    open_solve(st, total);
    st->need_norm = 0;
    *ticket = 0;
  }
}

// ---------------------------------------------------------------- host side

int sm_count_mg()
{
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 152;
  }
  return n;
}

int build_levels(const Grid *gr, int cap, MgLevelDesc *lv)
{
  double h[3] = { gr->dx, gr->dy, gr->dz };
  lv[0].n[0] = gr->imax;
  lv[0].n[1] = gr->jmax;
  lv[0].n[2] = gr->kmax;
  for (int a = 0; a < 3; a++) {
    lv[0].r[a] = 1;
    lv[0].ih2[a] = 1.0 / (h[a] * h[a]);
  }
  int nl = 1;
  while (nl < kMaxLevels && (cap <= 0 || nl < cap)) {
    MgLevelDesc &f = lv[nl - 1], &c = lv[nl];
    bool any = false;
    for (int a = 0; a < 3; a++) {
      if (f.n[a] % 2 == 0 && f.n[a] >= 16) {
        c.n[a] = f.n[a] / 2;
        c.r[a] = 2;
        h[a] *= 2.0;
        any = true;
      } else {
        c.n[a] = f.n[a];
        c.r[a] = 1;
      }
      c.ih2[a] = 1.0 / (h[a] * h[a]);
    }
    if (!any) break;
    nl++;
  }
  return nl;
}

// Inverse of the coarsest operator with its null space deflated:
// M = A - (s/n) 1 1^T, A the ghost-free Neumann Laplacian of level L, s its
// largest diagonal magnitude. -M is symmetric positive definite; for a
// mean-free b, x = M^-1 b solves A x = b with mean(x) = 0 (a b with a small
// mean gives the solution for b minus its mean). Cholesky of -M, then the
// n unit right-hand sides; row-major n x n result. Returns false if the
// factorisation fails.
bool coarse_inverse(const MgLevelDesc &L, std::vector<double> &minv)
{
  const int nx = L.n[0], ny = L.n[1], nz = L.n[2];
  const int n = nx * ny * nz;
  const double s = 2.0 * (L.ih2[0] + L.ih2[1] + L.ih2[2]);
  std::vector<double> a((size_t)n * n, s / n);  // this is -M: -A + (s/n) 1 1^T
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const int q = i + nx * (j + ny * k);
        const int idx[3] = { i, j, k }, n3[3] = { nx, ny, nz }, st[3] = { 1, nx, nx * ny };
        for (int ax = 0; ax < 3; ax++)
          for (int sgn = -1; sgn <= 1; sgn += 2) {
            const int c = idx[ax] + sgn;
            if (c < 0 || c >= n3[ax]) continue;
            a[(size_t)q * n + q] += L.ih2[ax];
            a[(size_t)q * n + q + sgn * st[ax]] -= L.ih2[ax];
          }
      }
  // Cholesky in place (lower triangle)
  for (int c = 0; c < n; c++) {
    double d = a[(size_t)c * n + c];
    for (int q = 0; q < c; q++) d -= a[(size_t)c * n + q] * a[(size_t)c * n + q];
    if (!(d > 0.0)) return false;
    d = std::sqrt(d);
    a[(size_t)c * n + c] = d;
    for (int r = c + 1; r < n; r++) {
      double v = a[(size_t)r * n + c];
      for (int q = 0; q < c; q++) v -= a[(size_t)r * n + q] * a[(size_t)c * n + q];
      a[(size_t)r * n + c] = v / d;
    }
  }
  minv.assign((size_t)n * n, 0.0);
  std::vector<double> y(n);
  for (int col = 0; col < n; col++) {
    for (int r = 0; r < n; r++) {  // L y = e_col
      double v = (r == col) ? 1.0 : 0.0;
      for (int q = 0; q < r; q++) v -= a[(size_t)r * n + q] * y[q];
      y[r] = v / a[(size_t)r * n + r];
    }
    for (int r = n - 1; r >= 0; r--) {  // L^T z = y
      double v = y[r];
      for (int q = r + 1; q < n; q++) v -= a[(size_t)q * n + r] * y[q];
      y[r] = v / a[(size_t)r * n + r];
    }
    for (int r = 0; r < n; r++) minv[(size_t)r * n + col] = -y[r];  // M^-1 = -(-M)^-1
  }
  return true;
}

template <typename T>
View<T> compact_view(const MgLevelDesc &L, T *x, const T *b)
{
  View<T> v;
  v.x = x;
  v.b = b;
  v.nx = L.n[0];
  v.ny = L.n[1];
  v.nz = L.n[2];
  v.sy = L.n[0];
  v.sz = L.n[0] * L.n[1];
  v.off = 0;
  const double d = 2.0 * (L.ih2[0] + L.ih2[1] + L.ih2[2]);
  v.ex = (T)L.ih2[0];
  v.ey = (T)L.ih2[1];
  v.ez = (T)L.ih2[2];
  v.diag = (T)d;
  v.inv_diag = (T)(L.relax / d);
  return v;
}

View<double> padded_view(const MgLevelDesc &L, double *x, const double *b)
{
  View<double> v = compact_view<double>(L, x, b);
  v.sy = L.n[0] + 2;
  v.sz = (L.n[0] + 2) * (L.n[1] + 2);
  v.off = 1 + v.sy + v.sz;
  return v;
}

int planes_per_block(int nx, int ny, int nz)
{
  const int gx = ((nx + 1) / 2 + kBX - 1) / kBX, gy = (ny + kBY - 1) / kBY;
  int kb = 16;
  while (kb > 1 && (int64_t)gx * gy * ((nz + kb - 1) / kb) < 4 * sm_count_mg()) kb >>= 1;
  return kb;
}

template <typename T, bool ZERO>
bool smooth_pass(const View<T> &v, int colour, const double *shift, const MgState *st)
{
  const int kb = planes_per_block(v.nx, v.ny, v.nz);
  dim3 grid(((v.nx + 1) / 2 + kBX - 1) / kBX, (v.ny + kBY - 1) / kBY, (v.nz + kb - 1) / kb);
  if constexpr (sizeof(T) == sizeof(float)) {
    // paired loads need every row to start on an even cell (compact, even nx)
    if (v.off == 0 && v.nx % 2 == 0 && shift == nullptr) {
      k_mg_smooth_f2<ZERO><<<grid, dim3(kBX, kBY), 0, stream()>>>(v, colour, kb, st);
      return launched("k_mg_smooth_f2");
    }
  }
  k_mg_smooth<T, ZERO><<<grid, dim3(kBX, kBY), 0, stream()>>>(v, colour, shift, kb, st);
  return launched("k_mg_smooth");
}

// `count` sweeps (odd colour, then even); the first from zero when zero_first
template <typename T>
bool sweeps(const View<T> &v, int count, bool zero_first, const double *shift,
    const MgState *st)
{
  for (int s = 0; s < count; s++) {
    const bool z = zero_first && s == 0;
    bool ok = z ? smooth_pass<T, true>(v, 1, shift, st) : smooth_pass<T, false>(v, 1, shift, st);
    if (!ok) return false;
    ok = z ? smooth_pass<T, true>(v, 0, shift, st) : smooth_pass<T, false>(v, 0, shift, st);
    if (!ok) return false;
  }
  return true;
}

int flat_blocks(int64_t n)
{
  int64_t b = (n + kNT - 1) / kNT;
  const int64_t cap = 8 * (int64_t)sm_count_mg();
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

// grid of k_mx_residual_df: 32 x 8 column tiles, the planes split into
// chunks of kb; kb minimises (waves of resident blocks) x (kb + 2 planes read
// per chunk), four blocks of the kernel being resident per SM (the kernel's
// partials fit mx_df_blocks)
dim3 mx_df_grid(int nx, int ny, int nz, int *kb)
{
  const int64_t gx = (nx + kBX - 1) / kBX, gy = (ny + kBY - 1) / kBY;
  const int64_t wave = 4 * (int64_t)sm_count_mg();
  int best = nz;
  int64_t best_cost = INT64_MAX;
  for (int c = 4; c <= 64; c++) {
    const int64_t blocks = gx * gy * ((nz + c - 1) / c);
    const int64_t cost = ((blocks + wave - 1) / wave) * (c + 2);
    if (cost < best_cost) {
      best_cost = cost;
      best = c;
    }
  }
  *kb = std::min(best, nz);
  return dim3((unsigned)gx, (unsigned)gy, (unsigned)((nz + *kb - 1) / *kb));
}

int mx_df_blocks(int nx, int ny, int nz)
{
  int kb;
  const dim3 g = mx_df_grid(nx, ny, nz, &kb);
  return (int)(g.x * g.y * g.z);
}

// the FP64 residual of mg-mixed (count_cycles, e_zero: see k_mx_residual)
bool mx_residual(MgHierarchy *H, const View<double> &v0, MgState *st, int count_cycles,
    float *e_zero)
{
  if (H->mx_df) {
    int kb;
    const dim3 grid = mx_df_grid(v0.nx, v0.ny, v0.nz, &kb);
    const DfStencil cs{ df::from_double_rn(v0.ex), df::from_double_rn(v0.ey),
                        df::from_double_rn(v0.ez), df::from_double_rn(-v0.diag) };
    k_mx_residual_df<<<grid, dim3(kBX, kBY), 0, stream()>>>(v0, cs, H->b32[0], st,
        H->red.partials, H->red.ticket, count_cycles, e_zero, kb);
    return launched("k_mx_residual_df");
  }
  const int64_t n0 = (int64_t)v0.nx * v0.ny * v0.nz;
  k_mx_residual<<<flat_blocks(n0), kNT, 0, stream()>>>(v0, H->b32[0], st, H->red.partials,
      H->red.ticket, count_cycles, e_zero);
  return launched("k_mx_residual");
}

template <typename T, int FOLD>
bool restrict_to(const View<T> &f, T *bc, const MgLevelDesc &C, const double *shift, MgState *st,
    ReduceScratch &red)
{
  const int64_t nc = (int64_t)C.n[0] * C.n[1] * C.n[2];
  const int blocks = flat_blocks(nc);
  if (FOLD != FOLD_NONE && red.capacity < blocks) {
    fail(NUSIF_ERR_STATE, "multigrid reduction scratch too small");
    return false;
  }
  const T inv = (T)(1.0 / (C.r[0] * C.r[1] * C.r[2]));
  // 3-D grid; planes strided so that the blocks fit the reduction scratch
  const int gx = (C.n[0] + 31) / 32, gy = (C.n[1] + 7) / 8;
  const int cap = FOLD != FOLD_NONE ? red.capacity : 8 * sm_count_mg();
  if constexpr (sizeof(T) == sizeof(float)) {
    if (!shift && C.r[0] == 2 && C.r[1] == 2 && C.r[2] == 2 && f.off % 2 == 0 && f.sy % 2 == 0 &&
        f.sz % 2 == 0 && (int64_t)gx * gy <= cap) {
      int gz = (int)std::min<int64_t>(C.n[2], cap / ((int64_t)gx * gy));
      const int kcz = (C.n[2] + gz - 1) / gz;
      gz = (C.n[2] + kcz - 1) / kcz;
      k_mg_restrict_f32<FOLD><<<dim3(gx, gy, gz), dim3(32, 8), 0, stream()>>>(f, bc, C.n[0],
          C.n[1], C.n[2], kcz, inv, st, red.partials, red.ticket);
      return launched("k_mg_restrict_f32");
    }
  }
  if (C.r[0] == 2 && (int64_t)gx * gy <= cap) {
    int gz = C.n[2];
    while (gz > 1 && (int64_t)gx * gy * gz > cap) gz = (gz + 1) / 2;
    k_mg_restrict_x2<T, FOLD><<<dim3(gx, gy, gz), dim3(32, 8), 0, stream()>>>(f, bc, C.n[0],
        C.n[1], C.n[2], C.r[1], C.r[2], inv, shift, st, red.partials, red.ticket);
    return launched("k_mg_restrict_x2");
  }
  k_mg_restrict<T, FOLD><<<blocks, kNT, 0, stream()>>>(f, bc, C.n[0], C.n[1], C.n[2], C.r[0],
      C.r[1], C.r[2], inv, shift, st, red.partials, red.ticket);
  return launched("k_mg_restrict");
}

template <typename T>
bool prolong_to(const View<T> &f, const T *xc, const MgLevelDesc &C, const MgState *st)
{
  if constexpr (sizeof(T) == sizeof(float)) {
    if (C.r[0] == 2 && C.r[1] == 2 && C.r[2] == 2 && f.nx % 4 == 0 && f.off % 4 == 0 &&
        f.sy % 4 == 0 && f.sz % 4 == 0) {
      const int gx = (f.nx / 4 + 31) / 32, gy = (f.ny + 7) / 8;
      int gz = C.n[2];
      while (gz > 1 && (int64_t)gx * gy * gz > 8 * sm_count_mg()) gz = (gz + 1) / 2;
      const int kcz = (C.n[2] + gz - 1) / gz;
      gz = (C.n[2] + kcz - 1) / kcz;
      k_mg_prolong_f32<<<dim3(gx, gy, gz), dim3(32, 8), 0, stream()>>>(f, xc, C.n[0], C.n[1],
          C.n[2], kcz, st);
      return launched("k_mg_prolong_f32");
    }
  }
  if (C.r[0] == 2 && f.nx % 4 == 0) {
    const dim3 blk(32, 8, 1);
    const int gx = (f.nx / 4 + 31) / 32, gy = (f.ny + 7) / 8;
    int gz = f.nz;
    while (gz > 1 && (int64_t)gx * gy * gz > 8 * sm_count_mg()) gz = (gz + 1) / 2;
    const dim3 grid(gx, gy, gz);
    const bool vec = sizeof(T) == 4 && f.off % 4 == 0 && f.sy % 4 == 0 && f.sz % 4 == 0;
    if (vec)
      k_mg_prolong_x4<T, true><<<grid, blk, 0, stream()>>>(f, xc, C.n[0], C.n[1], C.n[2], C.r[1],
          C.r[2], st);
    else
      k_mg_prolong_x4<T, false><<<grid, blk, 0, stream()>>>(f, xc, C.n[0], C.n[1], C.n[2],
          C.r[1], C.r[2], st);
    return launched("k_mg_prolong_x4");
  }
  if (C.r[0] == 2) {
    const dim3 blk(32, 4, 2);
    const dim3 grid((C.n[0] + 31) / 32, (f.ny + 3) / 4, (f.nz + 1) / 2);
    k_mg_prolong_x2<T><<<grid, blk, 0, stream()>>>(f, xc, C.n[0], C.n[1], C.n[2], C.r[1], C.r[2],
        st);
    return launched("k_mg_prolong_x2");
  }
  const int64_t nf = (int64_t)f.nx * f.ny * f.nz;
  k_mg_prolong<T><<<flat_blocks(nf), kNT, 0, stream()>>>(f, xc, C.n[0], C.n[1], C.n[2], C.r[0],
      C.r[1], C.r[2], st);
  return launched("k_mg_prolong");
}

template <typename T>
bool coarse_solve(const View<T> &v, int nsweeps, const MgState *st, const T *minv)
{
  const size_t n = (size_t)v.nx * v.ny * v.nz;
  if (minv) {
    k_mg_direct<T><<<(int)((n + 3) / 4), 128, n * sizeof(T), stream()>>>(minv, v.b, v.x, (int)n,
        st);
    return launched("k_mg_direct");
  }
  const size_t bytes = 2 * n * sizeof(T);
  if (bytes <= 48 * 1024) {
    k_mg_coarse<T><<<1, 512, bytes, stream()>>>(v, nsweeps, st);
    return launched("k_mg_coarse");
  }
  // larger coarsest grids: sweeps in global memory
  if (nsweeps == 0) {
    k_zero<T><<<flat_blocks((int64_t)n), kNT, 0, stream()>>>(v.x, (int64_t)n);
    return launched("k_zero");
  }
  return sweeps<T>(v, nsweeps, true, nullptr, st);
}

// V-cycle from level l on the compact arrays xs/bs of type T. x_l starts at
// zero when `zero` (always below the top level); `inner_test`: the fine
// restriction folds the residual norm for the mixed-precision inner stop.
// `count` whole red-black sweeps of an FP32 level with the one-kernel sweep;
// each swaps the level's current and ping-pong buffers (x32[l] stays current)
// Planes per block (chunk depth) of the one-kernel sweep. A block walks
// kc + 2 planes (the first-colour planes just outside its chunk are
// recomputed) and the grid runs in ceil(blocks / resident) waves; the rule
// minimises waves * (kc + 2). The chunk depth changes only how the work is
// split: every cell is computed the same way, so results do not depend on it.
// The one-kernel FP32 sweep of a level: k_rbgs_sweep_v where the rows are a
// multiple of 128 cells and the columns of 8 (the environment variable
// NUSIF_SWEEP=tile64 selects k_rbgs_sweep everywhere, for comparisons), else
// k_rbgs_sweep.
struct SweepShape {
  bool vec;
  int gx, gy, threads;
};

SweepShape sweep_shape(const MgLevelDesc &L)
{
  const char *e = getenv("NUSIF_SWEEP");
  const bool legacy = e && strcmp(e, "tile64") == 0;
  SweepShape r;
  r.vec = !legacy && L.n[0] % kVX == 0 && L.n[1] % kVY == 0;
  if (r.vec) {
    r.gx = L.n[0] / kVX;
    r.gy = L.n[1] / kVY;
    r.threads = kVThreads;
  } else {
    r.gx = (L.n[0] + kSX - 1) / kSX;
    r.gy = (L.n[1] + kSY - 1) / kSY;
    r.threads = 256;
  }
  return r;
}

void launch_rbgs(const SweepShape &sh, const View<float> &v, float *xb, int kc, const MgState *st,
    int keep)
{
  const dim3 grid(sh.gx, sh.gy, (v.nz + kc - 1) / kc);
  if (sh.vec)
    k_rbgs_sweep_v<<<grid, kVThreads, 0, stream()>>>(v, xb, kc, st, keep);
  else
    k_rbgs_sweep<<<grid, 256, 0, stream()>>>(v, xb, kc, st, keep);
}

int sweep_chunk_rule(const MgLevelDesc &L)
{
  const SweepShape sh = sweep_shape(L);
  static int resident[2] = { 0, 0 };
  int &res = resident[sh.vec ? 1 : 0];
  if (res == 0) {
    int per_sm = 0;
    if (sh.vec)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rbgs_sweep_v, kVThreads, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rbgs_sweep, 256, 0);
    res = (per_sm > 0 ? per_sm : 1) * sm_count_mg();
  }
  const int resident_blocks = res;
  const int gx = sh.gx, gy = sh.gy, nz = L.n[2];
  int kc = nz;
  int64_t best = -1;
  for (int c = 1; c <= nz; c++) {
    const int64_t blocks = (int64_t)gx * gy * ((nz + c - 1) / c);
    const int64_t cost = ((blocks + resident_blocks - 1) / resident_blocks) * (int64_t)(c + 2);
    if (best < 0 || cost < best) {
      best = cost;
      kc = c;
    }
  }
  return kc;
}

// Autotuner: the chunk depth of the one-kernel sweep measured on a level's own
// arrays (x, b read; xb written), once per level size (cached): the fastest
// of a few depths over three timed sweeps each, the rule's depth among them.
int sweep_chunk_tuned(const MgLevelDesc &L, float *x, float *xb, float *b)
{
  int dev = 0;
  cudaGetDevice(&dev);
  const SweepShape sh = sweep_shape(L);
  // (device, nx, ny, nz, kernel) -> planes per block
  static std::map<std::array<int, 5>, int> cache;
  const std::array<int, 5> key = { dev, L.n[0], L.n[1], L.n[2], sh.vec ? 1 : 0 };
  const auto hit = cache.find(key);
  if (hit != cache.end()) return hit->second;
  const int rule = sweep_chunk_rule(L);
  static std::map<int, MgState *> idle_state;  // per device: done = inner_done = 0
  MgState *&idle = idle_state[dev];
  if (!idle) {
    MgState *fresh = nullptr;
    if (cudaMalloc(&fresh, sizeof(MgState)) != cudaSuccess) {
      cudaGetLastError();
      return rule;
    }
    if (cudaMemset(fresh, 0, sizeof(MgState)) != cudaSuccess) {
      cudaFree(fresh);
      cudaGetLastError();
      return rule;
    }
    idle = fresh;
  }
  const int nz = L.n[2];
  const View<float> v = compact_view<float>(L, x, b);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    cudaGetLastError();
    return rule;
  }
  int kc = rule;
  float best = -1.0f;
  const int cand[] = { rule, 1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64 };
  for (const int c : cand) {
    if (c > nz) continue;
    launch_rbgs(sh, v, xb, c, idle, 0);  // warm-up
    cudaEventRecord(e0, stream());
    for (int r = 0; r < 3; r++) launch_rbgs(sh, v, xb, c, idle, 0);
    cudaEventRecord(e1, stream());
    float ms = 0.0f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      break;
    if (best < 0 || ms < best) {
      best = ms;
      kc = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess) return rule;
  cache[key] = kc;
  return kc;
}

bool fused_sweeps(MgHierarchy *H, int l, int count, bool zero_first, const MgState *st)
{
  const MgLevelDesc &L = H->lv[l];
  if (L.n[0] % 4 != 0) {  // rows not 16-byte aligned: the two-pass in-place sweep
    const View<float> v = compact_view<float>(L, H->x32[l], H->b32[l]);
    return sweeps<float>(v, count, zero_first, nullptr, st);
  }
  const SweepShape sh = sweep_shape(L);
  const int kc = H->kc[l] > 0 ? H->kc[l] : sweep_chunk_rule(L);
  for (int s = 0; s < count; s++) {
    const View<float> v = compact_view<float>(L, H->x32[l], H->b32[l]);
    if (zero_first && s == 0) {
      const int zx = (L.n[0] / 4 + 31) / 32, zy = (L.n[1] + 7) / 8;
      int zz = L.n[2];
      while (zz > 1 && (int64_t)zx * zy * zz > 8 * sm_count_mg()) zz = (zz + 1) / 2;
      k_rb_zero_sweep<<<dim3(zx, zy, zz), dim3(32, 8), 0, stream()>>>(v, H->x32b[l], st,
          H->keep_on_skip);
      if (!launched("k_rb_zero_sweep")) return false;
    } else {
      launch_rbgs(sh, v, H->x32b[l], kc, st, H->keep_on_skip);
      if (!launched(sh.vec ? "k_rbgs_sweep_v" : "k_rbgs_sweep")) return false;
    }
    float *t = H->x32[l];
    H->x32[l] = H->x32b[l];
    H->x32b[l] = t;
  }
  return true;
}

template <typename T>
bool level_sweeps(MgHierarchy *H, int l, View<T> &v, int count, bool zero_first,
    const MgState *st)
{
  if constexpr (sizeof(T) == sizeof(float)) {
    if (!fused_sweeps(H, l, count, zero_first, st)) return false;
    v.x = reinterpret_cast<T *>(H->x32[l]);
    return true;
  } else {
    (void)H;
    (void)l;
    return sweeps<T>(v, count, zero_first, nullptr, st);
  }
}

// levels l .. nl-1 in one kernel (k_mg_tail)
template <typename T>
bool tail_vcycle(MgHierarchy *H, int l, T **xs, T **bs, bool zero)
{
  TailArgs<T> a;
  a.count = H->nl - l;
  for (int q = 0; q < a.count; q++) {
    const MgLevelDesc &L = H->lv[l + q];
    TailLevel<T> &t = a.lv[q];
    for (int ax = 0; ax < 3; ax++) {
      t.n[ax] = L.n[ax];
      t.r[ax] = L.r[ax];
    }
    const double d = 2.0 * (L.ih2[0] + L.ih2[1] + L.ih2[2]);
    t.ex = (T)L.ih2[0];
    t.ey = (T)L.ih2[1];
    t.ez = (T)L.ih2[2];
    t.diag = (T)d;
    t.inv_diag = (T)(L.relax / d);
    t.x = xs[l + q];
    t.b = bs[l + q];
  }
  if constexpr (sizeof(T) == sizeof(double))
    a.minv = reinterpret_cast<const T *>(H->minv64);
  else
    a.minv = reinterpret_cast<const T *>(H->minv32);
  a.pre = H->pre;
  a.post = H->post;
  a.coarse_sweeps = H->coarse_sweeps;
  a.zero_top = zero ? 1 : 0;
  a.st = H->d_state;
  k_mg_tail<T><<<1, 1024, 0, stream()>>>(a);
  return launched("k_mg_tail");
}

template <typename T>
bool vcycle(MgHierarchy *H, int l, T **xs, T **bs, bool zero, bool inner_test)
{
  const MgLevelDesc &L = H->lv[l];
  View<T> v = compact_view<T>(L, xs[l], bs[l]);
  const size_t n = (size_t)L.n[0] * L.n[1] * L.n[2];
  MgState *st = H->d_state;
  if (H->tail_l0 > 0 && l == H->tail_l0) return tail_vcycle<T>(H, l, xs, bs, zero);
  if (l == H->nl - 1) {
    const T *minv = nullptr;
    if constexpr (sizeof(T) == sizeof(double))
      minv = reinterpret_cast<const T *>(H->minv64);
    else
      minv = reinterpret_cast<const T *>(H->minv32);
    return coarse_solve<T>(v, H->coarse_sweeps, st, minv);
  }
  if (H->pre > 0) {
    if (!level_sweeps<T>(H, l, v, H->pre, zero, st)) return false;
  } else if (zero) {
    k_zero<T><<<flat_blocks((int64_t)n), kNT, 0, stream()>>>(xs[l], (int64_t)n);
    if (!launched("k_zero")) return false;
  }
  const bool ok = inner_test
                      ? restrict_to<T, FOLD_INNER>(v, bs[l + 1], H->lv[l + 1], nullptr, st, H->red)
                      : restrict_to<T, FOLD_NONE>(v, bs[l + 1], H->lv[l + 1], nullptr, st, H->red);
  if (!ok) return false;
  if (!vcycle<T>(H, l + 1, xs, bs, true, false)) return false;
  if (!prolong_to<T>(v, xs[l + 1], H->lv[l + 1], st)) return false;
  return level_sweeps<T>(H, l, v, H->post, false, st);
}

// initial guess by extrapolation in time (whole padded arrays, ghosts
// included): linear p <- 2 p(n-1) - p(n-2), quadratic (once two earlier
// solutions exist) p <- 3 p(n-1) - 3 p(n-2) + p(n-3), or cubic (once three
// exist) p <- 4 p(n-1) - 6 p(n-2) + 4 p(n-3) - p(n-4); until enough history
// exists the next lower order. hist[0] counts the earlier solutions kept
// (0 .. order) on the device, so the same launches serve host-driven and
// graph-captured steps. The history lives in `order` buffers whose roles
// rotate (hist[1]): buf[r] holds p(n-2), buf[r + 1] p(n-3), buf[r + 2] p(n-4)
// (indices mod order); the oldest is overwritten with p(n-1), the next step's
// p(n-2), so no history value is copied (quadratic: 40 bytes per cell instead
// of 48). The linear history is one buffer updated in place.
__global__ void k_extrapolate(double *__restrict__ p, double *buf0, double *buf1, double *buf2,
    int64_t n, const int *hist, int order)
{
  const int h = hist[0], r = order > 1 ? hist[1] : 0;
  double *const buf[3] = { buf0, buf1, buf2 };
  const double *a = buf[r];                            // p(n-2)
  const double *b = buf[order > 1 ? (r + 1) % order : r];  // p(n-3)
  const double *c = buf[order > 2 ? (r + 2) % order : r];  // p(n-4)
  double *o = buf[(r + order - 1) % order];            // the oldest, then p(n-1)
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const double cur = p[q];
    if (h >= 1) {
      const double prev = a[q];
      if (order >= 3 && h >= 3)
        p[q] = fma(4.0, cur + b[q], -fma(6.0, prev, c[q]));
      else if (order >= 2 && h >= 2)
        p[q] = 3.0 * (cur - prev) + b[q];
      else
        p[q] = 2.0 * cur - prev;
    }
    o[q] = cur;
  }
}

__global__ void k_hist_advance(int *hist, int order)
{
  if (hist[0] < order) hist[0] += 1;
  if (order > 1) hist[1] = (hist[1] + order - 1) % order;
}

__global__ void k_mx_fold(View<float> e, double *p, int p_sj, int p_sk, const MgState *st)
{
  if (solve_finished(st)) return;
  const int64_t n = (int64_t)e.nx * e.ny * e.nz;
  const int64_t q0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  FlatWalk w(q0, stride, e.nx, e.ny);
  for (int64_t q = q0; q < n; q += stride, w.advance(e.nx, e.ny)) {
    const int i = w.i, j = w.j, k = w.k;
    const int64_t pc = (int64_t)(k + 1) * p_sk + (int64_t)(j + 1) * p_sj + (i + 1);
    const double np = p[pc] + to_f64(e.x[q]);  // widening on the integer pipe, one DADD
    p[pc] = np;
    if (i == 0) p[pc - 1] = np;
    if (i == e.nx - 1) p[pc + 1] = np;
    if (j == 0) p[pc - p_sj] = np;
    if (j == e.ny - 1) p[pc + p_sj] = np;
    if (k == 0) p[pc - p_sk] = np;
    if (k == e.nz - 1) p[pc + p_sk] = np;
  }
}

// The same fold four cells at a time (rows a multiple of 4 cells): one
// 16-byte load of e and four independent loads of p per thread and step, so
// more of each thread's memory accesses are in flight.
__global__ void __launch_bounds__(kNT) k_mx_fold4(View<float> e, double *__restrict__ p,
    int p_sj, int p_sk, const MgState *st)
{
  if (solve_finished(st)) return;
  const int nq = e.nx / 4;
  const int64_t n = (int64_t)nq * e.ny * e.nz;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = g / nq;
    const int i = 4 * (int)(g - row * nq);
    const int j = (int)(row % e.ny), k = (int)(row / e.ny);
    const float4 ev = *reinterpret_cast<const float4 *>(e.x + row * e.nx + i);
    double *pp = p + (int64_t)(k + 1) * p_sk + (int64_t)(j + 1) * p_sj + (i + 1);
    const double a0 = pp[0], a1 = pp[1], a2 = pp[2], a3 = pp[3];
    const double n0 = a0 + to_f64(ev.x), n1 = a1 + to_f64(ev.y), n2 = a2 + to_f64(ev.z),
                 n3 = a3 + to_f64(ev.w);
    pp[0] = n0;
    pp[1] = n1;
    pp[2] = n2;
    pp[3] = n3;
    if (i == 0) pp[-1] = n0;
    if (i + 4 == e.nx) pp[4] = n3;
    const bool jl = j == 0, jh = j == e.ny - 1, kl = k == 0, kh = k == e.nz - 1;
    if (jl || jh || kl || kh) {
      const double nv[4] = { n0, n1, n2, n3 };
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (jl) pp[q - p_sj] = nv[q];
        if (jh) pp[q + p_sj] = nv[q];
        if (kl) pp[q - p_sk] = nv[q];
        if (kh) pp[q + p_sk] = nv[q];
      }
    }
  }
}

bool launch_fold(const View<float> &e, double *p, int p_sj, int p_sk, const MgState *st)
{
  const int64_t n = (int64_t)e.nx * e.ny * e.nz;
  if (e.nx % 4 == 0) {
    k_mx_fold4<<<flat_blocks(n / 4), kNT, 0, stream()>>>(e, p, p_sj, p_sk, st);
    return launched("k_mx_fold4");
  }
  k_mx_fold<<<flat_blocks(n), kNT, 0, stream()>>>(e, p, p_sj, p_sk, st);
  return launched("k_mx_fold");
}

bool cycle_fp64(MgHierarchy *H, double *p, const double *rhs)
{
  MgState *st = H->d_state;
  const double *shift = &st->shift;
  View<double> v0 = padded_view(H->lv[0], p, rhs);
  if (H->nl == 1) {
    if (!sweeps<double>(v0, H->coarse_sweeps, false, shift, st)) return false;
    // residual norm only
    return restrict_to<double, FOLD_OUTER>(v0, nullptr, H->lv[0], shift, st, H->red);
  }
  if (!sweeps<double>(v0, H->pre, false, shift, st)) return false;
  if (!restrict_to<double, FOLD_OUTER>(v0, H->b64[1], H->lv[1], shift, st, H->red)) return false;
  if (!vcycle<double>(H, 1, H->x64, H->b64, true, false)) return false;
  if (!prolong_to<double>(v0, H->x64[1], H->lv[1], st)) return false;
  return sweeps<double>(v0, H->post, false, shift, st);
}

// one outer iteration of mixed-precision refinement: FP64 residual (and stop
// test), up to `inner` FP32 V-cycles on A e = r (stopped on the device once
// ||r - A e|| <= theta * rtol ||b||, theta the key mg_theta), p += e in FP64
bool cycle_mixed(MgHierarchy *H, double *p, const double *rhs)
{
  MgState *st = H->d_state;
  View<double> v0 = padded_view(H->lv[0], p, rhs);
  if (!mx_residual(H, v0, st, H->nl == 1 ? 1 : 0, nullptr)) return false;
  const int inner = H->nl == 1 ? 1 : H->inner;
  for (int q = 0; q < inner; q++)
    if (!vcycle<float>(H, 0, H->x32, H->b32, q == 0, true)) return false;
  View<float> e = compact_view<float>(H->lv[0], H->x32[0], H->b32[0]);
  return launch_fold(e, p, v0.sy, v0.sz, st);
}

}  // namespace

bool mg_setup(Solver *s, Discretization *d, SolverState *ss)
{
  MgHierarchy *H = new MgHierarchy();
  ss->mg = H;
  const Extras &x = ss->ext;
  H->mode = ss->kind == SOLVER_MG_MIXED ? 1 : 0;
  H->pre = x.mg_pre;
  H->post = x.mg_post;
  H->coarse_sweeps = x.mg_coarse_sweeps;
  H->maxcycles = x.mg_maxcycles;
  H->inner = x.mg_inner < 1 ? 1 : x.mg_inner;
  H->theta = x.mg_theta;
  H->mx_df = !x.arith_fp64;
  H->keep_on_skip = (H->pre % 2 != 0 || H->post % 2 != 0) ? 1 : 0;
  H->guess = x.mg_guess >= 1 && x.mg_guess <= 3 ? x.mg_guess : 0;
  H->use_graph = x.mg_graph != 0;
  for (cudaStream_t &c : H->cap)
    if (!cuda_ok(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking), "mg capture stream"))
      return false;
  if (H->guess >= 1) {
    const size_t padded =
        (size_t)(d->grid.imax + 2) * (d->grid.jmax + 2) * (d->grid.kmax + 2) * sizeof(double);
    if (!cuda_ok(cudaMalloc(&H->p_prev, padded), "cudaMalloc(p_prev)")) return false;
    if (H->guess >= 2 && !cuda_ok(cudaMalloc(&H->p_prev2, padded), "cudaMalloc(p_prev2)"))
      return false;
    if (H->guess >= 3 && !cuda_ok(cudaMalloc(&H->p_prev3, padded), "cudaMalloc(p_prev3)"))
      return false;
    if (!cuda_ok(cudaMalloc(&H->d_hist, 2 * sizeof(int)), "cudaMalloc(hist)") ||
        !cuda_ok(cudaMemset(H->d_hist, 0, 2 * sizeof(int)), "hist init"))
      return false;
  }
  H->rtol = x.rtol;
  if (H->pre < 0 || H->post < 0 || H->coarse_sweeps < 0 || H->maxcycles < 1 || !(H->rtol >= 0) ||
      !(H->theta > 0 && H->theta <= 1) || !(x.mg_omega > 0 && x.mg_omega < 2)) {
    fail(NUSIF_ERR_ARG,
         "multigrid: invalid mg_pre/mg_post/mg_coarse/mg_cycles/rtol/mg_theta/mg_omega");
    return false;
  }
  H->nl = build_levels(&d->grid, x.mg_levels, H->lv);
  // over-relaxed red-black smoothing (mg_omega; 1 is Gauss-Seidel): the FP64
  // residual still decides convergence
  for (int l = 0; l < H->nl; l++) H->lv[l].relax = x.mg_omega;
  // the coarse tail: from the first level below the finest with at most
  // mg_tail cells (0: off), when it leaves at least two levels to it
  H->tail_l0 = 0;
  for (int l = 1; x.mg_tail > 0 && l < H->nl - 1; l++) {
    if ((int64_t)H->lv[l].n[0] * H->lv[l].n[1] * H->lv[l].n[2] <= x.mg_tail) {
      H->tail_l0 = l;
      break;
    }
  }
  for (int l = 0; l < H->nl; l++) {
    const size_t n = (size_t)H->lv[l].n[0] * H->lv[l].n[1] * H->lv[l].n[2];
    if (H->mode == 0 && l > 0) {
      if (!cuda_ok(cudaMalloc(&H->x64[l], n * sizeof(double)), "cudaMalloc(mg x)")) return false;
      if (!cuda_ok(cudaMalloc(&H->b64[l], n * sizeof(double)), "cudaMalloc(mg b)")) return false;
      cudaMemset(H->x64[l], 0, n * sizeof(double));
    }
    if (H->mode == 1) {
      if (!cuda_ok(cudaMalloc(&H->x32[l], n * sizeof(float)), "cudaMalloc(mg x32)")) return false;
      if (!cuda_ok(cudaMalloc(&H->x32b[l], n * sizeof(float)), "cudaMalloc(mg x32b)")) return false;
      if (!cuda_ok(cudaMalloc(&H->b32[l], n * sizeof(float)), "cudaMalloc(mg b32)")) return false;
      cudaMemset(H->x32[l], 0, n * sizeof(float));
      cudaMemset(H->x32b[l], 0, n * sizeof(float));
      cudaMemset(H->b32[l], 0, n * sizeof(float));
      if (H->lv[l].n[0] % 4 == 0 && l < H->nl - 1)
        H->kc[l] = x.mg_chunk > 0 ? x.mg_chunk
                                  : sweep_chunk_tuned(H->lv[l], H->x32[l], H->x32b[l], H->b32[l]);
    }
  }
  // coarsest level: exact solve when mg_coarse is 0 and the level is small
  // (FP64 mg with a single level smooths p itself, so it keeps sweeps)
  const MgLevelDesc &Lc = H->lv[H->nl - 1];
  const int nc = Lc.n[0] * Lc.n[1] * Lc.n[2];
  const bool single_fp64 = H->mode == 0 && H->nl == 1;
  if (H->coarse_sweeps == 0 && (nc > kMaxDirect || single_fp64)) H->coarse_sweeps = 64;
  if (H->coarse_sweeps == 0) {
    std::vector<double> minv;
    if (!coarse_inverse(Lc, minv)) {
      fail(NUSIF_ERR_STATE, "multigrid: coarsest operator factorisation failed");
      return false;
    }
    if (H->mode == 0) {
      if (!cuda_ok(cudaMalloc(&H->minv64, minv.size() * sizeof(double)), "cudaMalloc(minv)") ||
          !cuda_ok(cudaMemcpy(H->minv64, minv.data(), minv.size() * sizeof(double),
                       cudaMemcpyHostToDevice),
              "upload minv"))
        return false;
    } else {
      std::vector<float> m32(minv.begin(), minv.end());
      if (!cuda_ok(cudaMalloc(&H->minv32, m32.size() * sizeof(float)), "cudaMalloc(minv32)") ||
          !cuda_ok(cudaMemcpy(H->minv32, m32.data(), m32.size() * sizeof(float),
                       cudaMemcpyHostToDevice),
              "upload minv32"))
        return false;
    }
  }
  const int64_t n0 = (int64_t)d->grid.imax * d->grid.jmax * d->grid.kmax;
  const int red_blocks = std::max(flat_blocks(n0),
      mx_df_blocks(d->grid.imax, d->grid.jmax, d->grid.kmax));
  if (!reduce_scratch_alloc(H->red, red_blocks + 16)) return false;
  if (!cuda_ok(cudaMalloc(&H->stats2, sizeof(double) * (size_t)flat_blocks(n0)),
          "cudaMalloc(rhs partials)"))
    return false;
  if (!cuda_ok(cudaMalloc(&H->d_state, sizeof(MgState)), "cudaMalloc(mg state)")) return false;
  if (!cuda_ok(cudaMallocHost(&H->h_state, sizeof(MgState)), "cudaMallocHost(mg state)"))
    return false;
  memset(H->h_state, 0, sizeof(MgState));
  // expose the level arrays like the reference's r[] / e[] (solver-mg.c:375-388)
  for (int l = 0; l < H->nl; l++) {
    H->h_ptrs[l] = H->mode == 0 ? H->b64[l] : reinterpret_cast<double *>(H->b32[l]);
    H->h_ptrs[kMaxLevels + l] = H->mode == 0 ? H->x64[l] : reinterpret_cast<double *>(H->x32[l]);
  }
  s->r = H->h_ptrs;
  s->e = H->h_ptrs + kMaxLevels;
  s->levels = H->nl;
  s->presmooth = H->pre;
  s->postsmooth = H->post;
  return cuda_ok(cudaDeviceSynchronize(), "mg setup");
}

namespace {

__global__ void k_mg_state_init(MgState *st, double rtol2, double theta2, int maxcycles)
{
  MgState s;
  memset(&s, 0, sizeof(s));
  s.rtol2 = rtol2;
  s.theta2 = theta2;
  s.maxcycles = maxcycles;
  *st = s;
}

// after a captured solve: count a step whose last residual is above rtol (a
// fixed queue that ran out, or the mg_cycles limit)
__global__ void k_mg_count_unconverged(const MgState *st, int *counter, int *last_cycles)
{
  if (!(st->res2 <= st->tol2)) *counter += 1;
  *last_cycles = st->cycles;
}

// end of one unit inside a graph while-loop: run another while the solve is
// open. The unit count stops the loop on its own, whatever the flags say.
__global__ void k_mg_continue(MgState *st, cudaGraphConditionalHandle h, int cap)
{
  const int n = st->loops + 1;
  st->loops = n;
  cudaGraphSetConditional(h, (st->done == 0 && n < cap) ? 1u : 0u);
}

// before the inner loop of one refinement step: enter it while the solve is open
__global__ void k_inner_open(const MgState *st, cudaGraphConditionalHandle h)
{
  cudaGraphSetConditional(h, st->done == 0 ? 1u : 0u);
}

// end of one FP32 V-cycle of the inner loop: another while the correction is
// not yet good enough and fewer than `inner` V-cycles ran
__global__ void k_inner_continue(MgState *st, cudaGraphConditionalHandle h, int inner)
{
  const int n = st->inner_it + 1;
  st->inner_it = n;
  cudaGraphSetConditional(h, (st->done == 0 && st->inner_done == 0 && n < inner) ? 1u : 0u);
}

// before the units loop that follows an unrolled prefix: enter it while the
// solve is open
__global__ void k_loop_open(const MgState *st, cudaGraphConditionalHandle h)
{
  cudaGraphSetConditional(h, st->done == 0 ? 1u : 0u);
}

// the extrapolated warm start of p (mg_guess 1 / 2), before the solve
bool enqueue_warm_start(MgHierarchy *H, const View<double> &v0, double *p)
{
  if (H->guess < 1) return true;
  const int64_t padded = (int64_t)(v0.nx + 2) * (v0.ny + 2) * (v0.nz + 2);
  k_extrapolate<<<flat_blocks(padded), kNT, 0, stream()>>>(p, H->p_prev, H->p_prev2, H->p_prev3,
      padded, H->d_hist, H->guess);
  if (!launched("k_extrapolate")) return false;
  k_hist_advance<<<1, 1, 0, stream()>>>(H->d_hist, H->guess);
  return launched("k_hist_advance");
}

bool enqueue_solve_head(MgHierarchy *H, const View<double> &v0)
{
  k_mg_state_init<<<1, 1, 0, stream()>>>(H->d_state, H->rtol * H->rtol, H->theta * H->theta,
                                         H->maxcycles);
  if (!launched("k_mg_state_init")) return false;
  const int64_t n0 = (int64_t)v0.nx * v0.ny * v0.nz;
  const int blocks = flat_blocks(n0);
  (H->mx_df ? k_mg_rhs_stats<true> : k_mg_rhs_stats<false>)<<<blocks, kNT, 0, stream()>>>(
      v0, H->d_state, H->red.partials, H->stats2,
      H->red.ticket);
  if (!launched("k_mg_rhs_stats")) return false;
  k_mg_rhs_norm<<<blocks, kNT, 0, stream()>>>(v0, H->d_state, H->red.partials, H->red.ticket);
  return launched("k_mg_rhs_norm");
}

bool enqueue_solve_tail(MgHierarchy *H, const View<double> &v0, double *p, int *unconverged,
    int *last_cycles)
{
  if (!launch_pressure_ghosts(make_dims(v0.nx, v0.ny, v0.nz), p)) return false;
  k_mg_count_unconverged<<<1, 1, 0, stream()>>>(H->d_state, unconverged, last_cycles);
  return launched("k_mg_count_unconverged");
}

// a conditional handle of the graph being captured on s
bool make_handle(cudaStream_t s, unsigned dflt, unsigned flags, cudaGraphConditionalHandle *h)
{
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t graph = nullptr;
  if (!cuda_ok(cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, nullptr, nullptr, nullptr),
          "capture info"))
    return false;
  if (cs != cudaStreamCaptureStatusActive) {
    fail(NUSIF_ERR_STATE, "multigrid graph: no stream capture in progress");
    return false;
  }
  return cuda_ok(cudaGraphConditionalHandleCreate(h, graph, dflt, flags), "conditional handle");
}

// A while node with handle h appended to the graph being captured on s (after
// everything captured so far); its body is whatever `fill` launches, captured
// on `body` with the library stream set to `body`.
template <typename F>
bool capture_while(cudaStream_t s, cudaStream_t body, cudaGraphConditionalHandle h, F &&fill)
{
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t graph = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  const cudaGraphEdgeData *edges = nullptr;
  size_t ndeps = 0;
  if (!cuda_ok(cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, &edges, &ndeps),
          "capture info"))
    return false;
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  if (!cuda_ok(cudaGraphAddNode(&node, graph, deps, edges, ndeps, &cp), "while node")) return false;
  if (!cuda_ok(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                   cudaStreamSetCaptureDependencies),
          "capture dependencies"))
    return false;
  cudaGraph_t loop = cp.conditional.phGraph_out[0];
  if (!cuda_ok(cudaStreamBeginCaptureToGraph(body, loop, nullptr, nullptr, 0,
                   cudaStreamCaptureModeThreadLocal),
          "loop body capture"))
    return false;
  nusifSetStream(body);
  const bool ok = fill();
  nusifSetStream(s);
  const bool ended = cuda_ok(cudaStreamEndCapture(body, &loop), "loop body end");
  return ok && ended;
}

// One refinement step for a graph: FP64 residual (zeroing the correction),
// an inner while-loop of FP32 V-cycles that ends as soon as the correction
// meets its target (no V-cycle is launched past that point), p += e.
bool cycle_mixed_nested(MgHierarchy *H, double *p, const double *rhs, cudaStream_t inner_body)
{
  MgState *st = H->d_state;
  View<double> v0 = padded_view(H->lv[0], p, rhs);
  if (!mx_residual(H, v0, st, 0, H->x32[0])) return false;
  cudaStream_t s = stream();
  cudaGraphConditionalHandle h;
  if (!make_handle(s, 0, 0, &h)) return false;
  k_inner_open<<<1, 1, 0, s>>>(st, h);
  if (!launched("k_inner_open")) return false;
  const int inner = H->inner;
  const unsigned long long c0 = launch_count();
  if (!capture_while(s, inner_body, h, [&] {
        if (!vcycle<float>(H, 0, H->x32, H->b32, false, true)) return false;
        k_inner_continue<<<1, 1, 0, stream()>>>(st, h, inner);
        return launched("k_inner_continue");
      }))
    return false;
  H->n_inner_capture = (int)(launch_count() - c0);
  View<float> e = compact_view<float>(H->lv[0], H->x32[0], H->b32[0]);
  return launch_fold(e, p, v0.sy, v0.sz, st);
}

// mg-mixed without nested while-loops: a graph's conditional nodes cost tens
// of microseconds per evaluation, about a sixth of an FP32 V-cycle, so the
// common solve -- one refinement step of mg_inner V-cycles, then the FP64-class
// residual that finds it converged -- runs as straight-line launches: residual,
// mg_inner V-cycles (each stops at once when the correction has met its target
// or the solve is done; the first starts from the zeroed correction with the
// zero-start sweep), fold, residual. Only if that residual finds the solve
// still open does a while-loop of further refinement steps (the same launches
// and its own residual) run. The sequence is the host-driven cycle_mixed's,
// kernel for kernel, so the results are the same bits.
bool enqueue_mixed_unrolled(MgHierarchy *H, double *p, const double *rhs, cudaStream_t body)
{
  MgState *st = H->d_state;
  View<double> v0 = padded_view(H->lv[0], p, rhs);
  View<float> e = compact_view<float>(H->lv[0], H->x32[0], H->b32[0]);
  const auto unit = [&]() {
    for (int q = 0; q < H->inner; q++)
      if (!vcycle<float>(H, 0, H->x32, H->b32, q == 0, true)) return false;
    return launch_fold(e, p, v0.sy, v0.sz, st) && mx_residual(H, v0, st, 0, H->x32[0]);
  };
  const unsigned long long c0 = launch_count();
  if (!mx_residual(H, v0, st, 0, H->x32[0]) || !unit()) return false;
  cudaStream_t s = stream();
  cudaGraphConditionalHandle h;
  if (!make_handle(s, 0, 0, &h)) return false;
  k_loop_open<<<1, 1, 0, s>>>(st, h);
  if (!launched("k_loop_open")) return false;
  H->n_prefix = (int)(launch_count() - c0);
  const unsigned long long c1 = launch_count();
  const bool ok = capture_while(s, body, h, [&] {
    if (!unit()) return false;
    k_mg_continue<<<1, 1, 0, stream()>>>(st, h, H->maxcycles + 2);
    return launched("k_mg_continue");
  });
  H->n_body = (int)(launch_count() - c1);
  H->unrolled = ok;
  return ok;
}

// The solve's units as a while-loop of the graph captured on the library
// stream: one unit per iteration (an FP64 V-cycle, or one refinement step
// with its own inner loop), ended by the device once the solve is done, or
// after mg_cycles + 2 units whatever the device flags say (the solve itself
// sets done by mg_cycles units).
bool enqueue_units_loop(MgHierarchy *H, double *p, const double *rhs, cudaStream_t outer_body,
    cudaStream_t inner_body)
{
  if (H->mode == 1 && H->nl > 1) return enqueue_mixed_unrolled(H, p, rhs, outer_body);
  H->unrolled = false;
  cudaStream_t s = stream();
  cudaGraphConditionalHandle h;
  if (!make_handle(s, 1, cudaGraphCondAssignDefault, &h)) return false;
  const unsigned long long c0 = launch_count();
  H->n_inner_capture = 0;
  const bool ok = capture_while(s, outer_body, h, [&] {
    bool ok;
    if (H->mode == 0) ok = cycle_fp64(H, p, rhs);
    else if (H->nl == 1) ok = cycle_mixed(H, p, rhs);
    else ok = cycle_mixed_nested(H, p, rhs, inner_body);
    if (!ok) return false;
    k_mg_continue<<<1, 1, 0, stream()>>>(H->d_state, h, H->maxcycles + 2);
    return launched("k_mg_continue");
  });
  H->n_inner = H->n_inner_capture;
  H->n_outer = (int)(launch_count() - c0) - H->n_inner;
  return ok;
}

// the whole solve (head, units loop, pressure ghosts) as one graph for p, rhs
bool build_solve_graph(MgHierarchy *H, double *p, const double *rhs)
{
  if (H->graph) {
    cudaGraphExecDestroy(H->graph);
    H->graph = nullptr;
  }
  cudaStream_t lib = stream();
  cudaGraph_t g = nullptr;
  const unsigned long long c0 = launch_count();
  if (!cuda_ok(cudaStreamBeginCapture(H->cap[0], cudaStreamCaptureModeThreadLocal), "capture"))
    return false;
  nusifSetStream(H->cap[0]);
  View<double> v0 = padded_view(H->lv[0], p, rhs);
  bool ok = enqueue_solve_head(H, v0);
  H->n_head = (int)(launch_count() - c0);
  ok = ok && enqueue_units_loop(H, p, rhs, H->cap[1], H->cap[2]);
  const unsigned long long c1 = launch_count();
  ok = ok && launch_pressure_ghosts(make_dims(v0.nx, v0.ny, v0.nz), p);
  H->n_tail = (int)(launch_count() - c1);
  set_launch_count(c0);  // nothing ran yet
  nusifSetStream(lib);
  const bool ended = cuda_ok(cudaStreamEndCapture(H->cap[0], &g), "capture end");
  ok = ok && ended && cuda_ok(cudaGraphInstantiate(&H->graph, g, 0), "solve graph");
  if (g) cudaGraphDestroy(g);
  if (ok) {
    H->graph_p = p;
    H->graph_rhs = rhs;
  }
  return ok;
}

}  // namespace

// The solve as a fixed sequence of launches with no host synchronisation
// (graph capture): state initialisation, right-hand-side statistics, `queue`
// units (FP64 V-cycles for mg, outer refinement iterations for mg-mixed; the
// device-side flags turn the surplus into empty launches), ghost refresh, and
// a check that records steps whose queue was too short.
bool mg_enqueue(SolverState *ss, double *p, const double *rhs, int queue, int *unconverged,
    int *last_cycles)
{
  MgHierarchy *H = ss->mg;
  if (!H) {
    fail(NUSIF_ERR_STATE, "mg enqueue without a hierarchy");
    return false;
  }
  View<double> v0 = padded_view(H->lv[0], p, rhs);
  if (!enqueue_warm_start(H, v0, p) || !enqueue_solve_head(H, v0)) return false;
  for (int q = 0; q < queue; q++)
    if (!(H->mode == 0 ? cycle_fp64(H, p, rhs) : cycle_mixed(H, p, rhs))) return false;
  return enqueue_solve_tail(H, v0, p, unconverged, last_cycles);
}

// The same solve with its units in graph while-loops (mg_solve's graph), so
// that a step runs exactly the units of the host-driven solve; `body`
// captures the outer loop's body. Needs a capture in progress on the library
// stream.
bool mg_enqueue_loop(SolverState *ss, double *p, const double *rhs, cudaStream_t body,
    int *unconverged, int *last_cycles)
{
  MgHierarchy *H = ss->mg;
  if (!H) {
    fail(NUSIF_ERR_STATE, "mg enqueue without a hierarchy");
    return false;
  }
  View<double> v0 = padded_view(H->lv[0], p, rhs);
  return enqueue_warm_start(H, v0, p) && enqueue_solve_head(H, v0) &&
         enqueue_units_loop(H, p, rhs, body, H->cap[2]) &&
         enqueue_solve_tail(H, v0, p, unconverged, last_cycles);
}

// FP32 sweeps swap buffers on the host; a captured sequence must end with the
// same buffer current as it started, so every level needs an even number of
// sweeps per V-cycle (pre + post even)
bool mg_capture_ok(const SolverState *ss)
{
  const MgHierarchy *H = ss->mg;
  return H && (H->mode == 0 || (H->pre + H->post) % 2 == 0);
}

double mg_solve(Solver *s, SolverState *ss, double *p, const double *rhs)
{
  MgHierarchy *H = ss->mg;
  if (!H) {
    fail(NUSIF_ERR_STATE, "mg solve without a hierarchy");
    return NAN;
  }
  MgState *h = H->h_state;
  View<double> v0 = padded_view(H->lv[0], p, rhs);
  const int64_t n0 = (int64_t)v0.nx * v0.ny * v0.nz;
  const int blocks = flat_blocks(n0);
  if (!enqueue_warm_start(H, v0, p)) return NAN;
  // learned warm start: may replace p by the network's guess (never a worse residual)
  if (ss->guess && !guess_before_solve(ss->guess, s->grid, p, rhs)) return NAN;

  if (H->use_graph && mg_capture_ok(ss)) {
    // one graph launch: head, while-loops of units (and of FP32 V-cycles),
    // pressure ghosts; captured once per (p, rhs)
    if ((!H->graph || H->graph_p != p || H->graph_rhs != rhs) && !build_solve_graph(H, p, rhs))
      return NAN;
    if (!cuda_ok(cudaGraphLaunch(H->graph, stream()), "solve graph launch") ||
        !cuda_ok(cudaMemcpyAsync(h, H->d_state, sizeof(MgState), cudaMemcpyDeviceToHost,
                     stream()),
            "mg state download") ||
        !cuda_ok(cudaStreamSynchronize(stream()), "mg sync"))
      return NAN;
    // the kernels the graph ran: head, outer units, inner V-cycles, tail
    if (H->unrolled)
      set_launch_count(launch_count() + H->n_head + H->n_prefix +
                       (unsigned long long)h->loops * H->n_body + H->n_tail);
    else
      set_launch_count(launch_count() + H->n_head + (unsigned long long)h->loops * H->n_outer +
                       H->n_tail);
  } else {
    memset(h, 0, sizeof(*h));
    h->rtol2 = H->rtol * H->rtol;
    h->theta2 = H->theta * H->theta;
    h->maxcycles = H->maxcycles;
    if (!cuda_ok(cudaMemcpyAsync(H->d_state, h, sizeof(MgState), cudaMemcpyHostToDevice,
                     stream()),
            "mg state upload"))
      return NAN;
    (H->mx_df ? k_mg_rhs_stats<true> : k_mg_rhs_stats<false>)<<<blocks, kNT, 0, stream()>>>(
        v0, H->d_state, H->red.partials, H->stats2,
        H->red.ticket);
    if (!launched("k_mg_rhs_stats")) return NAN;
    k_mg_rhs_norm<<<blocks, kNT, 0, stream()>>>(v0, H->d_state, H->red.partials, H->red.ticket);
    if (!launched("k_mg_rhs_norm")) return NAN;
    int chunk = H->last_cycles > 0 ? H->last_cycles : 4;
    for (;;) {
      for (int q = 0; q < chunk; q++) {
        const bool ok = H->mode == 0 ? cycle_fp64(H, p, rhs) : cycle_mixed(H, p, rhs);
        if (!ok) return NAN;
      }
      if (!cuda_ok(cudaMemcpyAsync(h, H->d_state, sizeof(MgState), cudaMemcpyDeviceToHost,
                       stream()),
              "mg state download"))
        return NAN;
      if (!cuda_ok(cudaStreamSynchronize(stream()), "mg sync")) return NAN;
      if (h->done) break;
      chunk = 2;
    }
    if (!launch_pressure_ghosts(make_dims(v0.nx, v0.ny, v0.nz), p)) return NAN;
  }
  if (ss->guess && !guess_after_solve(ss->guess, s->grid, p)) return NAN;
  // queue as many units next time: V-cycles (mg) or residual evaluations (mg-mixed)
  H->last_cycles = H->mode == 0 ? h->cycles : h->outer + 1;
  ss->last_iterations = h->cycles;
  const double rel = h->nb2 > 0.0 ? sqrt(h->res2 / h->nb2) : 0.0;
  const char *v = getenv("NUSIF_VERBOSE");
  if (v && v[0] && v[0] != '0')
    printf("Multigrid took %d V-cycles to reach relative residual %e\n", h->cycles, rel);
  return rel;
}

// Average duration of `reps` launches of one fine-level kernel, between CUDA
// events on the library stream: which = 0 the fine smoother (mg-mixed: one
// whole FP32 sweep, one kernel; mg: one colour pass of the FP64 smoother),
// 1 the FP64 residual of mg-mixed. It works on
// scratch copies or on the solver's own FP32 arrays, never on p; a private
// state that never stops keeps the kernels active.
bool mg_time_kernel(SolverState *ss, const double *p, const double *rhs, int which, int reps,
    double *ms_out)
{
  MgHierarchy *H = ss->mg;
  if (!H || reps < 1) return false;
  MgState host_st;
  memset(&host_st, 0, sizeof(host_st));
  host_st.maxcycles = 1 << 30;
  host_st.tol2 = -1.0;
  host_st.tol_inner = -1.0;
  MgState *tst = nullptr;
  double *pcopy = nullptr;
  const size_t padded = (size_t)(H->lv[0].n[0] + 2) * (H->lv[0].n[1] + 2) * (H->lv[0].n[2] + 2);
  bool ok = cuda_ok(cudaMalloc(&tst, sizeof(MgState)), "cudaMalloc(timing state)") &&
            cuda_ok(cudaMemcpy(tst, &host_st, sizeof(MgState), cudaMemcpyHostToDevice),
                "timing state upload") &&
            cuda_ok(cudaMalloc(&pcopy, padded * sizeof(double)), "cudaMalloc(timing p)") &&
            cuda_ok(cudaMemcpyAsync(pcopy, p, padded * sizeof(double), cudaMemcpyDeviceToDevice,
                        stream()),
                "timing p copy");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  View<double> v0 = padded_view(H->lv[0], pcopy, rhs);
  // which >= 2 (mg-mixed): one FP32 V-cycle from level which - 2 down, from
  // zero on that level's current right-hand side, captured once as a CUDA
  // graph and replayed (as inside a solve)
  cudaGraph_t vg = nullptr;
  cudaGraphExec_t vge = nullptr;
  if (ok && which >= 2) {
    if (H->mode != 1 || which - 2 >= H->nl) {
      fail(NUSIF_ERR_ARG, "nusifTimeKernel: which >= 2 times mg-mixed V-cycles from a level");
      ok = false;
    } else {
      // copies above are ordered before the capture stream's work
      ok = cuda_ok(cudaStreamSynchronize(stream()), "timing sync");
      MgState *keep = H->d_state;
      cudaStream_t lib = stream();
      const unsigned long long c0 = launch_count();
      H->d_state = tst;
      ok = ok && cuda_ok(cudaStreamBeginCapture(H->cap[0], cudaStreamCaptureModeThreadLocal),
                     "timing capture");
      nusifSetStream(H->cap[0]);
      const bool built = ok && vcycle<float>(H, which - 2, H->x32, H->b32, true, false);
      nusifSetStream(lib);
      set_launch_count(c0);  // the capture ran nothing
      ok = ok && cuda_ok(cudaStreamEndCapture(H->cap[0], &vg), "timing capture end") && built &&
           cuda_ok(cudaGraphInstantiate(&vge, vg, 0), "timing graph");
      H->d_state = keep;
    }
  }
  if (ok) {
    // one untimed launch, then the timed ones
    for (int q = 0; q <= reps && ok; q++) {
      if (q == 1) cudaEventRecord(e0, stream());
      if (which >= 2) {
        ok = cuda_ok(cudaGraphLaunch(vge, stream()), "timing graph launch");
      } else if (which == 1 && H->mode == 1) {
        ok = mx_residual(H, v0, tst, 0, nullptr);
      } else if (H->mode == 1) {
        ok = fused_sweeps(H, 0, 1, false, tst);  // one whole sweep
      } else {
        ok = smooth_pass<double, false>(v0, q & 1, nullptr, tst);
      }
    }
    cudaEventRecord(e1, stream());
  }
  float ms = 0.0f;
  if (ok && cuda_ok(cudaEventSynchronize(e1), "timing sync")) {
    cudaEventElapsedTime(&ms, e0, e1);
    *ms_out = ms / reps;
  } else {
    ok = false;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (vge) cudaGraphExecDestroy(vge);
  if (vg) cudaGraphDestroy(vg);
  if (tst) cudaFree(tst);
  if (pcopy) cudaFree(pcopy);
  return ok;
}

void mg_free(Solver *s, SolverState *ss)
{
  MgHierarchy *H = ss->mg;
  if (!H) return;
  for (int l = 0; l < kMaxLevels; l++) {
    if (H->x64[l]) cudaFree(H->x64[l]);
    if (H->b64[l]) cudaFree(H->b64[l]);
    if (H->x32[l]) cudaFree(H->x32[l]);
    if (H->x32b[l]) cudaFree(H->x32b[l]);
    if (H->b32[l]) cudaFree(H->b32[l]);
  }
  if (H->graph) cudaGraphExecDestroy(H->graph);
  if (H->stats2) cudaFree(H->stats2);
  for (cudaStream_t c : H->cap)
    if (c) cudaStreamDestroy(c);
  if (H->p_prev) cudaFree(H->p_prev);
  if (H->p_prev2) cudaFree(H->p_prev2);
  if (H->p_prev3) cudaFree(H->p_prev3);
  if (H->d_hist) cudaFree(H->d_hist);
  if (H->minv64) cudaFree(H->minv64);
  if (H->minv32) cudaFree(H->minv32);
  if (H->d_state) cudaFree(H->d_state);
  if (H->h_state) cudaFreeHost(H->h_state);
  reduce_scratch_free(H->red);
  delete H;
  ss->mg = nullptr;
  if (s) {
    s->r = nullptr;
    s->e = nullptr;
  }
}

}  // namespace nusif

using namespace nusif;

extern "C" {

// One or more exact red-black Gauss-Seidel sweeps of the multigrid's FP32
// smoother (the one-kernel sweep; ghost-free Neumann operator) on compact
// device arrays x[nz][ny][nx] -> xout; first colour (i + j + k) even, 0-based.
// x null: the sweeps start from zero (the first one by the zero-start kernel).
int nusifSmoothRBF32(const float *x, const float *b, float *xout, int nx, int ny, int nz,
    double hx, double hy, double hz, int sweeps)
{
  if (!b || !xout || nx < 4 || ny < 1 || nz < 1 || nx % 4 || sweeps < 1 || !(hx > 0) ||
      !(hy > 0) || !(hz > 0)) {
    fail(NUSIF_ERR_ARG, "nusifSmoothRBF32: needs device arrays, nx a multiple of 4, sweeps >= 1");
    return NUSIF_ERR_ARG;
  }
  MgHierarchy H;
  H.nl = 1;
  MgLevelDesc &L = H.lv[0];
  L.n[0] = nx;
  L.n[1] = ny;
  L.n[2] = nz;
  L.r[0] = L.r[1] = L.r[2] = 1;
  L.ih2[0] = 1.0 / (hx * hx);
  L.ih2[1] = 1.0 / (hy * hy);
  L.ih2[2] = 1.0 / (hz * hz);
  const size_t n = (size_t)nx * ny * nz;
  float *scratch = nullptr;
  MgState *st = nullptr;
  bool ok = cuda_ok(cudaMalloc(&scratch, 2 * n * sizeof(float)), "cudaMalloc(smooth)") &&
            cuda_ok(cudaMalloc(&st, sizeof(MgState)), "cudaMalloc(smooth)") &&
            cuda_ok(cudaMemsetAsync(st, 0, sizeof(MgState), stream()), "smooth state") &&
            (x ? cuda_ok(cudaMemcpyAsync(scratch, x, n * sizeof(float), cudaMemcpyDeviceToDevice,
                             stream()),
                     "smooth copy")
               : cuda_ok(cudaMemsetAsync(scratch, 0, n * sizeof(float), stream()), "smooth zero"));
  H.x32[0] = scratch;
  H.x32b[0] = scratch + n;
  H.b32[0] = const_cast<float *>(b);
  ok = ok && fused_sweeps(&H, 0, sweeps, x == nullptr, st) &&
       cuda_ok(cudaMemcpyAsync(xout, H.x32[0], n * sizeof(float), cudaMemcpyDeviceToDevice,
                   stream()),
           "smooth copy") &&
       cuda_ok(cudaStreamSynchronize(stream()), "smooth");
  H.x32[0] = H.x32b[0] = H.b32[0] = nullptr;
  if (scratch) cudaFree(scratch);
  if (st) cudaFree(st);
  return ok ? NUSIF_OK : NUSIF_ERR_CUDA;
}

int nusifConvertF64ToF32(const double *x, float *y, long long n)
{
  if (!x || !y || n < 0) {
    fail(NUSIF_ERR_ARG, "nusifConvertF64ToF32: needs device arrays and n >= 0");
    return NUSIF_ERR_ARG;
  }
  if (n == 0) return NUSIF_OK;
  k_to_f32<<<flat_blocks(n), kNT, 0, stream()>>>(x, y, n);
  return launched("k_to_f32") && cuda_ok(cudaStreamSynchronize(stream()), "convert")
             ? NUSIF_OK : NUSIF_ERR_CUDA;
}

int nusifConvertF32ToF64(const float *x, double *y, long long n)
{
  if (!x || !y || n < 0) {
    fail(NUSIF_ERR_ARG, "nusifConvertF32ToF64: needs device arrays and n >= 0");
    return NUSIF_ERR_ARG;
  }
  if (n == 0) return NUSIF_OK;
  k_to_f64<<<flat_blocks(n), kNT, 0, stream()>>>(x, y, n);
  return launched("k_to_f64") && cuda_ok(cudaStreamSynchronize(stream()), "convert")
             ? NUSIF_OK : NUSIF_ERR_CUDA;
}

}  // extern "C"
