// Learned pressure warm start around a multigrid solve (no reference
// counterpart). The network works on the half-resolution grid:
//
//   features  x = [R(b - s - A p0) / sigma_r, R(b - s) / sigma_b]
//   target    t = R(p* - p0) * kappa / sigma_r
//   guess     p1 = p0 + P(net(x) * sigma_r / kappa)
//
// p0 the warm start (previous or extrapolated p), p* the converged p, s the
// mean of b, A the multigrid's ghost-free Neumann operator, kappa =
// pi^2 (1/Lx^2 + 1/Ly^2 + 1/Lz^2) the scale of its smallest eigenvalues (so
// that targets are O(1) and independent of the resolution),
// R the 8-child mean, P trilinear interpolation (the multigrid's transfers),
// sigma the RMS of each restricted field. The solver keeps p1 only when its
// restricted residual ||R(b - s - A p1)|| is below that of p0, so the plain
// warm start stays the fallback; the V-cycles then run to the same tolerance
// either way.
//
// Every reduction folds per-block partials in a fixed order (deterministic).
#include <cmath>

#include "df32.cuh"
#include "fp_bits.cuh"
#include "nusif_internal.h"
#include "reduce.cuh"
#include "solver_internal.h"
#include "unet_internal.h"

namespace nusif {

struct GuessStats {
  double shift;    // mean of b over the interior
  double nb2;      // ||b - s||^2 (fine)
  double r2_warm;  // ||b - s - A p0||^2 (fine)
  double r2_cand;  // ||b - s - A p1||^2 (fine)
  double rc2, bc2; // sums of squares of the restricted residual of p0 and of the rhs
  double rc2_cand; // sum of squares of the restricted residual of p1 (the decision)
  double sigma_r, sigma_b;
  int used;        // p1 replaced p0
  int pad;
};

struct GuessState {
  NusifUNet *net = nullptr;
  float *rec_x = nullptr, *rec_t = nullptr;  // caller's buffers of a recording request
  bool recording = false;
  int nx = 0, ny = 0, nz = 0;
  float *x = nullptr;       // own feature buffer [nc][2]
  double *aux = nullptr;    // padded: p0 (recording) or p1 (candidate)
  double *partial = nullptr;
  GuessStats *d_stats = nullptr, *h_stats = nullptr;
  int64_t nc = 0;
  // key mg_probe P > 1: after two rejections in a row the network runs only
  // every P-th step until a guess is taken again (the plain warm start is used
  // in between, as after a rejection)
  int probe_every = 1;
  int rejections = 0;     // evaluated steps in a row whose guess lost
  int skip_left = 0;      // steps to go without the network
  bool evaluated = false; // the network ran for the current solve
  long long n_eval = 0, n_taken = 0;
};

namespace {

constexpr int kNT = 256;
constexpr int kBlocks = 4 * 152;  // partial slots per reduction

struct GGeom {
  int nx, ny, nz;     // fine interior
  int sj, sk;         // padded strides
  double ex, ey, ez;  // 1/h^2
  double kappa;       // pi^2 (1/Lx^2 + 1/Ly^2 + 1/Lz^2): the operator's smallest-eigenvalue scale
  __device__ int64_t pidx(int i, int j, int k) const
  {
    return (int64_t)(k + 1) * sk + (int64_t)(j + 1) * sj + (i + 1);
  }
};

// the operator's constants as double-float pairs: 1/h^2 per axis, -s
struct GPairs {
  df::f2 ex, ey, ez, ms;
};

template <int K>
__device__ __forceinline__ void block_partials(double (&v)[K], double *partial)
{
  __shared__ double sm[kNT / 32];
  // one slot per block of a 1-, 2- or 3-D grid, written by its first thread
  const int64_t bid =
      blockIdx.x + (int64_t)gridDim.x * (blockIdx.y + (int64_t)gridDim.y * blockIdx.z);
  const bool first = threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0;
#pragma unroll
  for (int q = 0; q < K; q++) {
    const double t = block_reduce_sum<kNT>(v[q], sm);
    if (first) partial[bid * K + q] = t;
  }
}

// component k of K per-block partials stored interleaved, summed by one whole
// block in a fixed order (thread t takes the blocks t, t + kNT, ..., then a
// fixed tree): deterministic, and the same order for every call on the same
// sequence of partials
template <int K>
__device__ __forceinline__ double fold_k(const double *partial, int nb, int k, double *sm)
{
  double s = 0.0;
  for (int q = threadIdx.x; q < nb; q += kNT) s += partial[K * q + k];
  return block_reduce_sum<kNT>(s, sm);
}

// sum of b over the interior: a block per interior row (j, k), its threads
// along the row
__global__ void __launch_bounds__(kNT) k_g_sum_b(GGeom g, const double *b, double *partial)
{
  const int rows = g.ny * g.nz;
  double v[1] = { 0.0 };
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const double *row = b + g.pidx(0, r % g.ny, r / g.ny);
    for (int i = threadIdx.x; i < g.nx; i += kNT) v[0] += row[i];
  }
  block_partials<1>(v, partial);
}

__global__ void __launch_bounds__(kNT) k_g_fold_shift(const double *partial, int nb, int64_t n,
    GuessStats *st)
{
  __shared__ double sm[kNT / 32];
  const double s = fold_k<1>(partial, nb, 0, sm);
  if (threadIdx.x == 0) st->shift = s / (double)n;
}

// The restricted residual R(b - s - A p) (and, with FEAT, R(b - s)) on 32 x 8
// tiles of fine columns marching an even chunk of fine planes. Each fine
// cell's residual b - s - A p of the ghost-free Neumann operator (a missing
// neighbour is the cell itself) in double-float pairs (about 2^-47 of the
// operands: the warm start's residual cancels b - A p to a small fraction of
// b), from a shared-memory plane of p split once per block and plane with a
// one-cell ring; a coarse cell's eight children combined in a fixed order: x
// pairs by shuffle, z pairs in registers, y pairs through shared memory. The
// squares are summed in FP32 over a coarse cell's children, then in FP64 per
// thread and block. FEAT writes the features x (unnormalised) and four sums
// of squares [fine residual, fine rhs, coarse residual, coarse rhs]; without
// it the kernel writes the two of the candidate [fine, coarse residual] with
// the same operations in the same order, so p1 == p0 gives the same bits.
constexpr int kGX = 32, kGY = 8;
template <bool FEAT>
__global__ void __launch_bounds__(kNT) k_g_coarse(GGeom g, GPairs pc, const double *p,
    const double *b, const GuessStats *st, float *x, double *partial, int kb)
{
  using namespace df;
  __shared__ f2 pl[2][kGY + 2][kGX + 2];
  __shared__ float ysum[kGY / 2][kGX / 2][6];  // odd rows' pair sums: rs, bs (pairs), rr2, bb2
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kGX + tx;
  const int i0 = blockIdx.x * kGX, j0 = blockIdx.y * kGY;
  const bool act = i0 + tx < g.nx;  // rows: ny is a multiple of 8
  const int i = min(i0 + tx, g.nx - 1), j = j0 + ty;
  const int k0 = blockIdx.z * kb, k1 = min(k0 + kb, g.nz);
  const auto at = [&](const double *a, int ii, int jj, int kk) {
    return a[g.pidx(min(max(ii, 0), g.nx - 1), min(max(jj, 0), g.ny - 1), min(max(kk, 0), g.nz - 1))];
  };
  // ring cell of this thread (threads 0..79): rows j0-1 and j0+8, columns i0-1 and i0+32
  const bool ring = tid < 2 * kGX + 2 * kGY;
  int rr = 0, rc = 0;
  if (ring) {
    if (tid < 2 * kGX) {
      rc = (tid & (kGX - 1)) + 1;
      rr = tid < kGX ? 0 : kGY + 1;
    } else {
      const int q = tid - 2 * kGX;
      rr = (q & (kGY - 1)) + 1;
      rc = q < kGY ? 0 : kGX + 1;
    }
  }
  const f2 ex = pc.ex, ey = pc.ey, ez = pc.ez, ms = split(-st->shift);
  f2 zb = split(at(p, i, j, k0 - 1)), zc = split(at(p, i, j, k0));
  double xn = at(p, i, j, k0 + 1);
  double rn = ring ? at(p, i0 - 1 + rc, j0 - 1 + rr, k0) : 0.0;
  f2 zr{ 0.0f, 0.0f }, zq{ 0.0f, 0.0f };  // z-pair sums of the x-pair sums of residual and rhs
  float zr2 = 0.0f, zb2 = 0.0f;
  constexpr int NV = FEAT ? 4 : 2;
  double v[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = 0.0;
  const int cx = g.nx / 2, cy = g.ny / 2;
  int buf = 0;
  for (int k = k0; k < k1; k++) {
    pl[buf][ty + 1][tx + 1] = zc;
    if (ring) pl[buf][rr][rc] = split(rn);
    const f2 zt = split(xn);
    if (k + 1 < k1) {
      xn = at(p, i, j, k + 2);
      if (ring) rn = at(p, i0 - 1 + rc, j0 - 1 + rr, k + 1);
    }
    const double bv = at(b, i, j, k);
    __syncthreads();
    // this cell's residual: the ghost-free Neumann Laplacian in pairs
    const f2 x2 = f2{ 2.0f * zc.hi, 2.0f * zc.lo };  // exact
    f2 lap = mul_u(ex, sub_u(add_u(pl[buf][ty + 1][tx], pl[buf][ty + 1][tx + 2]), x2));
    lap = fma_u(ey, sub_u(add_u(pl[buf][ty][tx + 1], pl[buf][ty + 2][tx + 1]), x2), lap);
    lap = fma_u(ez, sub_u(add_u(zb, zt), x2), lap);
    const f2 nb = add(split(bv), ms);
    const f2 r = sub(nb, lap);
    // x pairs (even lane + odd lane), then z pairs over the plane pair
    const f2 ro{ __shfl_xor_sync(0xffffffffu, r.hi, 1), __shfl_xor_sync(0xffffffffu, r.lo, 1) };
    const f2 bo{ __shfl_xor_sync(0xffffffffu, nb.hi, 1), __shfl_xor_sync(0xffffffffu, nb.lo, 1) };
    const f2 xr = add(r, ro), xb = add(nb, bo);
    const float xr2 = fmaf(ro.hi, ro.hi, r.hi * r.hi), xb2 = fmaf(bo.hi, bo.hi, nb.hi * nb.hi);
    if (((k - k0) & 1) == 0) {
      zr = xr;
      zq = xb;
      zr2 = xr2;
      zb2 = xb2;
    } else {
      zr = add(zr, xr);
      zq = add(zq, xb);
      zr2 += xr2;
      zb2 += xb2;
      // y pairs: the odd row hands its sums to the even row
      const bool lead = !(tx & 1);
      if ((ty & 1) && lead) {
        float *o = ysum[ty >> 1][tx >> 1];
        o[0] = zr.hi;
        o[1] = zr.lo;
        o[2] = zq.hi;
        o[3] = zq.lo;
        o[4] = zr2;
        o[5] = zb2;
      }
      __syncthreads();
      if (!(ty & 1) && lead && act) {
        const float *o = ysum[ty >> 1][tx >> 1];
        f2 rs = add(zr, f2{ o[0], o[1] }), bs = add(zq, f2{ o[2], o[3] });
        const float rr2 = zr2 + o[4], bb2 = zb2 + o[5];
        rs = f2{ 0.125f * rs.hi, 0.125f * rs.lo };  // exact
        bs = f2{ 0.125f * bs.hi, 0.125f * bs.lo };
        v[0] += to_f64(rr2);
        if (FEAT) {
          v[1] += to_f64(bb2);
          v[2] += to_f64(rs.hi * rs.hi);
          v[3] += to_f64(bs.hi * bs.hi);
          const int q = ((k >> 1) * cy + (j >> 1)) * cx + (i >> 1);
          x[2 * q] = rs.hi;
          x[2 * q + 1] = bs.hi;
        } else {
          v[NV - 1] += to_f64(rs.hi * rs.hi);
        }
      }
    }
    zb = zc;
    zc = zt;
    buf ^= 1;
  }
  block_partials<NV>(v, partial);
}

// the tiled kernel's grid: tiles of 32 x 8 columns, the planes in even chunks,
// at most kBlocks blocks where the tiles allow (the partials buffer's size)
dim3 coarse_grid(const GGeom &g, int &kb)
{
  const int tiles = ((g.nx + kGX - 1) / kGX) * (g.ny / kGY);
  int chunks = tiles >= kBlocks ? 1 : kBlocks / tiles;
  if (chunks > g.nz / 2) chunks = g.nz / 2;
  if (chunks < 1) chunks = 1;
  kb = ((g.nz / 2 + chunks - 1) / chunks) * 2;  // even
  chunks = (g.nz + kb - 1) / kb;
  return dim3((g.nx + kGX - 1) / kGX, g.ny / kGY, chunks);
}

__global__ void __launch_bounds__(kNT) k_g_fold_features(const double *partial, int nb,
    int64_t nc, GuessStats *st)
{
  __shared__ double sm[kNT / 32];
  double t[4];
  for (int k = 0; k < 4; k++) t[k] = fold_k<4>(partial, nb, k, sm);
  if (threadIdx.x != 0) return;
  st->r2_warm = t[0];
  st->nb2 = t[1];
  st->rc2 = t[2];
  st->bc2 = t[3];
  const double sr = sqrt(t[2] / (double)nc), sb = sqrt(t[3] / (double)nc);
  st->sigma_r = sr > 0.0 ? sr : 1.0;
  st->sigma_b = sb > 0.0 ? sb : 1.0;
  st->used = 0;
  st->r2_cand = 0.0;
}

__global__ void k_g_normalize(float *x, int64_t nc, const GuessStats *st)
{
  const float ir = (float)(1.0 / st->sigma_r), ib = (float)(1.0 / st->sigma_b);
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nc;
       q += (int64_t)gridDim.x * blockDim.x) {
    x[2 * q] *= ir;
    x[2 * q + 1] *= ib;
  }
}

// t = R(p* - p0) * kappa / sigma_r
__global__ void k_g_target(GGeom g, const double *pconv, const double *p0, const GuessStats *st,
    float *t)
{
  const int cx = g.nx / 2, cy = g.ny / 2, cz = g.nz / 2;
  const int64_t n = (int64_t)cx * cy * cz;
  const double scale = g.kappa / st->sigma_r;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int I = (int)(q % cx);
    const int64_t r = q / cx;
    const int J = (int)(r % cy), K = (int)(r / cy);
    double s = 0.0;
    for (int c = 0; c < 8; c++) {
      const int64_t f = g.pidx(2 * I + (c & 1), 2 * J + ((c >> 1) & 1), 2 * K + (c >> 2));
      s += pconv[f] - p0[f];
    }
    t[q] = (float)(0.125 * s * scale);
  }
}

// p1 = p0 + P(out * sigma_r / kappa) on the interior, Neumann ghosts from it;
// trilinear weights 3/4 and 1/4 toward the coarse neighbour on the fine
// cell's side (clamped at the walls), as the multigrid prolongation. The
// correction is interpolated in FP32 (the network's output is BF16-rounded)
// and added to the binary64 p0 in one FP64 addition.
__global__ void k_g_candidate(GGeom g, const double *p0, const float *out, const GuessStats *st,
    double *p1)
{
  const int cx = g.nx / 2, cy = g.ny / 2, cz = g.nz / 2;
  const float scale = (float)(st->sigma_r / g.kappa);
  // a block per interior row (j, k), its threads along the row
  for (int row = blockIdx.x; row < g.ny * g.nz; row += gridDim.x) {
    const int j = row % g.ny, k = row / g.ny;
    for (int i = threadIdx.x; i < g.nx; i += blockDim.x) {
      const int P[3] = { i >> 1, j >> 1, k >> 1 };
      const int C[3] = { cx, cy, cz };
      const int F[3] = { i, j, k };
      int Q[3];
      for (int a = 0; a < 3; a++) {
        const int nb = (F[a] & 1) ? P[a] + 1 : P[a] - 1;
        Q[a] = (nb < 0 || nb >= C[a]) ? P[a] : nb;
      }
      float e = 0.0f;
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const int X = (c & 1) ? Q[0] : P[0], Y = ((c >> 1) & 1) ? Q[1] : P[1], Z = (c >> 2) ? Q[2] : P[2];
        const float w = ((c & 1) ? 0.25f : 0.75f) * (((c >> 1) & 1) ? 0.25f : 0.75f) *
                        ((c >> 2) ? 0.25f : 0.75f);
        e = fmaf(w, out[(Z * cy + Y) * cx + X], e);
      }
      const int64_t pc = g.pidx(i, j, k);
      const double v = p0[pc] + to_f64(e * scale);
      p1[pc] = v;
      if (i == 0) p1[pc - 1] = v;
      if (i == g.nx - 1) p1[pc + 1] = v;
      if (j == 0) p1[pc - g.sj] = v;
      if (j == g.ny - 1) p1[pc + g.sj] = v;
      if (k == 0) p1[pc - g.sk] = v;
      if (k == g.nz - 1) p1[pc + g.sk] = v;
    }
  }
}

// the guess is kept when its restricted residual is smaller: the smooth error
// is what the V-cycles pay for; the high-frequency residual that interpolating
// a coarse correction leaves is removed by the first smoothing sweep
__global__ void __launch_bounds__(kNT) k_g_fold_select(const double *partial, int nb,
    GuessStats *st)
{
  __shared__ double sm[kNT / 32];
  const double s = fold_k<2>(partial, nb, 0, sm), sc = fold_k<2>(partial, nb, 1, sm);
  if (threadIdx.x != 0) return;
  st->r2_cand = s;
  st->rc2_cand = sc;
  st->used = sc < st->rc2 ? 1 : 0;
}

// p = p1 over the whole padded array when the guess won
__global__ void k_g_take(double *p, const double *p1, int64_t n, const GuessStats *st)
{
  if (!st->used) return;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    p[q] = p1[q];
}

// the operator's constants as pairs, formed on the host
GPairs gpairs(const GGeom &g)
{
  GPairs c;
  c.ex = df::from_double_rn(g.ex);
  c.ey = df::from_double_rn(g.ey);
  c.ez = df::from_double_rn(g.ez);
  c.ms = df::f2{ 0.0f, 0.0f };  // -shift, filled in on the device
  return c;
}

GGeom geom(const Grid *grid)
{
  GGeom g;
  g.nx = grid->imax;
  g.ny = grid->jmax;
  g.nz = grid->kmax;
  g.sj = grid->imax + 2;
  g.sk = (grid->imax + 2) * (grid->jmax + 2);
  g.ex = 1.0 / (grid->dx * grid->dx);
  g.ey = 1.0 / (grid->dy * grid->dy);
  g.ez = 1.0 / (grid->dz * grid->dz);
  const double lx = grid->imax * grid->dx, ly = grid->jmax * grid->dy, lz = grid->kmax * grid->dz;
  g.kappa = 9.869604401089358 * (1.0 / (lx * lx) + 1.0 / (ly * ly) + 1.0 / (lz * lz));
  return g;
}

int flat(int64_t n)
{
  int64_t b = (n + 255) / 256;
  return (int)(b > kBlocks ? kBlocks : (b < 1 ? 1 : b));
}

bool ensure(GuessState *gs, const Grid *grid)
{
  if (grid->imax % 8 || grid->jmax % 8 || grid->kmax % 8) {
    fail(NUSIF_ERR_ARG, "learned warm start: grid %dx%dx%d needs every edge a multiple of 8",
        grid->imax, grid->jmax, grid->kmax);
    return false;
  }
  if (gs->nx == grid->imax && gs->ny == grid->jmax && gs->nz == grid->kmax) return true;
  if (gs->nx) {
    fail(NUSIF_ERR_STATE, "learned warm start: grid changed");
    return false;
  }
  gs->nx = grid->imax;
  gs->ny = grid->jmax;
  gs->nz = grid->kmax;
  gs->nc = (int64_t)gs->nx * gs->ny * gs->nz / 8;
  const size_t padded = (size_t)(gs->nx + 2) * (gs->ny + 2) * (gs->nz + 2);
  // partials: kBlocks for the flat kernels, one per block of the tiled one (at
  // least one per 32 x 8 tile)
  const size_t tiles = (size_t)((gs->nx + kGX - 1) / kGX) * (gs->ny / kGY);
  const size_t nparts = tiles > (size_t)kBlocks ? tiles : (size_t)kBlocks;
  return cuda_ok(cudaMalloc(&gs->x, gs->nc * 2 * sizeof(float)), "cudaMalloc(guess)") &&
         cuda_ok(cudaMalloc(&gs->aux, padded * sizeof(double)), "cudaMalloc(guess)") &&
         cuda_ok(cudaMalloc(&gs->partial, nparts * 4 * sizeof(double)), "cudaMalloc(guess)") &&
         cuda_ok(cudaMalloc(&gs->d_stats, sizeof(GuessStats)), "cudaMalloc(guess)") &&
         cuda_ok(cudaMallocHost(&gs->h_stats, sizeof(GuessStats)), "cudaMallocHost(guess)") &&
         cuda_ok(cudaMemsetAsync(gs->d_stats, 0, sizeof(GuessStats), stream()), "guess init");
}

// shift, then the features of p into x (normalised); returns the block count
bool features(GuessState *gs, const GGeom &g, const double *p, const double *rhs, float *x)
{
  const int64_t n = (int64_t)g.nx * g.ny * g.nz;
  const int nb = flat(n);
  k_g_sum_b<<<nb, kNT, 0, stream()>>>(g, rhs, gs->partial);
  if (!launched("k_g_sum_b")) return false;
  k_g_fold_shift<<<1, kNT, 0, stream()>>>(gs->partial, nb, n, gs->d_stats);
  if (!launched("k_g_fold_shift")) return false;
  int kb = 0;
  const dim3 grid = coarse_grid(g, kb);
  const int nbc = (int)(grid.x * grid.y * grid.z);
  k_g_coarse<true><<<grid, dim3(kGX, kGY), 0, stream()>>>(g, gpairs(g), p, rhs, gs->d_stats, x,
      gs->partial, kb);
  if (!launched("k_g_coarse")) return false;
  k_g_fold_features<<<1, kNT, 0, stream()>>>(gs->partial, nbc, gs->nc, gs->d_stats);
  if (!launched("k_g_fold_features")) return false;
  k_g_normalize<<<flat(gs->nc), 256, 0, stream()>>>(x, gs->nc, gs->d_stats);
  return launched("k_g_normalize");
}

}  // namespace

bool guess_before_solve(GuessState *gs, const Grid *grid, double *p, const double *rhs)
{
  if (!gs || (!gs->net && !gs->recording)) return true;
  gs->evaluated = false;
  if (!gs->recording && gs->skip_left > 0) {  // backed off: the plain warm start only
    gs->skip_left--;
    return true;
  }
  if (!ensure(gs, grid)) return false;
  const GGeom g = geom(grid);
  const int64_t padded = (int64_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
  float *x = gs->recording ? gs->rec_x : gs->x;
  if (!features(gs, g, p, rhs, x)) return false;
  if (gs->recording) {
    // the target needs p0 after the solve
    return cuda_ok(cudaMemcpyAsync(gs->aux, p, padded * sizeof(double), cudaMemcpyDeviceToDevice,
                       stream()),
        "keep p0");
  }
  const float *out = nullptr;
  if (!unet_infer(gs->net, x, g.nz / 2, g.ny / 2, g.nx / 2, &out)) return false;
  const int64_t n = (int64_t)g.nx * g.ny * g.nz;
  k_g_candidate<<<flat(n), 256, 0, stream()>>>(g, p, out, gs->d_stats, gs->aux);
  if (!launched("k_g_candidate")) return false;
  // the features' kernel and grid: the same summation order
  int kb = 0;
  const dim3 cgrid = coarse_grid(g, kb);
  const int nb = (int)(cgrid.x * cgrid.y * cgrid.z);
  k_g_coarse<false><<<cgrid, dim3(kGX, kGY), 0, stream()>>>(g, gpairs(g), gs->aux, rhs,
      gs->d_stats, nullptr, gs->partial, kb);
  if (!launched("k_g_coarse")) return false;
  k_g_fold_select<<<1, kNT, 0, stream()>>>(gs->partial, nb, gs->d_stats);
  if (!launched("k_g_fold_select")) return false;
  k_g_take<<<flat(padded), 256, 0, stream()>>>(p, gs->aux, padded, gs->d_stats);
  if (!launched("k_g_take")) return false;
  // the outcome reaches the host with the solve's own synchronisation
  gs->evaluated = true;
  return cuda_ok(cudaMemcpyAsync(gs->h_stats, gs->d_stats, sizeof(GuessStats),
                     cudaMemcpyDeviceToHost, stream()),
      "guess outcome");
}

bool guess_after_solve(GuessState *gs, const Grid *grid, const double *p)
{
  if (!gs) return true;
  if (gs->evaluated) {  // the solve has synchronised: h_stats holds this step's outcome
    gs->evaluated = false;
    gs->n_eval++;
    if (gs->h_stats->used) {
      gs->n_taken++;
      gs->rejections = 0;
    } else if (++gs->rejections >= 2 && gs->probe_every > 1) {
      gs->skip_left = gs->probe_every - 1;
    }
  }
  if (!gs->recording) return true;
  gs->recording = false;
  const GGeom g = geom(grid);
  k_g_target<<<flat(gs->nc), 256, 0, stream()>>>(g, p, gs->aux, gs->d_stats, gs->rec_t);
  return launched("k_g_target");
}

void guess_free(GuessState *gs)
{
  if (!gs) return;
  if (gs->x) cudaFree(gs->x);
  if (gs->aux) cudaFree(gs->aux);
  if (gs->partial) cudaFree(gs->partial);
  if (gs->d_stats) cudaFree(gs->d_stats);
  if (gs->h_stats) cudaFreeHost(gs->h_stats);
  delete gs;
}

namespace {

GuessState *guess_state_for(Solver *s)
{
  SolverState *ss = s ? solver_state(s) : nullptr;
  if (!ss || !ss->mg) {
    fail(NUSIF_ERR_STATE, "learned warm start: needs a solver initialised with mg or mg-mixed");
    return nullptr;
  }
  if (!ss->guess) {
    ss->guess = new GuessState();
    ss->guess->probe_every = ss->ext.mg_guess_probe > 1 ? ss->ext.mg_guess_probe : 1;
  }
  return ss->guess;
}

}  // namespace
}  // namespace nusif

using namespace nusif;

extern "C" {

int nusifSolverSetGuessNet(Solver *s, NusifUNet *net)
{
  GuessState *gs = guess_state_for(s);
  if (!gs) return NUSIF_ERR_STATE;
  gs->net = net;
  gs->rejections = gs->skip_left = 0;
  gs->n_eval = gs->n_taken = 0;
  return NUSIF_OK;
}

int nusifSolverGuessCounts(Solver *s, long long *evaluated, long long *taken)
{
  GuessState *gs = guess_state_for(s);
  if (!gs) return NUSIF_ERR_STATE;
  if (evaluated) *evaluated = gs->n_eval;
  if (taken) *taken = gs->n_taken;
  return NUSIF_OK;
}

int nusifSolverRecordPair(Solver *s, float *x, float *t)
{
  GuessState *gs = guess_state_for(s);
  if (!gs) return NUSIF_ERR_STATE;
  if (!x || !t) {
    fail(NUSIF_ERR_ARG, "nusifSolverRecordPair: null buffer");
    return NUSIF_ERR_ARG;
  }
  gs->rec_x = x;
  gs->rec_t = t;
  gs->recording = true;
  return NUSIF_OK;
}

int nusifSolverGuessStats(Solver *s, int *used, double *rel_warm, double *rel_guess)
{
  GuessState *gs = guess_state_for(s);
  if (!gs) return NUSIF_ERR_STATE;
  if (!gs->d_stats) {
    if (used) *used = 0;
    if (rel_warm) *rel_warm = 0.0;
    if (rel_guess) *rel_guess = 0.0;
    return NUSIF_OK;
  }
  if (!cuda_ok(cudaMemcpyAsync(gs->h_stats, gs->d_stats, sizeof(GuessStats), cudaMemcpyDeviceToHost,
                   stream()),
          "guess stats") ||
      !cuda_ok(cudaStreamSynchronize(stream()), "guess stats"))
    return NUSIF_ERR_CUDA;
  const GuessStats &h = *gs->h_stats;
  const double nb = h.bc2 > 0.0 ? h.bc2 : 1.0;
  if (used) *used = h.used;
  if (rel_warm) *rel_warm = sqrt(h.rc2 / nb);
  if (rel_guess) *rel_guess = sqrt(h.rc2_cand / nb);
  return NUSIF_OK;
}

}  // extern "C"
