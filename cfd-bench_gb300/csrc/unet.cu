// Learned pressure warm start: a 3-level 3D U-Net trained and run on the GPU
// with this file's kernels (no reference counterpart: the reference solver has
// no learned component).
//
// Network (volumes channels-last [B][Z][Y][X][C]; every conv 3x3x3 with zero
// padding; weights W[tap][cout][cin], tap = 9(dz+1) + 3(dy+1) + (dx+1)):
//   e0a 2->16, e0b 16->16 | pool | e1a 16->32, e1b 32->32 | pool | e2a 32->64
//   | up, concat [up(e2a), e1b] | d1a 96->32, d1b 32->32 | up, concat
//   [up(d1b), e0b] | d0a 48->16, d0b 16->16 | out 16->1 (linear, FP32).
// ReLU after every conv but the last; pool = 2x2x2 mean, up = nearest.
//
// Precision: BF16 weights and activations, FP32 accumulation (tensor cores),
// FP32 master weights, gradients and Adam state. A layer's output gradient
// times its ReLU mask is rounded to BF16 before the tensor-core kernels use it.
//
// Kernels:
//  - k_conv_tc (unet_tc.cu): the forward and input-gradient convolutions on
//    the 5th-generation tensor cores (tcgen05.mma, TMEM accumulators, TMA
//    staging) whenever the volume's rows tile into 128-cell blocks; the
//    decoder's upsampled concat source is then materialised by k_upsample.
//  - k_conv_mma: implicit-GEMM conv on the tensor cores (mma.sync m16n8k16
//    BF16 -> FP32): M = cells (16 per warp), N = output channels, K = 27 taps x
//    input channels in chunks of 16. Its loader reads up to two sources, the
//    first optionally at half resolution (nearest upsampling and the concat
//    of the decoder are never materialised). The same kernel computes input
//    gradients with tap-flipped, transposed weights.
//  - k_wgrad_mma: weight gradients as a GEMM over cells (M = cout, N = cin,
//    K = cells) on the tensor cores, one block per (chunk of cells, tap),
//    per-chunk partials folded in a fixed order (deterministic).
//  - plain FP32 kernels for the 2-channel input layer and the 1-channel output
//    layer, pooling, masks, the loss and Adam.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "nusif_internal.h"
#include "unet_internal.h"
#include "unet_tc.h"

namespace nusif {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kLayers = 10;
enum { L_E0A, L_E0B, L_E1A, L_E1B, L_E2A, L_D1A, L_D1B, L_D0A, L_D0B, L_OUT };
struct LayerDesc {
  int cin, cout;
};
constexpr LayerDesc kDesc[kLayers] = { { 2, 16 }, { 16, 16 }, { 16, 32 }, { 32, 32 }, { 32, 64 },
  { 96, 32 }, { 32, 32 }, { 48, 16 }, { 16, 16 }, { 16, 1 } };

// ------------------------------------------------------------------ device helpers

__device__ __forceinline__ uint32_t ld_pair(const bf16 *p)
{
  return *reinterpret_cast<const uint32_t *>(p);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ uint32_t pack_raw(bf16 lo, bf16 hi)
{
  const uint32_t a = *reinterpret_cast<const unsigned short *>(&lo);
  const uint32_t b = *reinterpret_cast<const unsigned short *>(&hi);
  return a | (b << 16);
}

// D += A(16x16, row) * B(16x8, col), BF16 inputs, FP32 accumulators
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
    uint32_t b1)
{
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct Vol {
  int B, Z, Y, X;
  __host__ __device__ int64_t cells() const { return (int64_t)B * Z * Y * X; }
};

__device__ __forceinline__ void decompose(const Vol &v, int64_t c, int &b, int &z, int &y, int &x)
{
  x = (int)(c % v.X);
  int64_t r = c / v.X;
  y = (int)(r % v.Y);
  r /= v.Y;
  z = (int)(r % v.Z);
  b = (int)(r / v.Z);
}

// ------------------------------------------------------------------ tensor-core conv

struct ConvSrc {
  const bf16 *p;
  int c;   // channels (multiple of 16)
  int up;  // 1: stored at half resolution, read by nearest upsampling
};

struct ConvArgs {
  ConvSrc s0, s1;   // s1.c == 0: one source
  Vol v;            // output (= full input) resolution
  const bf16 *w;    // [27][COUT][cin]
  const float *bias;
  int relu;
  void *out;        // bf16 or float [cells][COUT]
};

// One warp = 16 consecutive output cells x all COUT channels. Rows g and g+8
// of the mma fragments are this thread's two cells.
template <int COUT, bool OUT_BF16>
__global__ void __launch_bounds__(128) k_conv_mma(ConvArgs a)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int64_t ncell = a.v.cells();
  const int64_t base = ((int64_t)blockIdx.x * 4 + warp) * 16;
  if (base >= ncell) return;
  const int cin = a.s0.c + a.s1.c;
  int cb[2], cz[2], cy[2], cx[2];
  bool live[2];
  for (int r = 0; r < 2; r++) {
    const int64_t c = base + g + 8 * r;
    live[r] = c < ncell;
    decompose(a.v, live[r] ? c : 0, cb[r], cz[r], cy[r], cx[r]);
  }
  const int hZ = a.v.Z >> 1, hY = a.v.Y >> 1, hX = a.v.X >> 1;
  float acc[COUT / 8][4];
#pragma unroll
  for (int j = 0; j < COUT / 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
  for (int tap = 0; tap < 27; tap++) {
    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    bool ok[2];
    int64_t n1[2], n0[2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int z = cz[r] + dz, y = cy[r] + dy, x = cx[r] + dx;
      ok[r] = live[r] && z >= 0 && z < a.v.Z && y >= 0 && y < a.v.Y && x >= 0 && x < a.v.X;
      n1[r] = ok[r] ? (((int64_t)cb[r] * a.v.Z + z) * a.v.Y + y) * a.v.X + x : 0;
      n0[r] = !a.s0.up ? n1[r]
                       : (ok[r] ? (((int64_t)cb[r] * hZ + (z >> 1)) * hY + (y >> 1)) * hX + (x >> 1)
                                : 0);
    }
    const bf16 *wt = a.w + (int64_t)tap * COUT * cin;
    for (int kc = 0; kc < cin; kc += 16) {
      const bool first = kc < a.s0.c;
      const bf16 *src = first ? a.s0.p : a.s1.p;
      const int cs = first ? a.s0.c : a.s1.c;
      const int c0 = (first ? kc : kc - a.s0.c) + 2 * t;
      const int64_t o0 = (first ? n0[0] : n1[0]) * cs + c0;
      const int64_t o1 = (first ? n0[1] : n1[1]) * cs + c0;
      uint32_t A[4];
      A[0] = ok[0] ? ld_pair(src + o0) : 0u;
      A[1] = ok[1] ? ld_pair(src + o1) : 0u;
      A[2] = ok[0] ? ld_pair(src + o0 + 8) : 0u;
      A[3] = ok[1] ? ld_pair(src + o1 + 8) : 0u;
#pragma unroll
      for (int j = 0; j < COUT / 8; j++) {
        const bf16 *wr = wt + (int64_t)(8 * j + g) * cin + kc + 2 * t;
        mma_bf16(acc[j], A, __ldg(reinterpret_cast<const unsigned *>(wr)),
            __ldg(reinterpret_cast<const unsigned *>(wr + 8)));
      }
    }
  }
#pragma unroll
  for (int r = 0; r < 2; r++) {
    if (!live[r]) continue;
    const int64_t c = base + g + 8 * r;
#pragma unroll
    for (int j = 0; j < COUT / 8; j++) {
      const int co = 8 * j + 2 * t;
      float v0 = acc[j][2 * r], v1 = acc[j][2 * r + 1];
      if (a.bias) {
        v0 += a.bias[co];
        v1 += a.bias[co + 1];
      }
      if (a.relu) {
        v0 = fmaxf(v0, 0.0f);
        v1 = fmaxf(v1, 0.0f);
      }
      if (OUT_BF16)
        *reinterpret_cast<uint32_t *>(static_cast<bf16 *>(a.out) + c * COUT + co) = pack_bf16(v0, v1);
      else
        *reinterpret_cast<float2 *>(static_cast<float *>(a.out) + c * COUT + co) = make_float2(v0, v1);
    }
  }
}

// ------------------------------------------------------------------ tensor-core weight gradient

struct WgradArgs {
  ConvSrc s0, s1;  // the layer's input, as in the forward pass
  const bf16 *g;   // masked output gradient [cells][COUT]
  Vol v;
  int64_t chunk;   // cells per block (multiple of 64)
  float *partial;  // [chunks][27][COUT][CIN]
};

// dW[tap][co][ci] = sum over cells of G[cell][co] * X[cell + off(tap)][ci]:
// A = G^T (co x cells), B = shifted X (cells x ci); 64-cell tiles staged in
// shared memory, fragments assembled from 16-bit shared loads.
template <int COUT, int CIN>
__global__ void __launch_bounds__(128) k_wgrad_mma(WgradArgs a)
{
  constexpr int kT = 64;
  constexpr int MT = COUT / 16, NT = CIN / 8, TILES = MT * NT, TPW = (TILES + 3) / 4;
  constexpr int GP = COUT + 2, XP = CIN + 2;  // padded rows (16-bit elements)
  __shared__ bf16 gs[kT][GP];
  __shared__ bf16 xs[kT][XP];
  const int tap = blockIdx.y;
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int64_t ncell = a.v.cells();
  const int64_t c_begin = blockIdx.x * a.chunk;
  const int64_t c_end = min(c_begin + a.chunk, ncell);
  const int hZ = a.v.Z >> 1, hY = a.v.Y >> 1, hX = a.v.X >> 1;
  float acc[TPW][4];
#pragma unroll
  for (int q = 0; q < TPW; q++) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.0f;
  for (int64_t c0 = c_begin; c0 < c_end; c0 += kT) {
    // stage G rows and the tap-shifted input rows of 64 cells
    for (int e = threadIdx.x; e < kT * (COUT / 2); e += blockDim.x) {
      const int r = e / (COUT / 2), k = 2 * (e % (COUT / 2));
      const int64_t c = c0 + r;
      uint32_t v = 0;
      if (c < c_end) v = ld_pair(a.g + c * COUT + k);
      *reinterpret_cast<uint32_t *>(&gs[r][k]) = v;
    }
    for (int e = threadIdx.x; e < kT * (CIN / 2); e += blockDim.x) {
      const int r = e / (CIN / 2), k = 2 * (e % (CIN / 2));
      const int64_t c = c0 + r;
      uint32_t v = 0;
      if (c < c_end) {
        int b, z, y, x;
        decompose(a.v, c, b, z, y, x);
        z += dz;
        y += dy;
        x += dx;
        if (z >= 0 && z < a.v.Z && y >= 0 && y < a.v.Y && x >= 0 && x < a.v.X) {
          if (k < a.s0.c) {
            const int64_t n = a.s0.up ? (((int64_t)b * hZ + (z >> 1)) * hY + (y >> 1)) * hX + (x >> 1)
                                      : (((int64_t)b * a.v.Z + z) * a.v.Y + y) * a.v.X + x;
            v = ld_pair(a.s0.p + n * a.s0.c + k);
          } else {
            const int64_t n = (((int64_t)b * a.v.Z + z) * a.v.Y + y) * a.v.X + x;
            v = ld_pair(a.s1.p + n * a.s1.c + (k - a.s0.c));
          }
        }
      }
      *reinterpret_cast<uint32_t *>(&xs[r][k]) = v;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < kT; ks += 16) {
#pragma unroll
      for (int q = 0; q < TPW; q++) {
        const int tile = warp + 4 * q;
        if (tile >= TILES) break;
        const int m0 = (tile / NT) * 16, n0 = (tile % NT) * 8;
        const int k0 = ks + 2 * t;
        uint32_t A[4];
        A[0] = pack_raw(gs[k0][m0 + g], gs[k0 + 1][m0 + g]);
        A[1] = pack_raw(gs[k0][m0 + g + 8], gs[k0 + 1][m0 + g + 8]);
        A[2] = pack_raw(gs[k0 + 8][m0 + g], gs[k0 + 9][m0 + g]);
        A[3] = pack_raw(gs[k0 + 8][m0 + g + 8], gs[k0 + 9][m0 + g + 8]);
        const uint32_t b0 = pack_raw(xs[k0][n0 + g], xs[k0 + 1][n0 + g]);
        const uint32_t b1 = pack_raw(xs[k0 + 8][n0 + g], xs[k0 + 9][n0 + g]);
        mma_bf16(acc[q], A, b0, b1);
      }
    }
    __syncthreads();
  }
  float *out = a.partial + ((int64_t)blockIdx.x * 27 + tap) * COUT * CIN;
#pragma unroll
  for (int q = 0; q < TPW; q++) {
    const int tile = warp + 4 * q;
    if (tile >= TILES) break;
    const int m0 = (tile / NT) * 16, n0 = (tile % NT) * 8;
    out[(m0 + g) * CIN + n0 + 2 * t] = acc[q][0];
    out[(m0 + g) * CIN + n0 + 2 * t + 1] = acc[q][1];
    out[(m0 + g + 8) * CIN + n0 + 2 * t] = acc[q][2];
    out[(m0 + g + 8) * CIN + n0 + 2 * t + 1] = acc[q][3];
  }
}

// dst[i] = sum over chunks of partial[chunk][i] (fixed order)
__global__ void k_fold_chunks(const float *__restrict__ partial, int chunks, int n,
    float *__restrict__ dst)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int c = 0; c < chunks; c++) s += partial[(int64_t)c * n + i];
  dst[i] = s;
}

// per-channel sums of a [cells][C] BF16 gradient: block partials (fixed order)
template <int C>
__global__ void __launch_bounds__(256) k_channel_sum(const bf16 *__restrict__ g, int64_t ncell,
    int64_t chunk, float *__restrict__ partial)
{
  constexpr int R = 256 / C;  // cells in flight per block step
  __shared__ float sm[256];
  const int ch = threadIdx.x % C, row = threadIdx.x / C;
  const int64_t c_begin = blockIdx.x * chunk, c_end = min(c_begin + chunk, ncell);
  float s = 0.0f;
  for (int64_t c = c_begin + row; c < c_end; c += R) s += __bfloat162float(g[c * C + ch]);
  sm[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < C) {
    float tot = 0.0f;
    for (int r = 0; r < R; r++) tot += sm[r * C + threadIdx.x];
    partial[(int64_t)blockIdx.x * C + threadIdx.x] = tot;
  }
}

// same for an FP32 [cells] gradient (the output layer's bias)
__global__ void __launch_bounds__(256) k_scalar_sum(const float *__restrict__ g, int64_t ncell,
    int64_t chunk, float *__restrict__ partial)
{
  __shared__ float sm[256];
  const int64_t c_begin = blockIdx.x * chunk, c_end = min(c_begin + chunk, ncell);
  float s = 0.0f;
  for (int64_t c = c_begin + threadIdx.x; c < c_end; c += 256) s += g[c];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

// ------------------------------------------------------------------ plain layers

// e0a: 2 -> 16, ReLU (FP32 arithmetic on BF16 values)
__global__ void __launch_bounds__(256) k_conv_first(const bf16 *__restrict__ x, Vol v,
    const bf16 *__restrict__ w, const float *__restrict__ bias, bf16 *__restrict__ y)
{
  __shared__ float ws[27 * 16 * 2];
  for (int i = threadIdx.x; i < 27 * 32; i += blockDim.x) ws[i] = __bfloat162float(w[i]);
  __syncthreads();
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= v.cells()) return;
  int b, z, yy, xx;
  decompose(v, c, b, z, yy, xx);
  float acc[16];
#pragma unroll
  for (int o = 0; o < 16; o++) acc[o] = bias[o];
  for (int tap = 0; tap < 27; tap++) {
    const int nz = z + tap / 9 - 1, ny = yy + (tap / 3) % 3 - 1, nx = xx + tap % 3 - 1;
    if (nz < 0 || nz >= v.Z || ny < 0 || ny >= v.Y || nx < 0 || nx >= v.X) continue;
    const int64_t n = (((int64_t)b * v.Z + nz) * v.Y + ny) * v.X + nx;
    const float x0 = __bfloat162float(x[2 * n]), x1 = __bfloat162float(x[2 * n + 1]);
#pragma unroll
    for (int o = 0; o < 16; o++) acc[o] += ws[(tap * 16 + o) * 2] * x0 + ws[(tap * 16 + o) * 2 + 1] * x1;
  }
#pragma unroll
  for (int o = 0; o < 16; o += 2)
    *reinterpret_cast<uint32_t *>(y + c * 16 + o) =
        pack_bf16(fmaxf(acc[o], 0.0f), fmaxf(acc[o + 1], 0.0f));
}

// out: 16 -> 1, linear, FP32 output
__global__ void __launch_bounds__(256) k_conv_last(const bf16 *__restrict__ x, Vol v,
    const bf16 *__restrict__ w, const float *__restrict__ bias, float *__restrict__ y)
{
  __shared__ float ws[27 * 16];
  for (int i = threadIdx.x; i < 27 * 16; i += blockDim.x) ws[i] = __bfloat162float(w[i]);
  __syncthreads();
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= v.cells()) return;
  int b, z, yy, xx;
  decompose(v, c, b, z, yy, xx);
  float acc = bias[0];
  for (int tap = 0; tap < 27; tap++) {
    const int nz = z + tap / 9 - 1, ny = yy + (tap / 3) % 3 - 1, nx = xx + tap % 3 - 1;
    if (nz < 0 || nz >= v.Z || ny < 0 || ny >= v.Y || nx < 0 || nx >= v.X) continue;
    const bf16 *xn = x + ((((int64_t)b * v.Z + nz) * v.Y + ny) * v.X + nx) * 16;
#pragma unroll
    for (int i = 0; i < 16; i++) acc += ws[tap * 16 + i] * __bfloat162float(xn[i]);
  }
  y[c] = acc;
}

// input gradient of the output layer: dX[c][i] = sum_tap dout[c - off] W[tap][i]
__global__ void __launch_bounds__(256) k_conv_last_dgrad(const float *__restrict__ dout, Vol v,
    const bf16 *__restrict__ w, float *__restrict__ dx)
{
  __shared__ float ws[27 * 16];
  for (int i = threadIdx.x; i < 27 * 16; i += blockDim.x) ws[i] = __bfloat162float(w[i]);
  __syncthreads();
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= v.cells()) return;
  int b, z, yy, xx;
  decompose(v, c, b, z, yy, xx);
  float acc[16];
#pragma unroll
  for (int i = 0; i < 16; i++) acc[i] = 0.0f;
  for (int tap = 0; tap < 27; tap++) {
    const int nz = z - (tap / 9 - 1), ny = yy - ((tap / 3) % 3 - 1), nx = xx - (tap % 3 - 1);
    if (nz < 0 || nz >= v.Z || ny < 0 || ny >= v.Y || nx < 0 || nx >= v.X) continue;
    const float d = dout[(((int64_t)b * v.Z + nz) * v.Y + ny) * v.X + nx];
#pragma unroll
    for (int i = 0; i < 16; i++) acc[i] += d * ws[tap * 16 + i];
  }
#pragma unroll
  for (int i = 0; i < 16; i += 2)
    *reinterpret_cast<float2 *>(dx + c * 16 + i) = make_float2(acc[i], acc[i + 1]);
}

// weight gradients of the plain layers, one block per (chunk, tap):
// partial[chunk][tap][co][ci] = sum over the chunk of G[c][co] * X[c + off][ci]
template <int CO, int CI, bool G_BF16>
__global__ void __launch_bounds__(256) k_wgrad_plain(const void *g_, const bf16 *__restrict__ x,
    Vol v, int64_t chunk, float *__restrict__ partial)
{
  constexpr int N = CO * CI;
  __shared__ float sm[256];
  const int tap = blockIdx.y;
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const int64_t ncell = v.cells();
  const int64_t c_begin = blockIdx.x * chunk, c_end = min(c_begin + chunk, ncell);
  float acc[N];
#pragma unroll
  for (int i = 0; i < N; i++) acc[i] = 0.0f;
  for (int64_t c = c_begin + threadIdx.x; c < c_end; c += 256) {
    int b, z, y, xx;
    decompose(v, c, b, z, y, xx);
    z += dz;
    y += dy;
    xx += dx;
    if (z < 0 || z >= v.Z || y < 0 || y >= v.Y || xx < 0 || xx >= v.X) continue;
    const int64_t n = (((int64_t)b * v.Z + z) * v.Y + y) * v.X + xx;
    float gv[CO], xv[CI];
#pragma unroll
    for (int o = 0; o < CO; o++)
      gv[o] = G_BF16 ? __bfloat162float(static_cast<const bf16 *>(g_)[c * CO + o])
                     : static_cast<const float *>(g_)[c * CO + o];
#pragma unroll
    for (int i = 0; i < CI; i++) xv[i] = __bfloat162float(x[n * CI + i]);
#pragma unroll
    for (int o = 0; o < CO; o++)
#pragma unroll
      for (int i = 0; i < CI; i++) acc[o * CI + i] += gv[o] * xv[i];
  }
  float *out = partial + ((int64_t)blockIdx.x * 27 + tap) * N;
  for (int i = 0; i < N; i++) {
    sm[threadIdx.x] = acc[i];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[i] = sm[0];
    __syncthreads();
  }
}

// ------------------------------------------------------------------ elementwise

// the 2-channel FP32 input as BF16, once as [cells][2] (the first layer's
// weight gradient) and once zero-padded to [cells][16] (the tensor-core
// first layer: K must be a multiple of 16)
__global__ void k_input_bf16(const float *__restrict__ x, int64_t n, bf16 *__restrict__ x2,
    bf16 *__restrict__ x16)
{
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = reinterpret_cast<const float2 *>(x)[c];
    const uint32_t v = pack_bf16(a.x, a.y);
    reinterpret_cast<uint32_t *>(x2)[c] = v;
    uint4 *o = reinterpret_cast<uint4 *>(x16 + c * 16);
    o[0] = make_uint4(v, 0u, 0u, 0u);
    o[1] = make_uint4(0u, 0u, 0u, 0u);
  }
}

// W[27][co][ci] (FP32) -> BF16 [27][16][16], zero outside co x ci (the first
// and last layers on the tensor cores)
__global__ void k_pad_weights16(const float *__restrict__ w, int co, int ci, bf16 *__restrict__ wp)
{
  const int n = 27 * 16 * 16;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int tap = i / 256, o = (i / 16) % 16, k = i % 16;
    wp[i] = __float2bfloat16_rn(o < co && k < ci ? w[(tap * co + o) * ci + k] : 0.0f);
  }
}

// nearest upsampling of a [half cells][C] BF16 volume to full resolution, 8
// channels (16 bytes) per thread
__global__ void k_upsample(const bf16 *__restrict__ c, Vol fv, int C, bf16 *__restrict__ f)
{
  const int g8 = C / 8;
  const int64_t n = fv.cells() * g8;
  const int hZ = fv.Z / 2, hY = fv.Y / 2, hX = fv.X / 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int grp = (int)(i % g8);
    int b, z, y, x;
    decompose(fv, i / g8, b, z, y, x);
    const int64_t cc = (((int64_t)b * hZ + (z >> 1)) * hY + (y >> 1)) * hX + (x >> 1);
    reinterpret_cast<uint4 *>(f)[i] = reinterpret_cast<const uint4 *>(c)[cc * g8 + grp];
  }
}

// G = bf16(dY * (Y > 0))
__global__ void k_relu_mask(const float *__restrict__ dy, const bf16 *__restrict__ y, int64_t n,
    bf16 *__restrict__ g)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    g[i] = __float2bfloat16_rn(__bfloat162float(y[i]) > 0.0f ? dy[i] : 0.0f);
}

// 2x2x2 mean of a [fine cells][C] BF16 volume; one thread per (coarse cell, channel)
__global__ void k_pool(const bf16 *__restrict__ f, Vol fv, int C, bf16 *__restrict__ o)
{
  const Vol cv = { fv.B, fv.Z / 2, fv.Y / 2, fv.X / 2 };
  const int64_t n = cv.cells() * C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int ch = (int)(i % C);
    int b, z, y, x;
    decompose(cv, i / C, b, z, y, x);
    float s = 0.0f;
    for (int q = 0; q < 8; q++) {
      const int64_t fc = (((int64_t)b * fv.Z + 2 * z + (q >> 2)) * fv.Y + 2 * y + ((q >> 1) & 1)) * fv.X +
                         2 * x + (q & 1);
      s += __bfloat162float(f[fc * C + ch]);
    }
    o[i] = __float2bfloat16_rn(s * 0.125f);
  }
}

// fine gradient += coarse gradient / 8 (adjoint of the mean pool)
__global__ void k_pool_back_add(const float *__restrict__ gc, Vol fv, int C, float *__restrict__ gf)
{
  const int64_t n = fv.cells() * C;
  const Vol cv = { fv.B, fv.Z / 2, fv.Y / 2, fv.X / 2 };
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int ch = (int)(i % C);
    int b, z, y, x;
    decompose(fv, i / C, b, z, y, x);
    const int64_t cc = (((int64_t)b * cv.Z + z / 2) * cv.Y + y / 2) * cv.X + x / 2;
    gf[i] += 0.125f * gc[cc * C + ch];
  }
}

// split the gradient of a concat [up(coarse) Cu, skip Cs] at fine resolution:
// skip part copied out, upsampled part summed over the 8 children (adjoint of
// nearest upsampling)
__global__ void k_split_concat(const float *__restrict__ dcat, Vol fv, int Cu, int Cs,
    float *__restrict__ dskip, float *__restrict__ dcoarse)
{
  const int C = Cu + Cs;
  const int64_t nskip = fv.cells() * Cs;
  const Vol cv = { fv.B, fv.Z / 2, fv.Y / 2, fv.X / 2 };
  const int64_t nup = cv.cells() * Cu;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nskip + nup;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i < nskip) {
      const int64_t c = i / Cs;
      dskip[i] = dcat[c * C + Cu + (i % Cs)];
    } else {
      const int64_t k = i - nskip;
      const int ch = (int)(k % Cu);
      int b, z, y, x;
      decompose(cv, k / Cu, b, z, y, x);
      float s = 0.0f;
      for (int q = 0; q < 8; q++) {
        const int64_t fc = (((int64_t)b * fv.Z + 2 * z + (q >> 2)) * fv.Y + 2 * y + ((q >> 1) & 1)) *
                               fv.X + 2 * x + (q & 1);
        s += dcat[fc * C + ch];
      }
      dcoarse[k] = s;
    }
  }
}

// squared error partial sums and the loss gradient 2 (out - t) / n
__global__ void __launch_bounds__(256) k_mse(const float *__restrict__ out,
    const float *__restrict__ tgt, int64_t n, int64_t chunk, float *__restrict__ dout,
    double *__restrict__ partial)
{
  __shared__ double sm[256];
  const int64_t c_begin = blockIdx.x * chunk, c_end = min(c_begin + chunk, n);
  const float inv = 2.0f / (float)n;
  double s = 0.0;
  for (int64_t i = c_begin + threadIdx.x; i < c_end; i += 256) {
    const float d = out[i] - tgt[i];
    s += (double)d * d;
    if (dout) dout[i] = inv * d;
  }
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

__global__ void k_fold_loss(const double *__restrict__ partial, int nb, int64_t n, float *loss)
{
  double s = 0.0;
  for (int i = 0; i < nb; i++) s += partial[i];
  *loss = (float)(s / (double)n);
}

__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
    float *__restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1, float c2)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// BF16 copies of one layer's weights: W[tap][co][ci] and, for input gradients,
// the tap-flipped transpose Wt[tap][ci][co] = W[26 - tap][co][ci]
__global__ void k_layer_bf16(const float *__restrict__ w, int co, int ci, bf16 *__restrict__ wb,
    bf16 *__restrict__ wt)
{
  const int n = 27 * co * ci;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    wb[i] = __float2bfloat16_rn(w[i]);
    if (wt) {
      const int tap = i / (co * ci), r = i % (co * ci), o = r / ci, k = r % ci;
      wt[((26 - tap) * ci + k) * co + o] = __float2bfloat16_rn(w[i]);
    }
  }
}

int blocks_for(int64_t n, int threads = 256)
{
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace

// ------------------------------------------------------------------ host side

struct UNetState {
  int64_t w_off[kLayers], b_off[kLayers];
  int64_t nparam = 0;
  float *master = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;  // device FP32
  bf16 *wb[kLayers] = {}, *wt[kLayers] = {};
  int adam_t = 0;
  // workspace for the current volume
  Vol vol = { 0, 0, 0, 0 };
  int64_t cap0 = 0;  // level-0 cells the workspace holds
  bf16 *x = nullptr, *e0a = nullptr, *e0b = nullptr, *p0 = nullptr, *e1a = nullptr,
       *e1b = nullptr, *p1 = nullptr, *e2a = nullptr, *d1a = nullptr, *d1b = nullptr,
       *d0a = nullptr, *d0b = nullptr, *G = nullptr;
  float *out = nullptr, *dout = nullptr, *F1 = nullptr, *F2 = nullptr, *Fe0b = nullptr,
        *Fe1b = nullptr, *partial = nullptr;
  int64_t partial_cap = 0;
  bf16 *up1 = nullptr, *up0 = nullptr;  // materialised up(e2a) [n1][64], up(d1b) [n0][32]
  bf16 *x16 = nullptr;                  // input zero-padded to 16 channels
  bf16 *w_first16 = nullptr, *w_last16 = nullptr;  // e0a and out weights padded to [27][16][16]
  int *err = nullptr;                   // device: a tensor-core kernel's wait timed out
  int use_tc = 1;                       // tcgen05 kernels where the volume allows
  double *loss_partial = nullptr;
  float *loss = nullptr;  // device scalar
  std::vector<void *> ws;
};

namespace {

template <typename T>
bool dalloc(UNetState *u, T **p, int64_t n)
{
  if (!cuda_ok(cudaMalloc(reinterpret_cast<void **>(p), (size_t)n * sizeof(T)), "cudaMalloc(unet)"))
    return false;
  u->ws.push_back(*p);
  return true;
}

void free_workspace(UNetState *u)
{
  for (void *p : u->ws) cudaFree(p);
  u->ws.clear();
  u->cap0 = 0;
}

bool ensure_workspace(UNetState *u, const Vol &v)
{
  if (v.Z % 4 || v.Y % 4 || v.X % 4 || v.B < 1 || v.Z < 4 || v.Y < 4 || v.X < 4) {
    fail(NUSIF_ERR_ARG, "unet: volume %dx%dx%d (batch %d) needs every edge a multiple of 4", v.X,
        v.Y, v.Z, v.B);
    return false;
  }
  u->vol = v;
  const int64_t n0 = v.cells();
  if (n0 <= u->cap0) return true;
  cudaStreamSynchronize(stream());
  free_workspace(u);
  const int64_t n1 = n0 / 8, n2 = n0 / 64;
  bool ok = dalloc(u, &u->x, 2 * n0) && dalloc(u, &u->e0a, 16 * n0) && dalloc(u, &u->e0b, 16 * n0) &&
            dalloc(u, &u->p0, 16 * n1) && dalloc(u, &u->e1a, 32 * n1) && dalloc(u, &u->e1b, 32 * n1) &&
            dalloc(u, &u->p1, 32 * n2) && dalloc(u, &u->e2a, 64 * n2) && dalloc(u, &u->d1a, 32 * n1) &&
            dalloc(u, &u->d1b, 32 * n1) && dalloc(u, &u->d0a, 16 * n0) && dalloc(u, &u->d0b, 16 * n0) &&
            dalloc(u, &u->G, 16 * n0) && dalloc(u, &u->out, n0) && dalloc(u, &u->dout, n0) &&
            dalloc(u, &u->F1, 48 * n0) && dalloc(u, &u->F2, 16 * n0) && dalloc(u, &u->Fe0b, 16 * n0) &&
            dalloc(u, &u->Fe1b, 32 * n1) && dalloc(u, &u->loss_partial, 1024) &&
            dalloc(u, &u->up1, 64 * n1) && dalloc(u, &u->up0, 32 * n0) &&
            dalloc(u, &u->x16, 16 * n0);
  if (!ok) return false;
  u->cap0 = n0;
  return true;
}

bool ensure_partial(UNetState *u, int64_t n)
{
  if (n <= u->partial_cap) return true;
  cudaStreamSynchronize(stream());
  if (u->partial) cudaFree(u->partial);
  u->partial = nullptr;
  u->partial_cap = 0;
  if (!cuda_ok(cudaMalloc(&u->partial, (size_t)n * sizeof(float)), "cudaMalloc(unet partial)"))
    return false;
  u->partial_cap = n;
  return true;
}

// cells per block of the weight-gradient kernels: at most 256 chunks
int64_t wgrad_chunk(int64_t ncell)
{
  int64_t c = (ncell + 255) / 256;
  c = (c + 63) / 64 * 64;
  return c < 64 ? 64 : c;
}

template <int COUT, bool OUT_BF16>
bool conv_mma(const ConvSrc &s0, const ConvSrc &s1, const Vol &v, const bf16 *w, const float *bias,
    int relu, void *out)
{
  ConvArgs a;
  a.s0 = s0;
  a.s1 = s1;
  a.v = v;
  a.w = w;
  a.bias = bias;
  a.relu = relu;
  a.out = out;
  const int64_t warps = (v.cells() + 15) / 16;
  k_conv_mma<COUT, OUT_BF16><<<(unsigned)((warps + 3) / 4), 128, 0, stream()>>>(a);
  return launched("k_conv_mma");
}

bool tc_ok(const UNetState *u, const Vol &v, int n, int c0, int c1)
{
  return u->use_tc && tc_conv_supported(v.X, v.Y, v.Z, v.B, n, c0, c1);
}

// forward conv of a tensor-core layer (BF16 out, bias, ReLU)
bool fwd(UNetState *u, int l, const ConvSrc &s0, const ConvSrc &s1, const Vol &v, bf16 *out)
{
  const float *bias = u->master + u->b_off[l];
  if (tc_ok(u, v, kDesc[l].cout, s0.c, s1.c)) {
    const bf16 *a0 = s0.p;
    if (s0.up) {  // the decoder's upsampled source, materialised at full resolution
      bf16 *dst = s0.c == 64 ? u->up1 : u->up0;
      k_upsample<<<blocks_for(v.cells() * (s0.c / 8)), 256, 0, stream()>>>(s0.p, v, s0.c, dst);
      if (!launched("k_upsample")) return false;
      a0 = dst;
    }
    return tc_conv(a0, s0.c, s1.p, s1.c, v.B, v.Z, v.Y, v.X, u->wb[l], kDesc[l].cout, bias, 1, true,
        out, u->err);
  }
  switch (kDesc[l].cout) {
  case 16: return conv_mma<16, true>(s0, s1, v, u->wb[l], bias, 1, out);
  case 32: return conv_mma<32, true>(s0, s1, v, u->wb[l], bias, 1, out);
  case 64: return conv_mma<64, true>(s0, s1, v, u->wb[l], bias, 1, out);
  }
  fail(NUSIF_ERR_STATE, "unet: no forward kernel for %d output channels", kDesc[l].cout);
  return false;
}

// input gradient of a tensor-core layer: G (cout channels) -> FP32 [cells][cin]
bool dgrad(UNetState *u, int l, const Vol &v, float *dx)
{
  const ConvSrc g = { u->G, kDesc[l].cout, 0 };
  const ConvSrc none = { nullptr, 0, 0 };
  if (tc_ok(u, v, kDesc[l].cin, kDesc[l].cout, 0))
    return tc_conv(u->G, kDesc[l].cout, nullptr, 0, v.B, v.Z, v.Y, v.X, u->wt[l], kDesc[l].cin,
        nullptr, 0, false, dx, u->err);
  switch (kDesc[l].cin) {
  case 16: return conv_mma<16, false>(g, none, v, u->wt[l], nullptr, 0, dx);
  case 32: return conv_mma<32, false>(g, none, v, u->wt[l], nullptr, 0, dx);
  case 48: return conv_mma<48, false>(g, none, v, u->wt[l], nullptr, 0, dx);
  case 96: return conv_mma<96, false>(g, none, v, u->wt[l], nullptr, 0, dx);
  }
  fail(NUSIF_ERR_STATE, "unet: no input-gradient kernel for %d channels", kDesc[l].cin);
  return false;
}

template <int COUT, int CIN>
bool wgrad_launch(const WgradArgs &a, int chunks)
{
  k_wgrad_mma<COUT, CIN><<<dim3(chunks, 27), 128, 0, stream()>>>(a);
  return launched("k_wgrad_mma");
}

// weight and bias gradients of a tensor-core layer from G and its input
bool wgrad(UNetState *u, int l, const ConvSrc &s0, const ConvSrc &s1, const Vol &v)
{
  const int co = kDesc[l].cout, ci = kDesc[l].cin;
  const int64_t n = v.cells(), chunk = wgrad_chunk(n);
  const int chunks = (int)((n + chunk - 1) / chunk);
  if (!ensure_partial(u, (int64_t)chunks * 27 * co * ci)) return false;
  WgradArgs a;
  a.s0 = s0;
  a.s1 = s1;
  a.g = u->G;
  a.v = v;
  a.chunk = chunk;
  a.partial = u->partial;
  bool ok = false;
  if (co == 16 && ci == 16) ok = wgrad_launch<16, 16>(a, chunks);
  else if (co == 32 && ci == 16) ok = wgrad_launch<32, 16>(a, chunks);
  else if (co == 32 && ci == 32) ok = wgrad_launch<32, 32>(a, chunks);
  else if (co == 64 && ci == 32) ok = wgrad_launch<64, 32>(a, chunks);
  else if (co == 32 && ci == 96) ok = wgrad_launch<32, 96>(a, chunks);
  else if (co == 16 && ci == 48) ok = wgrad_launch<16, 48>(a, chunks);
  else fail(NUSIF_ERR_STATE, "unet: no weight-gradient kernel for %dx%d", co, ci);
  if (!ok) return false;
  const int nw = 27 * co * ci;
  k_fold_chunks<<<(nw + 255) / 256, 256, 0, stream()>>>(u->partial, chunks, nw, u->grad + u->w_off[l]);
  if (!launched("k_fold_chunks")) return false;
  // bias: per-channel sums of G (partials after the weight partials are folded)
  const int64_t bchunk = (n + 1023) / 1024 * 4 < 256 ? 256 : (n + 1023) / 1024 * 4;
  const int bblocks = (int)((n + bchunk - 1) / bchunk);
  if (!ensure_partial(u, (int64_t)bblocks * co)) return false;
  switch (co) {
  case 16: k_channel_sum<16><<<bblocks, 256, 0, stream()>>>(u->G, n, bchunk, u->partial); break;
  case 32: k_channel_sum<32><<<bblocks, 256, 0, stream()>>>(u->G, n, bchunk, u->partial); break;
  case 64: k_channel_sum<64><<<bblocks, 256, 0, stream()>>>(u->G, n, bchunk, u->partial); break;
  default: fail(NUSIF_ERR_STATE, "unet: no bias-gradient kernel for %d channels", co); return false;
  }
  if (!launched("k_channel_sum")) return false;
  k_fold_chunks<<<1, 64, 0, stream()>>>(u->partial, bblocks, co, u->grad + u->b_off[l]);
  return launched("k_fold_chunks");
}

bool mask(const float *dy, const bf16 *y, int64_t n, bf16 *g)
{
  k_relu_mask<<<blocks_for(n), 256, 0, stream()>>>(dy, y, n, g);
  return launched("k_relu_mask");
}

bool pool_back(const float *gc, const Vol &fv, int C, float *gf)
{
  k_pool_back_add<<<blocks_for(fv.cells() * C), 256, 0, stream()>>>(gc, fv, C, gf);
  return launched("k_pool_back_add");
}

bool split(const float *dcat, const Vol &fv, int Cu, int Cs, float *dskip, float *dcoarse)
{
  const int64_t n = fv.cells() * Cs + fv.cells() / 8 * Cu;
  k_split_concat<<<blocks_for(n), 256, 0, stream()>>>(dcat, fv, Cu, Cs, dskip, dcoarse);
  return launched("k_split_concat");
}

Vol half(const Vol &v) { return { v.B, v.Z / 2, v.Y / 2, v.X / 2 }; }

bool refresh_bf16(UNetState *u)
{
  for (int l = 0; l < kLayers; l++) {
    const int n = 27 * kDesc[l].cout * kDesc[l].cin;
    k_layer_bf16<<<(n + 255) / 256, 256, 0, stream()>>>(u->master + u->w_off[l], kDesc[l].cout,
        kDesc[l].cin, u->wb[l], u->wt[l]);
    if (!launched("k_layer_bf16")) return false;
  }
  k_pad_weights16<<<27, 256, 0, stream()>>>(u->master + u->w_off[L_E0A], 16, 2, u->w_first16);
  if (!launched("k_pad_weights16")) return false;
  k_pad_weights16<<<27, 256, 0, stream()>>>(u->master + u->w_off[L_OUT], 1, 16, u->w_last16);
  return launched("k_pad_weights16");
}

}  // namespace

// forward pass on the workspace input u->x (BF16) -> u->out (FP32)
bool unet_forward(UNetState *u)
{
  const Vol v0 = u->vol, v1 = half(v0), v2 = half(v1);
  const int64_t n0 = v0.cells();
  const ConvSrc none = { nullptr, 0, 0 };
  if (tc_ok(u, v0, 16, 16, 0)) {
    if (!tc_conv(u->x16, 16, nullptr, 0, v0.B, v0.Z, v0.Y, v0.X, u->w_first16, 16,
            u->master + u->b_off[L_E0A], 1, true, u->e0a, u->err))
      return false;
  } else {
    k_conv_first<<<(unsigned)((n0 + 255) / 256), 256, 0, stream()>>>(u->x, v0, u->wb[L_E0A],
        u->master + u->b_off[L_E0A], u->e0a);
    if (!launched("k_conv_first")) return false;
  }
  if (!fwd(u, L_E0B, { u->e0a, 16, 0 }, none, v0, u->e0b)) return false;
  k_pool<<<blocks_for(v1.cells() * 16), 256, 0, stream()>>>(u->e0b, v0, 16, u->p0);
  if (!launched("k_pool")) return false;
  if (!fwd(u, L_E1A, { u->p0, 16, 0 }, none, v1, u->e1a)) return false;
  if (!fwd(u, L_E1B, { u->e1a, 32, 0 }, none, v1, u->e1b)) return false;
  k_pool<<<blocks_for(v2.cells() * 32), 256, 0, stream()>>>(u->e1b, v1, 32, u->p1);
  if (!launched("k_pool")) return false;
  if (!fwd(u, L_E2A, { u->p1, 32, 0 }, none, v2, u->e2a)) return false;
  if (!fwd(u, L_D1A, { u->e2a, 64, 1 }, { u->e1b, 32, 0 }, v1, u->d1a)) return false;
  if (!fwd(u, L_D1B, { u->d1a, 32, 0 }, none, v1, u->d1b)) return false;
  if (!fwd(u, L_D0A, { u->d1b, 32, 1 }, { u->e0b, 16, 0 }, v0, u->d0a)) return false;
  if (!fwd(u, L_D0B, { u->d0a, 16, 0 }, none, v0, u->d0b)) return false;
  if (tc_ok(u, v0, 16, 16, 0))
    return tc_conv(u->d0b, 16, nullptr, 0, v0.B, v0.Z, v0.Y, v0.X, u->w_last16, 16,
        u->master + u->b_off[L_OUT], 0, false, u->out, u->err, 1);
  k_conv_last<<<(unsigned)((n0 + 255) / 256), 256, 0, stream()>>>(u->d0b, v0, u->wb[L_OUT],
      u->master + u->b_off[L_OUT], u->out);
  return launched("k_conv_last");
}

namespace {

// plain-layer weight gradients: out layer (dout FP32 x d0b) and e0a (G x input)
bool wgrad_out(UNetState *u, const Vol &v)
{
  const int64_t n = v.cells(), chunk = wgrad_chunk(n);
  const int chunks = (int)((n + chunk - 1) / chunk);
  if (!ensure_partial(u, (int64_t)chunks * 27 * 16)) return false;
  k_wgrad_plain<1, 16, false><<<dim3(chunks, 27), 256, 0, stream()>>>(u->dout, u->d0b, v, chunk,
      u->partial);
  if (!launched("k_wgrad_plain")) return false;
  k_fold_chunks<<<(27 * 16 + 255) / 256, 256, 0, stream()>>>(u->partial, chunks, 27 * 16,
      u->grad + u->w_off[L_OUT]);
  if (!launched("k_fold_chunks")) return false;
  const int64_t bchunk = 4096;
  const int bblocks = (int)((n + bchunk - 1) / bchunk);
  if (!ensure_partial(u, bblocks)) return false;
  k_scalar_sum<<<bblocks, 256, 0, stream()>>>(u->dout, n, bchunk, u->partial);
  if (!launched("k_scalar_sum")) return false;
  k_fold_chunks<<<1, 32, 0, stream()>>>(u->partial, bblocks, 1, u->grad + u->b_off[L_OUT]);
  return launched("k_fold_chunks");
}

bool wgrad_first(UNetState *u, const Vol &v)
{
  const int64_t n = v.cells(), chunk = wgrad_chunk(n);
  const int chunks = (int)((n + chunk - 1) / chunk);
  if (!ensure_partial(u, (int64_t)chunks * 27 * 32)) return false;
  k_wgrad_plain<16, 2, true><<<dim3(chunks, 27), 256, 0, stream()>>>(u->G, u->x, v, chunk,
      u->partial);
  if (!launched("k_wgrad_plain")) return false;
  k_fold_chunks<<<(27 * 32 + 255) / 256, 256, 0, stream()>>>(u->partial, chunks, 27 * 32,
      u->grad + u->w_off[L_E0A]);
  if (!launched("k_fold_chunks")) return false;
  const int64_t bchunk = (n + 1023) / 1024 * 4 < 256 ? 256 : (n + 1023) / 1024 * 4;
  const int bblocks = (int)((n + bchunk - 1) / bchunk);
  if (!ensure_partial(u, (int64_t)bblocks * 16)) return false;
  k_channel_sum<16><<<bblocks, 256, 0, stream()>>>(u->G, n, bchunk, u->partial);
  if (!launched("k_channel_sum")) return false;
  k_fold_chunks<<<1, 64, 0, stream()>>>(u->partial, bblocks, 16, u->grad + u->b_off[L_E0A]);
  return launched("k_fold_chunks");
}

}  // namespace

// loss against `target` and the gradient of every parameter into u->grad
bool unet_backward(UNetState *u, const float *target)
{
  const Vol v0 = u->vol, v1 = half(v0), v2 = half(v1);
  const int64_t n0 = v0.cells(), n1 = v1.cells(), n2 = v2.cells();
  const ConvSrc none = { nullptr, 0, 0 };
  const int64_t lchunk = (n0 + 1023) / 1024 < 256 ? 256 : (n0 + 1023) / 1024;
  const int lblocks = (int)((n0 + lchunk - 1) / lchunk);
  k_mse<<<lblocks, 256, 0, stream()>>>(u->out, target, n0, lchunk, u->dout, u->loss_partial);
  if (!launched("k_mse")) return false;
  k_fold_loss<<<1, 1, 0, stream()>>>(u->loss_partial, lblocks, n0, u->loss);
  if (!launched("k_fold_loss")) return false;
  // out
  if (!wgrad_out(u, v0)) return false;
  k_conv_last_dgrad<<<(unsigned)((n0 + 255) / 256), 256, 0, stream()>>>(u->dout, v0, u->wb[L_OUT],
      u->F2);
  if (!launched("k_conv_last_dgrad")) return false;
  // d0b
  if (!mask(u->F2, u->d0b, 16 * n0, u->G)) return false;
  if (!wgrad(u, L_D0B, { u->d0a, 16, 0 }, none, v0) || !dgrad(u, L_D0B, v0, u->F1)) return false;
  // d0a (input concat [up(d1b) 32, e0b 16])
  if (!mask(u->F1, u->d0a, 16 * n0, u->G)) return false;
  if (!wgrad(u, L_D0A, { u->d1b, 32, 1 }, { u->e0b, 16, 0 }, v0) || !dgrad(u, L_D0A, v0, u->F1))
    return false;
  if (!split(u->F1, v0, 32, 16, u->Fe0b, u->F2)) return false;
  // d1b
  if (!mask(u->F2, u->d1b, 32 * n1, u->G)) return false;
  if (!wgrad(u, L_D1B, { u->d1a, 32, 0 }, none, v1) || !dgrad(u, L_D1B, v1, u->F1)) return false;
  // d1a (input concat [up(e2a) 64, e1b 32])
  if (!mask(u->F1, u->d1a, 32 * n1, u->G)) return false;
  if (!wgrad(u, L_D1A, { u->e2a, 64, 1 }, { u->e1b, 32, 0 }, v1) || !dgrad(u, L_D1A, v1, u->F2))
    return false;
  if (!split(u->F2, v1, 64, 32, u->Fe1b, u->F1)) return false;
  // e2a
  if (!mask(u->F1, u->e2a, 64 * n2, u->G)) return false;
  if (!wgrad(u, L_E2A, { u->p1, 32, 0 }, none, v2) || !dgrad(u, L_E2A, v2, u->F2)) return false;
  if (!pool_back(u->F2, v1, 32, u->Fe1b)) return false;
  // e1b
  if (!mask(u->Fe1b, u->e1b, 32 * n1, u->G)) return false;
  if (!wgrad(u, L_E1B, { u->e1a, 32, 0 }, none, v1) || !dgrad(u, L_E1B, v1, u->F1)) return false;
  // e1a
  if (!mask(u->F1, u->e1a, 32 * n1, u->G)) return false;
  if (!wgrad(u, L_E1A, { u->p0, 16, 0 }, none, v1) || !dgrad(u, L_E1A, v1, u->F2)) return false;
  if (!pool_back(u->F2, v0, 16, u->Fe0b)) return false;
  // e0b
  if (!mask(u->Fe0b, u->e0b, 16 * n0, u->G)) return false;
  if (!wgrad(u, L_E0B, { u->e0a, 16, 0 }, none, v0) || !dgrad(u, L_E0B, v0, u->F1)) return false;
  // e0a (no input gradient)
  if (!mask(u->F1, u->e0a, 16 * n0, u->G)) return false;
  return wgrad_first(u, v0);
}

bool unet_set_input(UNetState *u, const float *x, const Vol &v)
{
  if (!ensure_workspace(u, v)) return false;
  k_input_bf16<<<blocks_for(v.cells()), 256, 0, stream()>>>(x, v.cells(), u->x, u->x16);
  return launched("k_input_bf16");
}

}  // namespace nusif

using namespace nusif;

struct NusifUNet {
  UNetState s;
};

namespace {

// splitmix64 + Box-Muller: He-normal initial weights, zero biases
struct Rng {
  uint64_t s;
  uint64_t next()
  {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  double normal()
  {
    const double a = uniform(), b = uniform();
    return sqrt(-2.0 * log(a)) * cos(6.283185307179586 * b);
  }
};

NusifUNet *checked(NusifUNet *n)
{
  if (!n) fail(NUSIF_ERR_ARG, "unet: null network");
  return n;
}

// the tensor-core kernels' error flag (a bounded wait that ran out); synchronises
bool tc_clean(UNetState *u)
{
  int e = 0;
  if (!cuda_ok(cudaMemcpyAsync(&e, u->err, sizeof(int), cudaMemcpyDeviceToHost, stream()),
          "unet error flag") ||
      !cuda_ok(cudaStreamSynchronize(stream()), "unet error flag"))
    return false;
  if (e) {
    cudaMemsetAsync(u->err, 0, sizeof(int), stream());
    fail(NUSIF_ERR_CUDA, "unet: a tensor-core convolution timed out waiting for its operands");
    return false;
  }
  return true;
}

}  // namespace

namespace nusif {

bool unet_infer(NusifUNet *net, const float *x, int Z, int Y, int X, const float **out)
{
  UNetState *u = &net->s;
  const Vol v = { 1, Z, Y, X };
  if (!unet_set_input(u, x, v) || !unet_forward(u)) return false;
  *out = u->out;
  return true;
}

}  // namespace nusif

extern "C" {

NusifUNet *nusifUNetCreate(unsigned long long seed)
{
  NusifUNet *n = new NusifUNet();
  UNetState *u = &n->s;
  int64_t o = 0;
  for (int l = 0; l < kLayers; l++) {
    u->w_off[l] = o;
    o += 27 * kDesc[l].cout * kDesc[l].cin;
    u->b_off[l] = o;
    o += kDesc[l].cout;
  }
  u->nparam = o;
  std::vector<float> h(o, 0.0f);
  Rng rng{ seed };
  for (int l = 0; l < kLayers; l++) {
    const double sd = sqrt(2.0 / (27.0 * kDesc[l].cin));
    for (int64_t i = 0; i < 27 * kDesc[l].cout * kDesc[l].cin; i++)
      h[u->w_off[l] + i] = (float)(sd * rng.normal());
  }
  bool ok = cuda_ok(cudaMalloc(&u->master, o * sizeof(float)), "cudaMalloc(unet)") &&
            cuda_ok(cudaMalloc(&u->grad, o * sizeof(float)), "cudaMalloc(unet)") &&
            cuda_ok(cudaMalloc(&u->m, o * sizeof(float)), "cudaMalloc(unet)") &&
            cuda_ok(cudaMalloc(&u->v, o * sizeof(float)), "cudaMalloc(unet)") &&
            cuda_ok(cudaMalloc(&u->loss, sizeof(float)), "cudaMalloc(unet)") &&
            cuda_ok(cudaMalloc(&u->err, sizeof(int)), "cudaMalloc(unet)") &&
            cuda_ok(cudaMemset(u->err, 0, sizeof(int)), "unet init");
  ok = ok && cuda_ok(cudaMalloc(&u->w_first16, 27 * 256 * sizeof(bf16)), "cudaMalloc(unet)") &&
       cuda_ok(cudaMalloc(&u->w_last16, 27 * 256 * sizeof(bf16)), "cudaMalloc(unet)");
  for (int l = 0; ok && l < kLayers; l++) {
    const size_t nw = 27 * kDesc[l].cout * kDesc[l].cin;
    ok = cuda_ok(cudaMalloc(&u->wb[l], nw * sizeof(bf16)), "cudaMalloc(unet)") &&
         cuda_ok(cudaMalloc(&u->wt[l], nw * sizeof(bf16)), "cudaMalloc(unet)");
  }
  ok = ok && cuda_ok(cudaMemcpy(u->master, h.data(), o * sizeof(float), cudaMemcpyHostToDevice),
                 "unet init") &&
       cuda_ok(cudaMemset(u->grad, 0, o * sizeof(float)), "unet init") &&
       cuda_ok(cudaMemset(u->m, 0, o * sizeof(float)), "unet init") &&
       cuda_ok(cudaMemset(u->v, 0, o * sizeof(float)), "unet init") && refresh_bf16(u) &&
       cuda_ok(cudaStreamSynchronize(stream()), "unet init");
  if (!ok) {
    nusifUNetFree(n);
    return nullptr;
  }
  return n;
}

void nusifUNetFree(NusifUNet *n)
{
  if (!n) return;
  UNetState *u = &n->s;
  cudaDeviceSynchronize();
  free_workspace(u);
  if (u->partial) cudaFree(u->partial);
  for (float *p : { u->master, u->grad, u->m, u->v, u->loss })
    if (p) cudaFree(p);
  if (u->err) cudaFree(u->err);
  if (u->w_first16) cudaFree(u->w_first16);
  if (u->w_last16) cudaFree(u->w_last16);
  for (int l = 0; l < kLayers; l++) {
    if (u->wb[l]) cudaFree(u->wb[l]);
    if (u->wt[l]) cudaFree(u->wt[l]);
  }
  delete n;
}

long long nusifUNetParamCount(const NusifUNet *n) { return n ? n->s.nparam : 0; }

int nusifUNetGetParams(const NusifUNet *n, float *host, long long count)
{
  if (!checked(const_cast<NusifUNet *>(n)) || !host || count != n->s.nparam) {
    fail(NUSIF_ERR_ARG, "nusifUNetGetParams: need %lld values", n ? (long long)n->s.nparam : 0LL);
    return NUSIF_ERR_ARG;
  }
  if (!cuda_ok(cudaMemcpyAsync(host, n->s.master, count * sizeof(float), cudaMemcpyDeviceToHost,
                   stream()),
          "unet params") ||
      !cuda_ok(cudaStreamSynchronize(stream()), "unet params"))
    return NUSIF_ERR_CUDA;
  return NUSIF_OK;
}

int nusifUNetGetGrads(const NusifUNet *n, float *host, long long count)
{
  if (!checked(const_cast<NusifUNet *>(n)) || !host || count != n->s.nparam) {
    fail(NUSIF_ERR_ARG, "nusifUNetGetGrads: need %lld values", n ? (long long)n->s.nparam : 0LL);
    return NUSIF_ERR_ARG;
  }
  if (!cuda_ok(cudaMemcpyAsync(host, n->s.grad, count * sizeof(float), cudaMemcpyDeviceToHost,
                   stream()),
          "unet grads") ||
      !cuda_ok(cudaStreamSynchronize(stream()), "unet grads"))
    return NUSIF_ERR_CUDA;
  return NUSIF_OK;
}

int nusifUNetSetParams(NusifUNet *n, const float *host, long long count)
{
  if (!checked(n) || !host || count != n->s.nparam) {
    fail(NUSIF_ERR_ARG, "nusifUNetSetParams: need %lld values", n ? (long long)n->s.nparam : 0LL);
    return NUSIF_ERR_ARG;
  }
  UNetState *u = &n->s;
  if (!cuda_ok(cudaMemcpyAsync(u->master, host, count * sizeof(float), cudaMemcpyHostToDevice,
                   stream()),
          "unet params") ||
      !cuda_ok(cudaMemsetAsync(u->m, 0, count * sizeof(float), stream()), "unet adam") ||
      !cuda_ok(cudaMemsetAsync(u->v, 0, count * sizeof(float), stream()), "unet adam") ||
      !refresh_bf16(u) || !cuda_ok(cudaStreamSynchronize(stream()), "unet params"))
    return NUSIF_ERR_CUDA;
  u->adam_t = 0;
  return NUSIF_OK;
}

int nusifUNetForward(NusifUNet *n, const float *x, int B, int Z, int Y, int X, float *out)
{
  if (!checked(n) || !x || !out) return NUSIF_ERR_ARG;
  UNetState *u = &n->s;
  const Vol v = { B, Z, Y, X };
  if (!unet_set_input(u, x, v) || !unet_forward(u)) return has_error() ? NUSIF_ERR_CUDA : NUSIF_ERR_ARG;
  if (!cuda_ok(cudaMemcpyAsync(out, u->out, v.cells() * sizeof(float), cudaMemcpyDeviceToDevice,
                   stream()),
          "unet output"))
    return NUSIF_ERR_CUDA;
  return tc_clean(u) ? NUSIF_OK : NUSIF_ERR_CUDA;
}

int nusifUNetSetTensorCore(NusifUNet *n, int mode)
{
  if (!checked(n) || (mode != 0 && mode != 1)) {
    fail(NUSIF_ERR_ARG, "nusifUNetSetTensorCore: mode 0 (mma.sync) or 1 (tcgen05)");
    return NUSIF_ERR_ARG;
  }
  n->s.use_tc = mode;
  return NUSIF_OK;
}

int nusifUNetTrainStep(NusifUNet *n, const float *x, const float *target, int B, int Z, int Y,
    int X, float lr, int update, float *loss_host)
{
  if (!checked(n) || !x || !target) return NUSIF_ERR_ARG;
  UNetState *u = &n->s;
  const Vol v = { B, Z, Y, X };
  if (!unet_set_input(u, x, v) || !unet_forward(u) || !unet_backward(u, target))
    return NUSIF_ERR_CUDA;
  if (update) {
    u->adam_t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)u->adam_t), c2 = 1.0f - powf(b2, (float)u->adam_t);
    k_adam<<<blocks_for(u->nparam), 256, 0, stream()>>>(u->master, u->grad, u->m, u->v, u->nparam,
        lr, b1, b2, 1e-8f, c1, c2);
    if (!launched("k_adam") || !refresh_bf16(u)) return NUSIF_ERR_CUDA;
  }
  if (loss_host) {
    if (!cuda_ok(cudaMemcpyAsync(loss_host, u->loss, sizeof(float), cudaMemcpyDeviceToHost, stream()),
            "unet loss") ||
        !cuda_ok(cudaStreamSynchronize(stream()), "unet loss"))
      return NUSIF_ERR_CUDA;
    if (!tc_clean(u)) return NUSIF_ERR_CUDA;
  }
  return NUSIF_OK;
}

}  // extern "C"
