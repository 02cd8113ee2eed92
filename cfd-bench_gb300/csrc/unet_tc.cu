// 3x3x3 convolutions of the U-Net on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory, operands staged by TMA).
//
// Implicit GEMM: M = 128 cells of one z-plane (a tile of 16 x-columns by 8
// y-rows), N = output channels, K = 27 taps x input channels. The tile's rows
// are ordered x-major over 8-cell y-columns, so each x-column is one 8-row
// swizzle atom of the K-major operand layout. A stage carries one (dz, dy)
// row of taps: per source one TMA tiled load of the 18 x-columns x 8 y-rows
// around the tile (x from x0 - 1 to x0 + 16, through a tensor map whose
// second dimension is y and third x, so the box lands column by column), and
// one load of the row's three tap weights [3][N][C]. The three dx taps of the
// row read that one box through descriptors offset by 0, 1 and 2 atoms, so a
// cell row is loaded once per (dz, dy) instead of once per tap. Out-of-range
// x and y read as zero, which is the convolution's zero padding; a dz plane
// outside the volume is skipped for the whole tile. The swizzle is the one
// whose span is the cell row (32, 64 or 128 bytes for 16, 32 or 64 channels),
// which is also the canonical K-major operand layout for that span (8-row
// atoms; stride offset 8 rows). The MMA thread issues one tcgen05.mma
// (kind::f16, BF16 x BF16 -> FP32, M = 128, N = channels out, K = 16) per 16
// input channels per tap, the descriptors advanced by 32 bytes along the
// swizzled row, and commits the stage back to the producer. Accumulators are
// double-buffered in tensor memory, so four epilogue warps drain one tile
// (tcgen05.ld, bias, ReLU, BF16 or FP32 rows) while the next tile's products
// accumulate.
//
// Two sources (the decoder's concat) are two K ranges of the same tile.
// Every mbarrier wait is bounded (about one second); a wait that runs out
// sets an error flag the host reads, the warps stop issuing work, wait
// (bounded) for the copies and products already issued, free tensor memory
// and return.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <cstdlib>
#include <cstdio>

#include "nusif_internal.h"
#include "unet_tc.h"

namespace nusif {
namespace {

constexpr int kTileM = 128;
constexpr int kTileX = 16, kTileY = 8;  // tile: 16 x-columns of 8 y-cells
constexpr int kBoxX = kTileX + 2;       // loaded columns: the tile and one on each side
constexpr int kThreads = 192;  // warp 0 TMA producer, warp 1 MMA issuer, warps 2-5 epilogue
constexpr int kMaxStages = 16;
constexpr uint32_t kBarBytes = 512;  // barrier and flag region at the start of shared memory
constexpr uint64_t kWaitNs = 1000000000ull;  // bound of every mbarrier wait

struct TcParams {
  int N;                 // output channels (MMA N)
  int C0, C1;            // channels of source 0 and source 1 (0: none): 16, 32 or 64
  uint32_t a_off[2], b_off[2];  // offsets of each source's cell box and tap weights in a stage
  uint32_t atom[2];      // bytes of one x-column (8 cell rows) of each source
  uint32_t wtap[2];      // bytes of one tap's weights [N][C] of each source
  uint32_t stage_bytes, tx_bytes;
  int X, Y, Z, B;        // volume
  int tx, ty;            // tiles per row (X / 16) and per column (Y / 8)
  int ntiles;
  int stages;
  int tmem_cols;         // allocated tensor-memory columns (>= 2 N, power of two)
  uint32_t idesc;        // instruction descriptor
  const float *bias;     // [N] or nullptr
  int relu;
  int out_bf16;
  int out_ch;            // leading channels stored per cell (N, or 1 for a padded 1-channel layer)
  void *out;             // [cells][out_ch]
  int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t now_ns()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// the same test, the thread suspended (no issue slots) until the phase
// completes or about `hint_ns` pass
__device__ __forceinline__ bool mbar_try_sleep(uint32_t bar, uint32_t parity, uint32_t hint_ns)
{
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

// wait for the phase of `parity` to complete; false after the time bound or
// when another warp has raised the abort flag. Waiting threads sleep in the
// barrier rather than spin, so the single-thread producer and MMA issuer of
// the block's other warps keep their issue slots; the abort flag and the
// clock are read every 8th round.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err)
{
  if (mbar_try(bar, parity)) return true;
  const uint64_t t0 = now_ns();
  for (uint32_t round = 1;; round++) {
    if (mbar_try_sleep(bar, parity, 20000u)) return true;
    if ((round & 7u) == 0) {
      if (*abort_flag) return false;
      if (now_ns() - t0 > kWaitNs) {
        *abort_flag = 1;
        atomicExch(err, 1);
        return false;
      }
    }
  }
}

// bounded wait used while draining after an abort (does not re-raise it)
__device__ void mbar_drain(uint32_t bar, uint32_t parity)
{
  const uint64_t t0 = now_ns();
  while (!mbar_try(bar, parity) && now_ns() - t0 < kWaitNs) {
  }
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, uint32_t bar,
    int c0, int c1, int c2, int c3)
{
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, uint32_t bar,
    int c0, int c1, int c2)
{
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}

// shared-memory matrix descriptor, K-major, rows of `row_bytes` (32, 64 or
// 128) in the swizzle of that span: stride offset = one 8-row atom, leading
// offset unused (1), base offset 0 (atoms 1024-byte aligned)
__device__ __forceinline__ uint64_t smem_desc_sw(uint32_t addr, uint32_t row_bytes)
{
  const uint64_t mode = row_bytes == 128u ? 2u : row_bytes == 64u ? 4u : 6u;
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= 1ull << 16;                                      // leading byte offset (unused)
  d |= (uint64_t)(((8u * row_bytes) >> 4) & 0x3FFFu) << 32;  // stride byte offset
  d |= 1ull << 46;  // descriptor version of this architecture
  d |= mode << 61;  // swizzle mode
  return d;
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
    uint32_t accumulate)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this warp's 32 lanes (one row per thread)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t pack2(float a, float b)
{
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&v);
}

struct Tile {
  int x0, y0, zb, z;
};

__device__ __forceinline__ Tile tile_of(const TcParams &P, int t)
{
  Tile r;
  r.x0 = (t % P.tx) * kTileX;
  const int rest = t / P.tx;
  r.y0 = (rest % P.ty) * kTileY;
  r.zb = rest / P.ty;
  r.z = r.zb % P.Z;
  return r;
}

// resident blocks per SM the compiler keeps registers for: eight of the
// 16-channel layers (the full-resolution ones, bound by per-block latency)
constexpr int conv_min_blocks(int nch) { return nch == 16 ? 8 : 1; }

template <int NCH>  // output channels, a multiple of 16
__global__ void __launch_bounds__(kThreads, conv_min_blocks(NCH)) k_conv_tc(const __grid_constant__ CUtensorMap tm_a0,
    const __grid_constant__ CUtensorMap tm_a1, const __grid_constant__ CUtensorMap tm_w0,
    const __grid_constant__ CUtensorMap tm_w1, const TcParams P)
{
  extern __shared__ __align__(1024) unsigned char smem[];
  // [0, kBarBytes): barriers, then the tensor-memory address and the abort
  // flag; stages from the first 1024-byte boundary after that
  static_assert((2 * kMaxStages + 4) * 8 + 8 <= kBarBytes, "barriers overlap the flags");
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
  uint64_t *full = bars, *empty = bars + kMaxStages, *acc_full = bars + 2 * kMaxStages,
           *acc_empty = bars + 2 * kMaxStages + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + kBarBytes - 8);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + kBarBytes - 4);
  // stages start at the first 1024-byte boundary past the barriers (TMA destinations
  // need 128-byte alignment)
  const uint32_t sbase = smem_u32(smem);
  unsigned char *stage_base = smem + (((sbase + kBarBytes + 1023u) & ~1023u) - sbase);
  const uint32_t stage_bytes = P.stage_bytes;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < P.stages; s++) {
      mbar_init(smem_u32(full + s), 1);
      mbar_init(smem_u32(empty + s), 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(smem_u32(acc_full + b), 1);
      mbar_init(smem_u32(acc_empty + b), 128);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {  // tensor memory for two accumulators
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(P.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer ----------------
    bool armed[kMaxStages];
    uint32_t armed_par[kMaxStages];
    for (int s = 0; s < kMaxStages; s++) armed[s] = false;
    int stage = 0;
    uint32_t phase = 0;
    bool ok = true;
    for (int t = blockIdx.x; ok && t < P.ntiles; t += gridDim.x) {
      const Tile tl = tile_of(P, t);
      for (int row = 0; row < 9; row++) {  // (dz, dy) rows of taps; a stage per row
        const int dz = row / 3 - 1, dy = row % 3 - 1;
        if (tl.z + dz < 0 || tl.z + dz >= P.Z) continue;
        if (!mbar_wait(smem_u32(empty + stage), phase ^ 1u, abort_flag, P.err)) {
          ok = false;
          break;
        }
        armed[stage] = false;
        const uint32_t fb = smem_u32(full + stage);
        const uint32_t sa = smem_u32(stage_base + (size_t)stage * stage_bytes);
        mbar_expect_tx(fb, P.tx_bytes);
        // the box (C, 8 y, 18 x) at y0 + dy, x0 - 1; the row's three taps' weights
        tma_load_4d(sa + P.a_off[0], &tm_a0, fb, 0, tl.y0 + dy, tl.x0 - 1, tl.zb + dz);
        tma_load_3d(sa + P.b_off[0], &tm_w0, fb, 0, 0, 3 * row);
        if (P.C1 > 0) {
          tma_load_4d(sa + P.a_off[1], &tm_a1, fb, 0, tl.y0 + dy, tl.x0 - 1, tl.zb + dz);
          tma_load_3d(sa + P.b_off[1], &tm_w1, fb, P.C0, 0, 3 * row);
        }
        armed[stage] = true;
        armed_par[stage] = phase;
        if (++stage == P.stages) {
          stage = 0;
          phase ^= 1u;
        }
      }
    }
    if (!ok)  // let the copies already issued land before the shared memory goes away
      for (int s = 0; s < P.stages; s++)
        if (armed[s]) mbar_drain(smem_u32(full + s), armed_par[s]);
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    int stage = 0;
    uint32_t phase = 0;
    int acc = 0;
    uint32_t acc_phase = 0;
    bool ok = true;
    bool issued = false;
    for (int t = blockIdx.x; ok && t < P.ntiles; t += gridDim.x) {
      const Tile tl = tile_of(P, t);
      if (!mbar_wait(smem_u32(acc_empty + acc), acc_phase ^ 1u, abort_flag, P.err)) {
        ok = false;
        break;
      }
      fence_after();
      const uint32_t d = tmem + (uint32_t)(acc * (P.tmem_cols / 2));
      uint32_t accumulate = 0;
      for (int row = 0; row < 9; row++) {
        const int dz = row / 3 - 1;
        if (tl.z + dz < 0 || tl.z + dz >= P.Z) continue;
        if (!mbar_wait(smem_u32(full + stage), phase, abort_flag, P.err)) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t sa = smem_u32(stage_base + (size_t)stage * stage_bytes);
        // the descriptors' start-address field is (address >> 4) in 14 bits;
        // every operand lies below 256 KB, so offsets add to it without carry
        uint64_t a0[2], b0[2];
        uint32_t da[2], db[2];
        int ks[2];
        for (int src = 0; src < 2; src++) {
          ks[src] = (src == 0 ? P.C0 : P.C1) / 16;
          const uint32_t rb = 32u * (uint32_t)ks[src];
          a0[src] = smem_desc_sw(sa + P.a_off[src], rb);
          b0[src] = smem_desc_sw(sa + P.b_off[src], rb);
          da[src] = P.atom[src] >> 4;
          db[src] = P.wtap[src] >> 4;
        }
        for (int q = 0; q < 3; q++) {  // dx = q - 1: the box read q atoms in
          for (int src = 0; src < 2; src++) {
            for (int j = 0; j < ks[src]; j++) {
              mma_f16(d, a0[src] + (uint64_t)(q * da[src] + 2u * j),
                  b0[src] + (uint64_t)(q * db[src] + 2u * j), P.idesc, accumulate);
              accumulate = 1;
              issued = true;
            }
          }
        }
        mma_commit(smem_u32(empty + stage));
        if (++stage == P.stages) {
          stage = 0;
          phase ^= 1u;
        }
      }
      if (!ok) break;
      mma_commit(smem_u32(acc_full + acc));
      if (++acc == 2) {
        acc = 0;
        acc_phase ^= 1u;
      }
    }
    if (!ok && issued) {  // wait for every product already issued
      mma_commit(smem_u32(acc_full + acc));
      mbar_drain(smem_u32(acc_full + acc), acc_phase);
    }
  } else if (warp >= 2) {
    // ---------------- epilogue: tensor memory -> bias, ReLU -> global ----------------
    const int q = warp & 3;  // this warp may read lanes 32q .. 32q + 31
    const int row = 32 * q + lane;
    int acc = 0;
    uint32_t acc_phase = 0;
    for (int t = blockIdx.x; t < P.ntiles; t += gridDim.x) {
      // warp-uniform: the tensor-memory loads below need the whole warp
      const bool ready = mbar_wait(smem_u32(acc_full + acc), acc_phase, abort_flag, P.err);
      if (!__all_sync(0xffffffffu, ready)) break;
      fence_after();
      float v[NCH];
#pragma unroll
      for (int c = 0; c < NCH; c += 16) {
        float part[16];
        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(acc * (P.tmem_cols / 2) + c),
            part);
#pragma unroll
        for (int e = 0; e < 16; e++) v[c + e] = part[e];
      }
      tmem_wait_ld();
      fence_before();
      mbar_arrive(smem_u32(acc_empty + acc));
      // accumulator row = x-column * 8 + y within the tile
      const Tile tl = tile_of(P, t);
      const int64_t cell =
          ((int64_t)tl.zb * P.Y + tl.y0 + (row & 7)) * P.X + tl.x0 + (row >> 3);
      if (P.out_ch == 1) {  // one channel (the output layer, its weights padded to 16 rows)
        const float x = v[0] + (P.bias ? __ldg(P.bias) : 0.0f);
        static_cast<float *>(P.out)[cell] = P.relu ? fmaxf(x, 0.0f) : x;
      } else {
#pragma unroll
        for (int c = 0; c < NCH; c++) {
          const float x = v[c] + (P.bias ? __ldg(P.bias + c) : 0.0f);
          v[c] = P.relu ? fmaxf(x, 0.0f) : x;
        }
      }
      if (P.out_ch == 1) {
      } else if (P.out_bf16) {
        uint4 *o = reinterpret_cast<uint4 *>(static_cast<__nv_bfloat16 *>(P.out) + cell * NCH);
#pragma unroll
        for (int c = 0; c < NCH; c += 8)
          o[c / 8] = make_uint4(pack2(v[c], v[c + 1]), pack2(v[c + 2], v[c + 3]),
              pack2(v[c + 4], v[c + 5]), pack2(v[c + 6], v[c + 7]));
      } else {
        float4 *o = reinterpret_cast<float4 *>(static_cast<float *>(P.out) + cell * NCH);
#pragma unroll
        for (int c = 0; c < NCH; c += 4) o[c / 4] = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
      }
      if (++acc == 2) {
        acc = 0;
        acc_phase ^= 1u;
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(P.tmem_cols)
                 : "memory");
  }
}

// ------------------------------------------------------------------ host side

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
            &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

CUtensorMapSwizzle swizzle_for(int channels)
{
  return channels == 64 ? CU_TENSOR_MAP_SWIZZLE_128B
                        : channels == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
}

// channels-last BF16 volume [zb][y][x][C] as a 4-D map (C, Y, X, Z*B) -- y
// before x, so a box (C, 8, 18, 1) lands as 18 x-columns of 8 cell rows --
// one C x 2-byte row per cell, swizzled over that span
bool map_volume(CUtensorMap *m, const void *base, int C, int X, int Y, int ZB)
{
  auto fn = encode_fn();
  if (!fn) {
    fail(NUSIF_ERR_CUDA, "unet: cuTensorMapEncodeTiled unavailable");
    return false;
  }
  const cuuint64_t dims[4] = { (cuuint64_t)C, (cuuint64_t)Y, (cuuint64_t)X, (cuuint64_t)ZB };
  const cuuint64_t strides[3] = { (cuuint64_t)X * C * 2, (cuuint64_t)C * 2,
    (cuuint64_t)Y * X * C * 2 };
  const cuuint32_t box[4] = { (cuuint32_t)C, (cuuint32_t)kTileY, (cuuint32_t)kBoxX, 1 };
  const cuuint32_t es[4] = { 1, 1, 1, 1 };
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(base), dims,
      strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(C),
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    fail(NUSIF_ERR_CUDA, "unet: tensor map of a %dx%dx%dx%d volume failed (%d)", C, X, Y, ZB, (int)r);
    return false;
  }
  return true;
}

// weights [27][N][K] as a 3-D map (K, N, 27), box (C, N, 3): the C columns of
// one source for one (dz, dy) row of three taps, swizzled like that source's
// cell rows
bool map_weights(CUtensorMap *m, const void *base, int K, int N, int C)
{
  auto fn = encode_fn();
  if (!fn) {
    fail(NUSIF_ERR_CUDA, "unet: cuTensorMapEncodeTiled unavailable");
    return false;
  }
  const cuuint64_t dims[3] = { (cuuint64_t)K, (cuuint64_t)N, 27 };
  const cuuint64_t strides[2] = { (cuuint64_t)K * 2, (cuuint64_t)N * K * 2 };
  const cuuint32_t box[3] = { (cuuint32_t)C, (cuuint32_t)N, 3 };
  const cuuint32_t es[3] = { 1, 1, 1 };
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(base), dims,
      strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(C),
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    fail(NUSIF_ERR_CUDA, "unet: weight tensor map %dx%d failed (%d)", K, N, (int)r);
    return false;
  }
  return true;
}

int sm_count_tc()
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

uint32_t align1k(uint32_t x) { return (x + 1023u) & ~1023u; }

template <int NCH>
bool launch_tc(const CUtensorMap &a0, const CUtensorMap &a1, const CUtensorMap &w0,
    const CUtensorMap &w1, TcParams P)
{
  // per source: the box of 18 x-columns (8 cell rows each), then the row's
  // three taps' weights [3][N][C], each region 1024-byte aligned (the
  // 128-byte swizzle's atom; an x-column and a tap's weights are whole
  // multiples of every swizzle's 8-row repeat)
  uint32_t off = 0, tx = 0;
  for (int src = 0; src < 2; src++) {
    const uint32_t rb = 2u * (uint32_t)(src == 0 ? P.C0 : P.C1);
    P.atom[src] = (uint32_t)kTileY * rb;
    P.wtap[src] = (uint32_t)NCH * rb;
    P.a_off[src] = off;
    off = align1k(off + (uint32_t)kBoxX * P.atom[src]);
    P.b_off[src] = off;
    off = align1k(off + 3u * P.wtap[src]);
    if (src == 0 || P.C1 > 0) tx += (uint32_t)kBoxX * P.atom[src] + 3u * P.wtap[src];
  }
  P.stage_bytes = off;
  P.tx_bytes = tx;
  const size_t stage_bytes = P.stage_bytes;
  // two stages: the fewer the stages, the more blocks an SM holds, and more
  // blocks measured faster than deeper pipelines (the 128^3 forward pass:
  // 1.77 ms with 2 stages and six blocks of 16 -> 16 layers per SM (1.73 ms
  // with eight, their registers capped for it), 1.81 ms
  // with 4, 2.36 ms with 8, 2.43 ms with 16 stages and two blocks per SM);
  // NUSIF_TC_STAGES overrides the count
  int stages = 2;
  if (const char *e = getenv("NUSIF_TC_STAGES")) {
    const int s = atoi(e);
    if (s >= 2) stages = s;
  }
  const int fit = (int)((227 * 1024 - kBarBytes - 1024) / stage_bytes);
  if (stages > fit) stages = fit;
  if (stages > kMaxStages) stages = kMaxStages;
  if (stages < 2) stages = 2;
  P.stages = stages;
  int cols = 32;
  while (cols < 2 * NCH) cols <<= 1;
  P.tmem_cols = cols;
  // barriers and flags, alignment to 1024 bytes, stages
  const size_t smem = kBarBytes + 1024 + (size_t)stages * stage_bytes;
  if (smem > 227 * 1024) {
    fail(NUSIF_ERR_ARG, "unet: convolution stage of %zu bytes too large", stage_bytes);
    return false;
  }
  // at most 512 / cols blocks of an SM may hold tensor memory at once
  const int per_sm_tmem = 512 / cols;
  static bool attr_set[64] = {};
  int dev = 0;
  if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return false;
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    if (!cuda_ok(cudaFuncSetAttribute(k_conv_tc<NCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                     227 * 1024),
            "k_conv_tc shared memory"))
      return false;
    attr_set[dev] = true;
  }
  // a persistent grid: no more blocks than can be resident at once, by shared
  // memory (1 KB reserved per block), registers (8-register granules per
  // thread) and tensor memory
  cudaFuncAttributes fa{};
  if (!cuda_ok(cudaFuncGetAttributes(&fa, k_conv_tc<NCH>), "k_conv_tc attributes")) return false;
  const int regs_block = ((fa.numRegs + 7) / 8) * 8 * kThreads;
  int per_sm = (int)((228 * 1024) / (smem + 1024));
  if (regs_block > 0 && per_sm > 65536 / regs_block) per_sm = 65536 / regs_block;
  if (per_sm > per_sm_tmem) per_sm = per_sm_tmem;
  if (per_sm < 1) per_sm = 1;
  int grid = sm_count_tc() * per_sm;
  if (grid > P.ntiles) grid = P.ntiles;
  P.idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NCH >> 3) << 17) |
            ((uint32_t)(kTileM >> 4) << 24);
  k_conv_tc<NCH><<<grid, kThreads, smem, stream()>>>(a0, a1, w0, w1, P);
  return launched("k_conv_tc");
}

}  // namespace

bool tc_conv_supported(int X, int Y, int Z, int B, int N, int C0, int C1)
{
  if (X <= 0 || Y <= 0 || Z <= 0 || B <= 0) return false;
  auto ok_c = [](int c) { return c == 16 || c == 32 || c == 64; };
  if (!ok_c(C0) || (C1 != 0 && !ok_c(C1))) return false;
  if (N != 16 && N != 32 && N != 48 && N != 64 && N != 96) return false;
  if (X % kTileX || Y % kTileY) return false;
  return encode_fn() != nullptr;
}

bool tc_conv(const void *s0, int C0, const void *s1, int C1, int B, int Z, int Y, int X,
    const void *w, int N, const float *bias, int relu, bool out_bf16, void *out, int *err,
    int out_ch)
{
  TcParams P{};
  P.N = N;
  P.C0 = C0;
  P.C1 = C1;
  P.X = X;
  P.Y = Y;
  P.Z = Z;
  P.B = B;
  P.tx = X / kTileX;
  P.ty = Y / kTileY;
  P.ntiles = (int)((int64_t)B * Z * P.ty * P.tx);
  P.bias = bias;
  P.relu = relu;
  P.out_bf16 = out_bf16 ? 1 : 0;
  P.out_ch = out_ch > 0 ? out_ch : N;
  if (P.out_ch != N && !(P.out_ch == 1 && !out_bf16)) {
    fail(NUSIF_ERR_ARG, "unet: a convolution stores all its channels or one FP32 channel");
    return false;
  }
  P.out = out;
  P.err = err;
  CUtensorMap a0, a1, w0, w1;
  if (!map_volume(&a0, s0, C0, X, Y, Z * B)) return false;
  if (!map_weights(&w0, w, C0 + C1, N, C0)) return false;
  if (C1 > 0) {
    if (!map_volume(&a1, s1, C1, X, Y, Z * B)) return false;
    if (!map_weights(&w1, w, C0 + C1, N, C1)) return false;
  } else {
    a1 = a0;
    w1 = w0;
  }
  switch (N) {
  case 16: return launch_tc<16>(a0, a1, w0, w1, P);
  case 32: return launch_tc<32>(a0, a1, w0, w1, P);
  case 48: return launch_tc<48>(a0, a1, w0, w1, P);
  case 64: return launch_tc<64>(a0, a1, w0, w1, P);
  case 96: return launch_tc<96>(a0, a1, w0, w1, P);
  }
  fail(NUSIF_ERR_ARG, "unet: no tensor-core convolution for %d output channels", N);
  return false;
}

}  // namespace nusif
