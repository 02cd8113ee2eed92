// Block-level reductions and the "last block folds" ticket used by every
// reduction of the library. The ticket makes a reduction deterministic (the
// last block to finish sums the per-block partials in a fixed order) without
// any spin-wait.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace nusif {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ float warp_sum_f(float v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// (i, j, k) of the flat index q = i + nx*(j + ny*k) in a grid-stride loop:
// the fixed stride is split into its (i, j, k) steps once, and each step of
// the loop adds them with carries instead of dividing a 64-bit index.
struct FlatWalk {
  int i, j, k;
  int di, dj, dk;
  __device__ __forceinline__ FlatWalk(int64_t q0, int64_t stride, int nx, int ny)
  {
    i = (int)(q0 % nx);
    const int64_t r = q0 / nx;
    j = (int)(r % ny);
    k = (int)(r / ny);
    di = (int)(stride % nx);
    const int64_t s = stride / nx;
    dj = (int)(s % ny);
    dk = (int)(s / ny);
  }
  __device__ __forceinline__ void advance(int nx, int ny)
  {
    i += di;
    const int ci = i >= nx;
    if (ci) i -= nx;
    j += dj + ci;
    const int cj = j >= ny;
    if (cj) j -= ny;
    k += dk + cj;
  }
};

// linear thread index for 1-, 2- and 3-D blocks
__device__ __forceinline__ int flat_tid()
{
  return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
}

// Sum over the block; every thread returns the total. NT = threads per block,
// sm must hold NT/32 doubles.
template <int NT>
__device__ __forceinline__ double block_reduce_sum(double v, double *sm)
{
  const int t = flat_tid();
  v = warp_sum(v);
  __syncthreads();
  if ((t & 31) == 0) sm[t >> 5] = v;
  __syncthreads();
  double r = 0.0;
#pragma unroll
  for (int q = 0; q < NT / 32; q++) r += sm[q];
  return r;
}

template <int NT>
__device__ __forceinline__ double block_reduce_max(double v, double *sm)
{
  const int t = flat_tid();
  v = warp_max(v);
  __syncthreads();
  if ((t & 31) == 0) sm[t >> 5] = v;
  __syncthreads();
  double r = sm[0];
#pragma unroll
  for (int q = 1; q < NT / 32; q++) r = fmax(r, sm[q]);
  return r;
}

// Called by one thread per block after it stored the block's partial result:
// true for the block that finishes last.
__device__ __forceinline__ bool ticket_is_last(unsigned *ticket)
{
  __threadfence();
  const unsigned total = gridDim.x * gridDim.y * gridDim.z;
  const unsigned t = atomicAdd(ticket, 1u);
  return t == total - 1;
}

__device__ __forceinline__ double ld_cg(const double *p) { return __ldcg(p); }

// Sum of partials[0..n) in a fixed order by one whole block; NT threads.
template <int NT>
__device__ __forceinline__ double fold_partials(const double *partials, int n, double *sm)
{
  double s = 0.0;
  for (int q = flat_tid(); q < n; q += NT) s += ld_cg(partials + q);
  return block_reduce_sum<NT>(s, sm);
}

}  // namespace nusif
