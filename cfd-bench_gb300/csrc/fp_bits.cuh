// IEEE-754 binary64 <-> binary32 conversions and an ordering key for |x|, on
// the integer pipe.
//
// GB300 executes FP64 instructions at two lanes per SM and clock; the
// double <-> float conversions and the FP64 min/max run on that same pipe. In
// the kernels bound by it (the FP64 residual of mixed-precision multigrid, the
// correction fold, the CFL maximum) these helpers do the same work with
// 32-bit integer operations, from the binary64 / binary32 encodings
// (sign | biased exponent | fraction; exponent biases 1023 and 127):
//  - to_f32_rn: round to nearest, ties to even. Results in the normal float
//    range and zeros are assembled here; the rest (float subnormals,
//    overflow, infinities, NaN) take the hardware conversion, so every input
//    gets exactly the hardware's result.
//  - to_f64: exact widening; zeros and normal floats here, the rest by the
//    hardware conversion.
//  - abs_max_key: a running maximum of |x| kept as its bit pattern
//    (non-negative doubles order like their bit patterns); NaN is skipped,
//    as fmax and the reference's `>` test skip it.
#pragma once

#include <cstdint>

namespace nusif {

__device__ __forceinline__ float to_f32_rn(double x)
{
  const unsigned hi = (unsigned)__double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e - 897u <= 253u) {  // binary32 exponent 1..254
    // 23 fraction bits: the 20 of the high word and the top 3 of the low word
    const unsigned frac = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;  // the 29 dropped bits
    unsigned bits = (hi & 0x80000000u) | ((e - 896u) << 23) | frac;
    // ties to even; a carry out of the fraction steps the exponent (to
    // infinity from the largest finite float, as rounding requires)
    bits += (rest > 0x10000000u || (rest == 0x10000000u && (frac & 1u))) ? 1u : 0u;
    return __uint_as_float(bits);
  }
  if (e == 0u) return __uint_as_float(hi & 0x80000000u);  // zero or FP64 subnormal: signed zero
  return __double2float_rn(x);
}

__device__ __forceinline__ double to_f64(float x)
{
  const unsigned b = __float_as_uint(x);
  const unsigned e = (b >> 23) & 0xffu;
  if (e - 1u <= 253u)  // normal: rebias the exponent by 1023 - 127 = 896
    return __hiloint2double((int)((b & 0x80000000u) | (((b & 0x7fffffffu) >> 3) + (896u << 20))),
                            (int)(b << 29));
  if ((b & 0x7fffffffu) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
  return (double)x;
}

// running maximum of |x| as the pair (high word, low word) of its bit
// pattern, compared lexicographically with 32-bit operations (a 64-bit
// integer maximum would use the FP64 pipe's 64-bit datapath)
__device__ __forceinline__ void abs_max_key(unsigned &mh, unsigned &ml, double x)
{
  const unsigned h = (unsigned)__double2hiint(x) & 0x7fffffffu;
  const unsigned l = (unsigned)__double2loint(x);
  const bool nan = h > 0x7ff00000u || (h == 0x7ff00000u && l != 0u);
  const bool gt = !nan && (h > mh || (h == mh && l > ml));
  mh = gt ? h : mh;
  ml = gt ? l : ml;
}

// the larger of two keys (high, low), lexicographically in 32-bit operations
__device__ __forceinline__ void key_max(unsigned &mh, unsigned &ml, unsigned h, unsigned l)
{
  const bool gt = h > mh || (h == mh && l > ml);
  mh = gt ? h : mh;
  ml = gt ? l : ml;
}

// the warp's largest key, in every lane
__device__ __forceinline__ void warp_key_max(unsigned &mh, unsigned &ml)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    key_max(mh, ml, __shfl_xor_sync(0xffffffffu, mh, off), __shfl_xor_sync(0xffffffffu, ml, off));
}

}  // namespace nusif
