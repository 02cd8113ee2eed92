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
//  - abs_key: |x| as an unsigned integer whose order is the numeric order of
//    |x| (non-negative doubles order like their bit patterns); NaN maps to 0,
//    so a maximum over keys ignores NaN as fmax does.
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

__device__ __forceinline__ unsigned long long abs_key(double x)
{
  const unsigned long long k = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
  return k > 0x7ff0000000000000ull ? 0ull : k;
}

}  // namespace nusif
