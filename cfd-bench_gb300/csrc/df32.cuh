// Double-float arithmetic: a value is an unevaluated sum of two binary32
// numbers (hi + lo), good to about 2^-46 of the magnitudes involved.
//
// GB300 issues FP64 instructions at two lanes per SM and clock, 64x below
// FP32. A stencil whose FP64 instruction count, not its memory traffic,
// bounds it runs several times faster when its arithmetic is carried in pairs
// of FP32 numbers on the FP32 pipe. The error-free transformations used here
// are the classical ones:
//  - two_sum (Knuth): s = fl(a + b) and the exact rounding error e, a + b = s + e;
//  - two_prod (with a fused multiply-add): p = fl(a b), e = fma(a, b, -p), a b = p + e.
// Sums and products of pairs keep the leading terms exactly and the small
// cross terms in plain FP32 (so "sloppy" in the usual classification), then
// renormalise the pair (fast two-sum, so |lo| <= ulp(hi)/2): the error of a
// result is a few units of 2^-47 of the largest operand, not of the result,
// which is also the error model of the FP64 operations they replace (about
// 2^-53 of the operands). Skipping the renormalisation saves three
// operations per result but, measured on computeFG, doubles the error.
//
// split() turns a binary64 number into a pair without conversion
// instructions (GB300 runs double -> float and integer -> float conversions on
// its FP64 pipe): hi is x with its fraction truncated to 23 bits (integer
// operations), lo the 29 dropped bits rounded to a float (two exact FP32
// subtractions and one fused multiply-add), so hi + lo = x to 2^-47 |x|
// (to 2^-97 for |x| < 2^-74).
// Magnitudes below 2^-126 become 0 and beyond the float range hi takes the
// hardware conversion (infinite), out of line.
//
// The header compiles for the device and, for CPU checks of the arithmetic,
// for the host (plain C++ with fmaf from <cmath>).
#pragma once

#include <cstdint>
#include <cstring>
#include <cmath>

#ifdef __CUDACC__
#define DF_FN __host__ __device__ __forceinline__
#else
#define DF_FN inline
#endif

namespace nusif {
namespace df {

struct f2 {
  float hi, lo;
};

DF_FN unsigned f32_bits(float x)
{
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  unsigned u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}

DF_FN float f32_from_bits(unsigned u)
{
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}

DF_FN unsigned hi_word(double x)
{
#ifdef __CUDA_ARCH__
  return (unsigned)__double2hiint(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return (unsigned)(u >> 32);
#endif
}

DF_FN unsigned lo_word(double x)
{
#ifdef __CUDA_ARCH__
  return (unsigned)__double2loint(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return (unsigned)u;
#endif
}

DF_FN double from_words(unsigned hi, unsigned lo)
{
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  uint64_t u = ((uint64_t)hi << 32) | lo;
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}

DF_FN float fmaf_(float a, float b, float c)
{
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

// a + b and a * b, rounded once: on the device the intrinsics keep the
// compiler from fusing a product into a later add, which would change the
// error terms the transformations below rely on
DF_FN float add_(float a, float b)
{
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}

DF_FN float mul_(float a, float b)
{
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

// Rare cases of split() and widen(), out of line on the device: GB300 runs
// the hardware double <-> float and integer -> float conversions on its FP64
// pipe, and a conversion the compiler if-converts into the common path would
// issue for every value.
#ifdef __CUDA_ARCH__
#define DF_RARE __device__ __noinline__
#else
#define DF_RARE inline
#endif

// |x| outside the normal float range: zeros and tiny values (below 2^-126)
// become zero, huge values, infinities and NaN take the hardware conversion
DF_RARE f2 split_rare(double x)
{
  f2 r;
  const unsigned h = hi_word(x);
  const unsigned e = (h >> 20) & 0x7ffu;
  if (e < 897u) {
    r.hi = f32_from_bits(h & 0x80000000u);
  } else {
    r.hi = (float)x;
  }
  r.lo = 0.0f;
  return r;
}

// float subnormals, infinities and NaN
DF_RARE double widen_rare(float x) { return (double)x; }

// binary64 -> pair on the integer and FP32 pipes (see the header comment)
DF_FN f2 split(double x)
{
  const unsigned h = hi_word(x), l = lo_word(x);
  const unsigned e = (h >> 20) & 0x7ffu;
  if (e - 897u > 253u) return split_rare(x);  // truncated value outside the normal float range
  const unsigned sign = h & 0x80000000u;
  f2 r;
  r.hi = f32_from_bits(sign | ((e - 896u) << 23) | ((h & 0xfffffu) << 3) | (l >> 29));
  // the 29 dropped bits, an integer below 2^29, rounded to a float without a
  // conversion instruction: its two parts below 2^23 and 2^6 are exact as
  // (2^23 + n) - 2^23, and one fused multiply-add rounds their sum once
  const unsigned rest = l & 0x1fffffffu;
  const float top = add_(f32_from_bits(0x4b000000u | (rest >> 6)), -8388608.0f);
  const float low = add_(f32_from_bits(0x4b000000u | (rest & 63u)), -8388608.0f);
  const float rn = fmaf_(top, 64.0f, low);
  // they weigh 2^(e - 1023 - 52) each; that scale is a normal float for
  // e >= 949 (below, |x| < 2^-74 and the remainder, under 2^-97, is dropped)
  const float scale = f32_from_bits(e >= 949u ? ((e - 948u) << 23) : 0u);
  r.lo = f32_from_bits(f32_bits(mul_(rn, scale)) | sign);
  return r;
}

// exact binary32 -> binary64 widening on the integer pipe (normal floats and
// zeros; the rest through the hardware conversion, out of line)
DF_FN double widen(float x)
{
  const unsigned b = f32_bits(x);
  const unsigned e = (b >> 23) & 0xffu;
  if (e - 1u <= 253u)
    return from_words((b & 0x80000000u) | (((b & 0x7fffffffu) >> 3) + (896u << 20)), b << 29);
  if ((b & 0x7fffffffu) == 0u) return from_words(b & 0x80000000u, 0u);
  return widen_rare(x);
}

// a pair as a binary64 number (one FP64 add; both widenings are exact)
DF_FN double to_double(f2 a) { return widen(a.hi) + widen(a.lo); }

// a pair from a binary64 constant, on the host or once per thread
DF_FN f2 from_double_rn(double x)
{
  f2 r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}

DF_FN f2 neg(f2 a) { return f2{ -a.hi, -a.lo }; }

// s + e = a + b exactly (Knuth's two-sum, no ordering of |a|, |b| needed)
DF_FN f2 two_sum(float a, float b)
{
  const float s = add_(a, b);
  const float bb = add_(s, -a);
  const float e = add_(add_(a, -add_(s, -bb)), add_(b, -bb));
  return f2{ s, e };
}

// p + e = a * b exactly
DF_FN f2 two_prod(float a, float b)
{
  const float p = mul_(a, b);
  return f2{ p, fmaf_(a, b, -p) };
}

// (hi, lo) with |lo| small against |hi| (or hi == 0) -> the same value with
// |lo| <= ulp(hi)/2 (fast two-sum)
DF_FN f2 renorm(float hi, float lo)
{
  const float s = add_(hi, lo);
  return f2{ s, add_(lo, -add_(s, -hi)) };
}

// a + b
DF_FN f2 add(f2 a, f2 b)
{
  const f2 s = two_sum(a.hi, b.hi);
  return renorm(s.hi, add_(s.lo, add_(a.lo, b.lo)));
}

DF_FN f2 sub(f2 a, f2 b) { return add(a, neg(b)); }

// a * b
DF_FN f2 mul(f2 a, f2 b)
{
  const f2 p = two_prod(a.hi, b.hi);
  return renorm(p.hi, add_(p.lo, fmaf_(a.hi, b.lo, mul_(a.lo, b.hi))));
}

// a * b + c
DF_FN f2 fma(f2 a, f2 b, f2 c)
{
  const f2 p = two_prod(a.hi, b.hi);
  const f2 s = two_sum(p.hi, c.hi);
  return renorm(s.hi, add_(add_(s.lo, p.lo), add_(c.lo, fmaf_(a.hi, b.lo, mul_(a.lo, b.hi)))));
}

// a * x + b * y
DF_FN f2 dot2(f2 a, f2 x, f2 b, f2 y)
{
  const f2 p = two_prod(a.hi, x.hi), q = two_prod(b.hi, y.hi);
  const f2 s = two_sum(p.hi, q.hi);
  const float cross =
      fmaf_(a.hi, x.lo, fmaf_(a.lo, x.hi, fmaf_(b.hi, y.lo, mul_(b.lo, y.hi))));
  return renorm(s.hi, add_(add_(s.lo, add_(p.lo, q.lo)), cross));
}

// The same operations without the final renormalisation (an "unnormalised"
// pair: hi + lo is the value, |lo| may exceed ulp(hi)/2). Safe where the result
// only feeds further pair arithmetic -- two_sum and two_prod stay exact for any
// inputs and the low parts' FP32 rounding stays a few 2^-47 of the operands --
// and not where the sign of hi is read (an unnormalised hi can be 0 or carry the
// wrong sign when the value is tiny).
DF_FN f2 add_u(f2 a, f2 b)
{
  const f2 s = two_sum(a.hi, b.hi);
  return f2{ s.hi, add_(s.lo, add_(a.lo, b.lo)) };
}

DF_FN f2 sub_u(f2 a, f2 b) { return add_u(a, neg(b)); }

DF_FN f2 mul_u(f2 a, f2 b)
{
  const f2 p = two_prod(a.hi, b.hi);
  return f2{ p.hi, add_(p.lo, fmaf_(a.hi, b.lo, mul_(a.lo, b.hi))) };
}

DF_FN f2 fma_u(f2 a, f2 b, f2 c)
{
  const f2 p = two_prod(a.hi, b.hi);
  const f2 s = two_sum(p.hi, c.hi);
  return f2{ s.hi, add_(add_(s.lo, p.lo), add_(c.lo, fmaf_(a.hi, b.lo, mul_(a.lo, b.hi)))) };
}

DF_FN f2 dot2_u(f2 a, f2 x, f2 b, f2 y)
{
  const f2 p = two_prod(a.hi, x.hi), q = two_prod(b.hi, y.hi);
  const f2 s = two_sum(p.hi, q.hi);
  const float cross =
      fmaf_(a.hi, x.lo, fmaf_(a.lo, x.hi, fmaf_(b.hi, y.lo, mul_(b.lo, y.hi))));
  return f2{ s.hi, add_(add_(s.lo, add_(p.lo, q.lo)), cross) };
}

}  // namespace df
}  // namespace nusif
