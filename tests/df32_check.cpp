// Host check of the double-float helpers (cfd-bench_gb300/csrc/df32.cuh),
// compiled by tests/test_df32_host.py: split() against its definition (hi the
// truncated binary64, lo the rounded remainder, the same bits as the hardware
// integer -> float conversion would give), its error bound, and the exact
// widening of every float class.
#include "df32.cuh"

#include <cmath>
#include <cstdio>
#include <random>

using namespace nusif::df;

int main(int argc, char **argv)
{
  const long samples = argc > 1 ? atol(argv[1]) : 2000000;
  std::mt19937_64 gen(20261204);
  long checked = 0, bad_lo = 0, bad_err = 0, bad_widen = 0;
  for (long q = 0; q < samples; q++) {
    const uint64_t u = gen();
    double x;
    memcpy(&x, &u, 8);
    if (!std::isnan(x)) {
      const f2 r = split(x);
      const unsigned h = hi_word(x), l = lo_word(x), e = (h >> 20) & 0x7ffu;
      if (e - 897u <= 253u) {
        const unsigned rest = l & 0x1fffffffu;
        const float scale = f32_from_bits(e >= 949u ? ((e - 948u) << 23) : 0u);
        const float lo = f32_from_bits(f32_bits((float)rest * scale) | (h & 0x80000000u));
        if (f32_bits(lo) != f32_bits(r.lo)) bad_lo++;
        const long double err = fabsl((long double)r.hi + (long double)r.lo - (long double)x);
        if (err > fmaxl(ldexpl(fabsl((long double)x), -47), ldexpl(1.0L, -97))) bad_err++;
        checked++;
      } else if (e < 897u ? (r.hi != 0.0f || r.lo != 0.0f) : !std::isinf(r.hi)) {
        bad_err++;
      }
    }
    float fx;
    const unsigned fb = (unsigned)(u >> 17);
    memcpy(&fx, &fb, 4);
    if (!std::isnan(fx) && widen(fx) != (double)fx) bad_widen++;
  }
  // every float exponent class once more: zeros, subnormals, normals, infinities
  const unsigned edge[] = { 0u, 0x80000000u, 1u, 0x807fffffu, 0x00800000u, 0x7f7fffffu,
                            0x7f800000u, 0xff800000u, 0x3f800000u, 0xbf800001u };
  for (unsigned b : edge) {
    float fx;
    memcpy(&fx, &b, 4);
    if (widen(fx) != (double)fx) bad_widen++;
  }
  printf("%ld %ld %ld %ld\n", checked, bad_lo, bad_err, bad_widen);
  return 0;
}
