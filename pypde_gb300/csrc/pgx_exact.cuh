// Exact scalings by a power of two without the FP64 pipe.
//
// On GB300 an SM sub-partition retires one FP64 warp instruction per ~64 cycles, while integer
// instructions issue every cycle on another pipe.  Multiplying by +-1/2 is exact in binary floating
// point except for results below the normal range, so it can be done on the bit pattern: the
// exponent field drops by one; a subnormal or smallest-normal operand has its significand (with
// the hidden bit) halved and rounded to nearest, ties to even, as the FP64 multiply rounds it.
// Zeros keep their sign, infinities stay infinite, NaNs stay NaNs.  The result equals
// x * (neg ? -0.5 : 0.5) bit for bit for every non-NaN x.
#ifndef PGX_EXACT_CUH
#define PGX_EXACT_CUH

#include <stdint.h>

#ifdef __CUDACC__
#define PGX_HD __host__ __device__ __forceinline__
#else
#define PGX_HD inline
#endif

#if defined(__CUDA_ARCH__)
PGX_HD int64_t pgx_bits_of(double x) { return __double_as_longlong(x); }
PGX_HD double pgx_double_of(int64_t b) { return __longlong_as_double(b); }
#else
#include <string.h>
PGX_HD int64_t pgx_bits_of(double x) {
  int64_t b;
  memcpy(&b, &x, sizeof b);
  return b;
}
PGX_HD double pgx_double_of(int64_t b) {
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
}
#endif

PGX_HD double pgx_half_signed(double x, bool neg) {
  const int64_t kExp = 0x7FF0000000000000LL, kOne = 0x0010000000000000LL, kMan = 0x000FFFFFFFFFFFFFLL;
  const int64_t kSign = (int64_t)0x8000000000000000ULL;
  int64_t b = pgx_bits_of(x);
  const int64_t e = b & kExp;
  if (e > kOne && e != kExp) {
    b -= kOne;  // normal result: one less in the exponent field
  } else if (e != kExp) {
    // zero, subnormal or the smallest normal exponent: halve the significand, round half to even
    const int64_t m = (b & kMan) | (e ? kOne : 0);
    int64_t h = m >> 1;
    if ((m & 1) && (h & 1)) ++h;
    b = (b & kSign) | h;  // h <= 2^52: a carry into bit 52 is the smallest normal number, as it should be
  }
  if (neg) b ^= kSign;
  return pgx_double_of(b);
}

#undef PGX_HD
#endif  // PGX_EXACT_CUH
