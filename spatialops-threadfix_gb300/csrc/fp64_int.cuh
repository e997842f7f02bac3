// Fixed-point helpers of the library's FP64 kernels: the exp and sin of NeboFixMath.h, 128-bit
// fixed-point plane sums (the box filter) and the quotient helpers of the particle operators.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#include <spatialops/NeboFixMath.h>

namespace nebo {
namespace fixmath {

#ifdef __CUDACC__
// Biased exponent of a double (integer pipe).
__device__ __forceinline__ int dexp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }

// 128-bit fixed point for exact sums of doubles that share one scale.  A plane (tile) whose
// largest biased exponent is E counts in units of 2^(E-1144): |x| < 2^(E-1022) becomes an
// integer below 2^122, sums of up to 32 of them stay below 2^127, and every x down to 2^-69 of
// the plane's largest keeps all of its 53 bits.  Integer pipe only; host and device (the host
// build is what tests/cpp/fixpoint_host.cu checks against exact rational arithmetic).
typedef __int128 fix128;

__host__ __device__ __forceinline__ fix128 make128(long long hi, unsigned long long lo) {
  return (fix128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}

// x (biased exponent <= E, not inf/NaN) in units of 2^(E-1144), rounded to nearest (halves up):
// the 53-bit significand m lands at bit sh = e - E + 69 <= 69 of a 128-bit integer.
__host__ __device__ __forceinline__ fix128 to_units(double x, int E) {
  const long long b = (long long)bits(x);
  const int e = (int)((b >> 52) & 0x7ff);
  const unsigned long long m = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
  const int sh = (e ? e : 1) - E + 69;
  unsigned long long hi, lo;
  if (sh >= 64) {
    hi = m << (sh - 64);
    lo = 0;
  } else if (sh > 0) {
    hi = m >> (64 - sh);
    lo = m << sh;
  } else {
    hi = 0;
    lo = sh == 0 ? m : (-sh > 62 ? 0ull : (m + (1ull << (-sh - 1))) >> -sh);
  }
  const fix128 f = make128((long long)hi, lo);
  return b < 0 ? -f : f;
}

// RN(t 2^u) for t != 0, assuming the result is normal.
__host__ __device__ __forceinline__ double units_to_double(fix128 t, int u) {
  const bool neg = t < 0;
  const unsigned __int128 a = neg ? (unsigned __int128)(-t) : (unsigned __int128)t;
  const unsigned long long hi = (unsigned long long)(a >> 64), lo = (unsigned long long)a;
  unsigned long long top, rest;
  int msb;  // position of the leading bit
  if (hi) {
    const int lz = clz64(hi);
    top = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;
    rest = lo << lz;  // bits below `top` (only whether any is set matters)
    msb = 127 - lz;
  } else {
    const int lz = clz64(lo);
    top = lo << lz;
    rest = 0;
    msb = 63 - lz;
  }
  unsigned long long mant = top >> 11;  // 53 bits
  const unsigned long long rb = top & 0x7ffull;
  const bool up = rb > 0x400ull || (rb == 0x400ull && (rest != 0 || (mant & 1ull)));
  int ex = msb + u + 1023;
  mant += up ? 1ull : 0ull;
  if (mant >> 53) {
    mant >>= 1;
    ++ex;
  }
  const unsigned long long out = ((unsigned long long)neg << 63) | ((unsigned long long)ex << 52) |
                                 (mant & 0xFFFFFFFFFFFFFull);
  return from_bits(out);
}

// RN(t 2^u), +0 for t == 0, assuming a nonzero result is normal.
__host__ __device__ __forceinline__ double units_to_double0(fix128 t, int u) {
  return t == 0 ? 0.0 : units_to_double(t, u);
}

// A divisor whose reciprocal div_by may use: positive, exponent within 2^+-400 (integer pipe).
__device__ __forceinline__ bool divisor_ok(double b) {
  const int e = dexp(b);
  return __double_as_longlong(b) >= 0 && e >= 1023 - 400 && e <= 1023 + 400;
}

// RN(a / b) given y = RN(1/b) (one reciprocal serves many quotients by the same b).
//
// Main path (a, b > 0, everything normal): q0 = RN(a y) is within 1.5 ulps of a/b (y is within
// half an ulp of 1/b).  With a = A 2^(ea-1075), b = B 2^(eb-1075), q0 = Q 2^(eq-1075) (A, B, Q
// the 53-bit integer significands), the remainder a - q0 b equals 2^(eq+eb-2150) R with
// R = A 2^s - Q B, s = ea - eq - eb + 1075, and (a/b - q0) / ulp(q0) = R / B.  |R| < 1.5 B < 2^55,
// so R is exact in 64-bit integer arithmetic (modulo 2^64), and RN(a/b) = q0 + k ulp with k the
// integer nearest R / B (a quotient of two doubles is never a tie).  When q0 lies within two
// ulps of its binade's ends the step k ulp could cross the binade; those quotients, and every
// other case, take the second path.
//
// Second path: two FMA corrections q' = RN(q + (a - b q) y).  By Markstein's theorem
// (P. W. Markstein, "Computation of elementary functions on the IBM RISC System/6000 processor",
// IBM J. Res. Dev. 34(1), 1990), when y is within half an ulp of 1/b and q within one ulp of
// a/b, a - b q is exact and q' = RN(a/b); the first correction brings q0 within one ulp.  Used
// where a / b and every intermediate stay normal (b_ok: divisor_ok(b); a's exponent within
// 2^+-500; a zero quotient is a * y); anywhere else the division itself.
__device__ __forceinline__ double div_by(double a, double b, double y, bool b_ok) {
  const double q0 = __dmul_rn(a, y);
  const long long ab = __double_as_longlong(a), bb = __double_as_longlong(b), qb = __double_as_longlong(q0);
  const int ea = (int)((ab >> 52) & 0x7ff), eb = (int)((bb >> 52) & 0x7ff), eq = (int)((qb >> 52) & 0x7ff);
  const unsigned long long frac = 0xFFFFFFFFFFFFFull, one = 1ull << 52;
  const unsigned long long mq = (unsigned long long)qb & frac;
  const int s = ea - eq - eb + 1075;
  if (b_ok && ab > 0 && ea >= 1 && ea <= 2046 && eq >= 1 && eq <= 2046 && mq >= 2 && mq <= frac - 2 && s >= 40 &&
      s <= 62) {
    const unsigned long long A = ((unsigned long long)ab & frac) | one, B = ((unsigned long long)bb & frac) | one;
    const unsigned long long Q = mq | one;
    const long long R = (long long)((A << s) - Q * B);
    const long long k = (long long)(2 * R > (long long)B) - (long long)(2 * R < -(long long)B);
    return __longlong_as_double(qb + k);
  }
  if (b_ok && ea >= 1023 - 500 && ea <= 1023 + 500) {
    const double q1 = __fma_rn(__fma_rn(-q0, b, a), y, q0);
    return __fma_rn(__fma_rn(-q1, b, a), y, q1);
  }
  if (b_ok && a == 0.0) return q0;
  return __ddiv_rn(a, b);
}
#endif

}  // namespace fixmath
}  // namespace nebo
