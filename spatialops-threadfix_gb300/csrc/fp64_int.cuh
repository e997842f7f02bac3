// FP64 exp and sin evaluated mostly on the integer pipe.
//
// On this GPU an FP64 instruction issues at about 1/64 of the FP32 rate, while 32-bit integer
// multiply-adds, shifts and logic issue at 64 lanes per clock per SM, so a kernel whose time goes
// to FP64 transcendentals runs faster when the polynomial work moves to 64-bit fixed point.  Only
// the argument reduction stays in FP64 (three instructions, for the exact Cody-Waite product).
//
// exp(x), |x| < 708   Tang's table method (P. T. P. Tang, ACM TOMS 15(2), 1989):
//     x = (64 m + j) ln2/64 + r,  |r| <= ln2/128 (+ rounding),
//     exp(x) = 2^m * 2^(j/64) * (1 + p(r)),   p(r) = r + r^2/2 + ... + r^6/720 (Taylor; the first
//     dropped term r^7/5040 < 2^-64).  k = 64 m + j from the FP64 product x * 64/ln2; the exact
//     r1 = x - k*L1 in FP64 (L1 = ln2/64 to 29 bits, so k*L1 is exact for |k| < 2^24); then
//     r = r1 - k*L2 in fixed point (L2 = ln2/64 - L1 to 2^-102).  p, 2^(j/64)*(1 + p) and the
//     rounding to a double run in signed 64-bit fixed point with 62 fraction bits.
// sin(x), |x| < 2^20  x = k pi/64 + r,  |r| <= pi/128:
//     sin(x) = S_k cos r + C_k sin r  with S_k, C_k = sin, cos(k pi/64) (128-entry table),
//     sin r = r (1 - u/6 + u^2/120 - u^3/5040), cos r = 1 - u/2 + u^2/24 - u^3/720 + u^4/40320,
//     u = r^2 (Taylor; dropped terms below 2^-66 and 2^-71).  r1 = x - k*A1 exactly in FP64
//     (A1 = pi/64 to 27 bits), r = r1 - k*A23 in fixed point (A23 = pi/64 - A1 to 2^-96).  When
//     k is a multiple of 64 the result is +-sin r, which can be tiny: then r is formed in FP64
//     (three more FMAs with pi/64 in four parts, 2^-173) and sin r = r * (1 - u/6 + ...) is a
//     floating product of r's significand.
// Everything else -- |x| beyond those ranges, NaN, infinities -- goes to CUDA's exp and sin.
//
// Fixed-point products keep the high bits: mulq(a, b) = floor(a*b / 2^62) up to 3 units of
// 2^-62 (the high word shifted; used inside the polynomials, whose errors are scaled down by r),
// mulx(a, b) = floor(a*b / 2^62) exactly (high and low words; used where the error would reach the
// result).  The error bound of both functions stays below one ulp; the tests compare them with
// CUDA's exp and sin (at most 2 ulp apart) on random and edge inputs.
//
// The tables (2^(j/64), sin and cos of k pi/64 in fixed point) are computed on the host in long
// double and uploaded once per device; the functions are __host__ __device__ so the host can run
// the same integer arithmetic.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>

namespace nebo {
namespace fixmath {

struct Tables {
  int64_t exp2j[64];   // round(2^(j/64) * 2^62)
  int64_t sink[128];   // round(sin(k pi/64) * 2^62)
  int64_t cosk[128];   // round(cos(k pi/64) * 2^62)
};

constexpr int64_t ONE = (int64_t)1 << 62;
// ln2/64 - L1 at 2^-102 and pi/64 - A1 at 2^-96 (computed with 300-bit arithmetic)
constexpr int64_t L2_FIX102 = -3328307820869995624LL;
constexpr int64_t A23_FIX96 = 2456304730009003561LL;

inline void fill_tables(Tables* t) {
  for (int j = 0; j < 64; ++j) t->exp2j[j] = (int64_t)llroundl(exp2l((long double)j / 64.0L) * 4611686018427387904.0L);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int k = 0; k < 128; ++k) {
    t->sink[k] = (int64_t)llroundl(sinl((long double)k * pi / 64.0L) * 4611686018427387904.0L);
    t->cosk[k] = (int64_t)llroundl(cosl((long double)k * pi / 64.0L) * 4611686018427387904.0L);
  }
  // exact values at multiples of pi/2
  const int64_t qs[4] = {0, ONE, 0, -ONE}, qc[4] = {ONE, 0, -ONE, 0};
  for (int i = 0; i < 4; ++i) {
    t->sink[32 * i] = qs[i];
    t->cosk[32 * i] = qc[i];
  }
}

__host__ __device__ __forceinline__ int64_t hi_s(int64_t a, int64_t b) {
#ifdef __CUDA_ARCH__
  return __mul64hi(a, b);
#else
  return (int64_t)(((__int128)a * (__int128)b) >> 64);
#endif
}
__host__ __device__ __forceinline__ uint64_t hi_u(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * (unsigned __int128)b) >> 64);
#endif
}
__host__ __device__ __forceinline__ int clz64(uint64_t a) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)a);
#else
  return a ? __builtin_clzll(a) : 64;
#endif
}
__host__ __device__ __forceinline__ uint64_t bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}
__host__ __device__ __forceinline__ double from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

// a*b / 2^62, high word only (error < 4 units of 2^-62)
__host__ __device__ __forceinline__ int64_t mulq(int64_t a, int64_t b) { return hi_s(a, b) * 4; }
// floor(a*b / 2^62)
__host__ __device__ __forceinline__ int64_t mulx(int64_t a, int64_t b) {
  return (int64_t)(((uint64_t)hi_s(a, b) << 2) | (((uint64_t)a * (uint64_t)b) >> 62));
}

// A finite double with |v| < 2 as fixed point with 62 fraction bits (truncated toward zero).
__host__ __device__ __forceinline__ int64_t to_fix(double v) {
  const uint64_t b = bits(v);
  const int e = (int)((b >> 52) & 0x7ff);
  const uint64_t m = (b & 0xfffffffffffffULL) | 0x10000000000000ULL;
  const int sh = e - 1013;  // v = m * 2^(e - 1075), fixed = v * 2^62
  uint64_t f;
  if (sh >= 0)
    f = m << sh;
  else
    f = sh > -64 ? m >> -sh : 0;
  if (e == 0) f = 0;
  return (b >> 63) ? -(int64_t)f : (int64_t)f;
}

// k * C / 2^s for a signed 32-bit k and a positive 62-bit constant C, 32 <= s < 64 (floor).
template <int S>
__host__ __device__ __forceinline__ int64_t mul_k(int k, int64_t c) {
  const int64_t hi = (int64_t)k * (c >> 32);                     // |.| < 2^(31+30)
  const int64_t lo = (int64_t)k * (int64_t)(uint32_t)c;          // |.| < 2^63
  return (hi + (lo >> 32)) >> (S - 32);
}

// Positive fixed-point y (62 fraction bits, y < 2^63) times 2^e as a double, rounded to nearest.
// The result must be a normal number.
__host__ __device__ __forceinline__ uint64_t fix_to_bits(uint64_t y, int e) {
  const int lz = clz64(y);
  const uint64_t yn = y << lz;                     // top bit at 63
  const uint64_t m = (yn >> 11) + ((yn >> 10) & 1);  // rounded 53-bit significand (2^53 on carry)
  // value = (yn / 2^63) * 2^(1 - lz + e); the implicit bit of m adds one to the exponent field
  return ((uint64_t)(e + 1 - lz + 1022) << 52) + m;
}

template <class T>
__host__ __device__ __forceinline__ double exp_fix(double x, const T& tb) {
  const uint64_t xb = bits(x);
  if ((uint32_t)(xb >> 32 & 0x7fffffffu) >= 0x40862000u) {  // |x| >= 708, inf, NaN
#ifdef __CUDA_ARCH__
    return exp(x);
#else
    return std::exp(x);
#endif
  }
  const double shifter = 6755399441055744.0;  // 1.5 * 2^52
  const double t = fma(x, 92.33248261689366, shifter);  // x * 64/ln2 rounded to an integer
  const int k = (int)(uint32_t)bits(t);
  const double kd = t - shifter;
  const double r1 = fma(-kd, 0.010830424696905538, x);  // exact: L1 has 29 significant bits
  const int64_t r = to_fix(r1) - mul_k<40>(k, L2_FIX102);
  // p = r + r^2 (1/2 + r (1/6 + r (1/24 + r (1/120 + r/720))))
  int64_t h = 6405119470038039LL;                  // 1/720
  h = 38430716820228233LL + mulq(r, h);           // 1/120
  h = 192153584101141163LL + mulq(r, h);          // 1/24
  h = 768614336404564651LL + mulq(r, h);          // 1/6
  h = 2305843009213693952LL + mulq(r, h);         // 1/2
  const int64_t p = r + mulq(mulq(r, r), h);
  const int64_t tj = tb.exp2j[k & 63];
  const uint64_t y = (uint64_t)(tj + mulx(tj, p));
  return from_bits(fix_to_bits(y, k >> 6));
}

template <class T>
__host__ __device__ __forceinline__ double sin_fix(double x, const T& tb) {
  const uint64_t xb = bits(x);
  if ((uint32_t)(xb >> 32 & 0x7fffffffu) >= 0x41300000u) {  // |x| >= 2^20, inf, NaN
#ifdef __CUDA_ARCH__
    return sin(x);
#else
    return std::sin(x);
#endif
  }
  const double shifter = 6755399441055744.0;
  const double t = fma(x, 20.371832715762604, shifter);  // x * 64/pi rounded to an integer
  const int k = (int)(uint32_t)bits(t);
  const double kd = t - shifter;
  const double r1 = fma(-kd, 0.049087385181337595, x);  // exact: A1 has 27 significant bits
  const int q = k & 127;
  if ((k & 63) == 0) {
    // +-sin r with r possibly tiny: r in FP64, then r * S(u) as a product of significands
    double rd = fma(-kd, 3.100292418622974e-11, r1);
    rd = fma(-kd, 1.7878714769093224e-19, rd);
    rd = fma(-kd, 1.3549703328318407e-36, rd);  // pi/64 in four parts: x near j*pi keeps its digits
    const uint64_t rb = bits(rd) ^ ((uint64_t)(q >> 6) << 63);  // sin(r + pi) = -sin r
    const int er = (int)((rb >> 52) & 0x7ff);
    if (er < 1023 - 26) return from_bits(rb);                   // |r| < 2^-26: sin r = r
    const int64_t rf = to_fix(rd);
    const int64_t u = mulq(rf, rf);
    int64_t s = -915017067148291LL;                 // -1/5040
    s = 38430716820228233LL + mulq(u, s);           // 1/120
    s = -768614336404564651LL + mulq(u, s);         // -1/6
    s = ONE + mulq(u, s);
    const uint64_t mr = ((rb & 0xfffffffffffffULL) | 0x10000000000000ULL) << 11;  // top bit 63
    const uint64_t pr = hi_u(mr, (uint64_t)s << 1);  // |r| significand * S, top bit 62 or 63
    const int lz = clz64(pr);
    const uint64_t pn = pr << lz;
    const uint64_t m = (pn >> 11) + ((pn >> 10) & 1);
    // sin r = (pn / 2^63) * 2^(er - 1022 - lz); m's implicit bit adds one to the exponent field
    return from_bits((rb & 0x8000000000000000ULL) | (((uint64_t)(er - lz) << 52) + m));
  }
  const int64_t r = to_fix(r1) - mul_k<34>(k, A23_FIX96);
  const int64_t u = mulq(r, r);
  int64_t s = -915017067148291LL;                   // -1/5040
  s = 38430716820228233LL + mulq(u, s);             // 1/120
  s = -768614336404564651LL + mulq(u, s);           // -1/6
  const int64_t sr = r + mulx(r, mulq(u, s));       // sin r
  int64_t c = 114377133393536LL;                    // 1/40320
  c = -6405119470038039LL + mulq(u, c);             // -1/720
  c = 192153584101141163LL + mulq(u, c);            // 1/24
  c = -2305843009213693952LL + mulq(u, c);          // -1/2
  const int64_t cm = mulx(u, c);                    // cos r - 1
  const int64_t sk = tb.sink[q], ck = tb.cosk[q];
  const int64_t v = sk + mulx(sk, cm) + mulx(ck, sr);
  const uint64_t sign = (uint64_t)v & 0x8000000000000000ULL;
  return from_bits(sign | fix_to_bits((uint64_t)(v < 0 ? -v : v), 0));
}

#ifdef __CUDACC__
// Device copy of the tables (one per device, uploaded by tables_init).
static __device__ Tables g_fix_tables;

inline int tables_init() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  std::lock_guard<std::mutex> g(mu);
  if (done[dev]) return 0;
  Tables h;
  fill_tables(&h);
  if (cudaMemcpyToSymbol(g_fix_tables, &h, sizeof(h)) != cudaSuccess) return 1;
  done[dev] = true;
  return 0;
}

__device__ __forceinline__ double exp_i(double x) { return exp_fix(x, g_fix_tables); }
__device__ __forceinline__ double sin_i(double x) { return sin_fix(x, g_fix_tables); }
#endif

}  // namespace fixmath
}  // namespace nebo
