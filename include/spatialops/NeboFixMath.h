// FP64 exp and sin evaluated mostly outside the FP64 pipe (header-only, host and device).
//
// Measured on this GPU (per clock per SM): FP64 add/FMA and every conversion between FP64 and
// FP32 or integers about 2 (all on the FP64 pipe); unsigned 64-bit high product about 6; 64-bit
// integer add, logic, shift and compare 13-45 and 32-bit multiply-adds and FP32 arithmetic more
// (ALU and FMA pipes).  A kernel whose time goes to FP64 transcendentals therefore runs faster
// when (1) the FP64 pipe keeps only the one exact Cody-Waite product that needs all 53 bits of x,
// (2) the polynomials run in fixed point with as few 64-bit products as the error budget allows,
// (3) the low-order terms use FP32 or 32x32-bit products, and (4) the few FP64<->FP32/integer
// conversions are built from the bits with integer operations.
//
// exp(x), |x| < 708   Tang's table method (P. T. P. Tang, ACM TOMS 15(2), 1989) with 256 entries:
//     x = (256 m + j) ln2/256 + r,  |r| <= ln2/512 (+0.02 % from the FP32 rounding of k),
//     exp(x) = 2^m * 2^(j/256) * (1 + p),  p = r + r^2 (1/2 + r (1/6 + r (1/24 + r/120)))
//     (Taylor; the dropped r^6/720 < 2^-66).  k = round(x * 256/ln2) in FP32 (any k within one of
//     the nearest works); r1 = x - k*L1 exactly in FP64 (L1 = ln2/256 to 35 bits, so k*L1 is exact
//     for |k| < 2^18); r = r1 - k*L2 in fixed point (L2 = ln2/256 - L1 to 2^-104).  The inner
//     factors 1/24 + r/120 (FP32) and 1/6 + r*(...), 1/2 + r*(...) (32x32-bit products) need few
//     bits; r^2, r^2*(...) and 2^(j/256)*(1 + p) are 64-bit products; the result is rounded to a
//     double from the 62-fraction-bit fixed point.
// sin(x), |x| < 2^20  x = k pi/256 + r,  |r| <= pi/512 (+1 % from the FP32 rounding of k):
//     sin(x) = S_k (1 + (cos r - 1)) + C_k sin r,  S_k, C_k = sin, cos(k pi/256) from a 128-entry
//     quarter table and the quadrant of k;  sin r = r (1 - u/6 + u^2/120),
//     cos r - 1 = -u/2 + u^2/24 - u^3/720,  u = r^2 (Taylor; dropped terms below 2^-70).
//     k in FP32 for |x| < 4096, else in FP64 (two more instructions); r1 = x - k*A1 exactly in
//     FP64 (A1 = pi/256 to 26 bits, exact for |k| < 2^26.3); r = r1 - k*A23 in fixed point
//     (A23 = pi/256 - A1 to 2^-94).  When k is a multiple of 256 (x near j*pi) the result is
//     +-sin r and may be tiny: r is then formed in FP64 from pi/256 in four parts (error 2^-170)
//     and sin r = r * (1 - u/6 + u^2/120) is a product of r's significand.
// Everything else -- |x| beyond those ranges, NaN, infinities -- goes to CUDA's exp and sin.
//
// Fixed point: signed or unsigned 64-bit integers with 62 fraction bits ("at 2^62").  Error: exp
// within 0.52 ulp, sin within about 1.1 ulp (the FP64 rounding of r before the final rounding in
// the multiple-of-pi branch; fixed-point roundings where |sin x| is near sin(pi/512), whose ulp is
// 4 units of 2^-62); the tests compare both with long double on the host and with CUDA's
// functions on the device.
//
// The tables (2^(j/256); sin and cos of j pi/256, j < 128, at 2^62) are literals generated by
// spatialops-threadfix_gb300/gen_fixmath_tables.py in 400-bit arithmetic
// (detail/NeboFixMathTables.h): each translation unit that includes this header holds its own
// statically initialised device copy, so nothing is set up or uploaded at run time.  Every
// function is __host__ __device__, so the host runs the same integer arithmetic in the CPU tests.
//
// Used by the library's deep chain (nebo_deep_chain) and by the drop-in expression engine for
// exp and sin of FP64 fields in `<<=` expressions.
#ifndef SpatialOps_NeboFixMath_h
#define SpatialOps_NeboFixMath_h

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#include <spatialops/detail/NeboFixMathTables.h>

namespace nebo {
namespace fixmath {

constexpr int64_t ONE = (int64_t)1 << 62;
constexpr int64_t HALF = (int64_t)1 << 61;
constexpr int64_t SIXTH = 768614336404564651LL;                 // 2^62 / 6
constexpr uint64_t SIXTH64 = 0x2AAAAAAAAAAAAAABULL;            // 2^64 / 6, rounded up
constexpr uint32_t C24 = 178956971u;                            // 2^32 / 24
constexpr uint32_t C120 = 35791394u;                            // 2^32 / 120
constexpr uint32_t C720 = 5965232u;                             // 2^32 / 720
// ln2/256 = L1 + L2: L1 to 35 significant bits, L2 at 2^-104.  pi/256 = A1 + A23: A1 to 26
// bits, A23 at 2^-94; A23 = A2 + A3 + A4 as doubles (A2 to 26 bits).  (300-bit arithmetic.)
constexpr double L1 = 0.0027076061741126978;
constexpr int64_t L2_FIX104 = -1022464811656301672LL;
constexpr double A1 = 0.01227184641174972;
constexpr int64_t A23_FIX94 = -2152323963588131229LL;
constexpr double A2 = -1.0866459121405825e-10, A3 = 4.783776559169348e-19, A4 = -1.1698319569212264e-35;

// ------------------------------------------------------------------ integer helpers
__host__ __device__ __forceinline__ uint64_t umulhi(uint64_t a, uint64_t b) {
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
__host__ __device__ __forceinline__ int fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_int(x);
#else
  int b;
  std::memcpy(&b, &x, 4);
  return b;
#endif
}
__host__ __device__ __forceinline__ uint64_t uabs(int64_t a) { return a < 0 ? 0 - (uint64_t)a : (uint64_t)a; }

// a * b / 2^62 for a, b >= 0: high word only (truncation below 4 units of 2^-62), and rounded to
// nearest (the full 128-bit product plus one half, a < 2^64, a * b < 2^126).  ssq: a^2 / 2^62
// truncated like umulq, from the signed high word (a^2 = |a|^2, so the same bits as umulq(|a|, |a|)).
__host__ __device__ __forceinline__ uint64_t umulq(uint64_t a, uint64_t b) { return umulhi(a, b) << 2; }
__host__ __device__ __forceinline__ uint64_t ssq(int64_t a) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__mul64hi(a, a) << 2;
#else
  return (uint64_t)(((__int128)a * (__int128)a) >> 64) << 2;
#endif
}
__host__ __device__ __forceinline__ uint64_t umulx(uint64_t a, uint64_t b) {
  const uint64_t lo = a * b, lo2 = lo + (1ULL << 61);
  return ((umulhi(a, b) + (lo2 < lo)) << 2) | (lo2 >> 62);
}
// signed a * b / 2^62 rounded to nearest (halves up), from the signed 128-bit product
// (|a * b| < 2^125)
__host__ __device__ __forceinline__ int64_t smulx(int64_t a, int64_t b) {
#ifdef __CUDA_ARCH__
  const uint64_t lo = (uint64_t)a * (uint64_t)b;
  const int64_t hi = __mul64hi(a, b);
#else
  const __int128 pr = (__int128)a * (__int128)b;
  const uint64_t lo = (uint64_t)pr;
  const int64_t hi = (int64_t)(pr >> 64);
#endif
  const uint64_t lo2 = lo + (1ULL << 61);
  const uint64_t hi2 = (uint64_t)hi + (lo2 < lo);
  return (int64_t)((hi2 << 2) | (lo2 >> 62));
}

// A finite double with |v| < 2 at 2^62 (truncated toward zero; 0 for subnormals).
__host__ __device__ __forceinline__ int64_t to_fix(double v) {
  const uint64_t b = bits(v);
  const int e = (int)((b >> 52) & 0x7ff);
  const uint64_t m = (b & 0xfffffffffffffULL) | 0x10000000000000ULL;
  const int sh = e - 1013;  // v = m * 2^(e - 1075)
  uint64_t f = sh >= 0 ? m << sh : (sh > -64 ? m >> -sh : 0);
  if (e == 0) f = 0;
  return (b >> 63) ? -(int64_t)f : (int64_t)f;
}

// k * C / 2^S for a signed 32-bit k and a 62-bit signed constant C, 32 <= S < 64, rounded
// (|k * (C mod 2^32)| < 2^62).
template <int S>
__host__ __device__ __forceinline__ int64_t mul_k(int k, int64_t c) {
  const int64_t hi = (int64_t)k * (c >> 32);
  const int64_t lo = (int64_t)k * (int64_t)(uint32_t)c;
  const int64_t v = hi + ((lo + (1LL << 31)) >> 32);
  if (S == 32) return v;
  return (v + (1LL << (S - 33 > 0 ? S - 33 : 0))) >> (S - 32);
}

// Bits of the double y * 2^(e - 62) for 0 < y < 2^64, rounded to nearest (normal results only).
__host__ __device__ __forceinline__ uint64_t fix_to_bits(uint64_t y, int e) {
  const int lz = clz64(y);
  const uint64_t yn = y << lz;                       // top bit at 63
  const uint64_t m = (yn >> 11) + ((yn >> 10) & 1);  // 53-bit significand, 2^53 on carry-out
  // value = (yn / 2^63) * 2^(1 - lz + e); m's implicit bit adds one to the exponent field
  return ((uint64_t)(e + 1 - lz + 1022) << 52) + m;
}

__host__ __device__ __forceinline__ float from_fbits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, 4);
  return x;
#endif
}
__host__ __device__ __forceinline__ int clz32(uint32_t a) {
#ifdef __CUDA_ARCH__
  return __clz((int)a);
#else
  return a ? __builtin_clz(a) : 32;
#endif
}

// Conversions between FP64 and FP32 or integers issue on the FP64 pipe on this GPU (at the FP64
// rate), so the few this code needs are built from the bits with integer operations instead.
// v as a float, significand truncated (|v| < 2^128; |v| < 2^-126 gives +-0).
__host__ __device__ __forceinline__ float f32_trunc(double v) {
  const uint64_t b = bits(v);
  const uint32_t hi = (uint32_t)(b >> 32);
  const int e = (int)((hi >> 20) & 0x7ff);
  const uint32_t sign = hi & 0x80000000u;
  const uint32_t f = sign | ((uint32_t)(e - 896) << 23) | ((uint32_t)(b >> 29) & 0x7fffffu);
  return from_fbits(e > 896 ? f : sign);
}
// A float as a double, exactly (subnormals, zeros, infinities and NaNs included).
__host__ __device__ __forceinline__ double f32_to_f64(float f) {
  const uint32_t b = (uint32_t)fbits(f);
  const uint32_t e = (b >> 23) & 0xff, m = b & 0x7fffffu;
  const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
  const uint64_t normal = ((uint64_t)(e + 896) << 52) | ((uint64_t)m << 29);
  const uint64_t special = (0x7ffULL << 52) | ((uint64_t)m << 29);  // inf / NaN
  const int p = 31 - clz32(m);                                     // subnormal: m * 2^-149
  const uint64_t sub = m ? (((uint64_t)(874 + p) << 52) | (((uint64_t)m << (52 - p)) & 0xfffffffffffffULL)) : 0;
  return from_bits(sign | (e == 0 ? sub : (e == 0xff ? special : normal)));
}
// A double rounded to the nearest float, ties to even (the hardware's cvt.rn.f32.f64 for every
// result in the normal float range; results below 2^-126 in magnitude give +-0).
__host__ __device__ __forceinline__ float f64_to_f32_rn(double v) {
  const uint64_t b = bits(v);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff);
  const uint64_t m = b & 0xfffffffffffffULL;
  const uint32_t f = (uint32_t)(m >> 29);
  const uint32_t rem = (uint32_t)(m & 0x1fffffffu);
  const uint32_t up = (rem > 0x10000000u) || (rem == 0x10000000u && (f & 1u));
  uint32_t out = ((uint32_t)(e - 896) << 23) + f + up;  // a carry moves into the exponent
  if (e <= 896) out = 0;
  if (e >= 1151) out = 0x7f800000u;                      // overflow to infinity
  if (e == 2047 && m) out = 0x7fc00000u;                 // NaN
  return from_fbits(sign | out);
}

// k (|k| < 2^31) as a double.
__host__ __device__ __forceinline__ double i32_to_f64(int k) {
  const uint32_t a = k < 0 ? 0u - (uint32_t)k : (uint32_t)k;
  const int e = 31 - clz32(a);  // a's top bit
  const uint64_t m = ((uint64_t)a << (52 - e)) & 0xfffffffffffffULL;
  const uint64_t b = ((uint64_t)(k < 0) << 63) | ((uint64_t)(1023 + e) << 52) | m;
  return from_bits(a ? b : 0);
}

// k = round(x * c) (within one) through FP32, |x * c| < 2^22; kd = k as a double.
__host__ __device__ __forceinline__ int k_f32(double x, float c, double* kd) {
  const float t = fmaf(f32_trunc(x), c, 12582912.0f);  // 1.5 * 2^23
  const int k = fbits(t) - 0x4B400000;
  *kd = i32_to_f64(k);
  return k;
}

// ------------------------------------------------------------------ exp
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
  double kd;
  const int k = k_f32(x, 369.32992553710938f, &kd);  // 256/ln2
  const double r1 = fma(-kd, L1, x);                  // exact
  const int64_t r = to_fix(r1) - mul_k<42>(k, L2_FIX104);
  // g2 = 1/24 + r/120 in FP32, in [2^-5, 2^-4): its significand at 2^35 is exact
  const float g2 = fmaf(f32_trunc(r1), 1.0f / 120.0f, 1.0f / 24.0f);
  const int32_t g2f = (int32_t)(((uint32_t)fbits(g2) & 0x7fffffu) | 0x800000u) << 7;
  const int32_t r40 = (int32_t)(r >> 22);  // r at 2^40
  const int64_t g = SIXTH + (((int64_t)r40 * g2f) >> 13);               // 1/6 + r g2
  const int64_t h = HALF + (((int64_t)r40 * (int32_t)(g >> 30)) >> 10);  // 1/2 + r g
  const uint64_t u = ssq(r);                                            // r^2
  const int64_t p = r + (int64_t)umulq(u, (uint64_t)h);
  const int64_t tj = tb.e(k & 255);
  const uint64_t y = (uint64_t)(tj + smulx(tj, p));
  return from_bits(fix_to_bits(y, k >> 8));
}

// ------------------------------------------------------------------ sin
// -u/6 + u^2/120 and cos r - 1 = -u/2 + u^2/24 - u^3/720 at 2^62, from u = r^2 at 2^62 (u < 2^-14)
__host__ __device__ __forceinline__ void sin_cos_poly(uint64_t u, int64_t* sfac_m1, int64_t* cm1) {
  const uint32_t u46 = (uint32_t)(u >> 16);                          // u at 2^46
  const uint32_t uu60 = (uint32_t)(((uint64_t)u46 * u46) >> 32);      // u^2 at 2^60
  const int64_t u2_120 = (int64_t)(((uint64_t)uu60 * C120) >> 30);    // u^2/120 at 2^62
  const int64_t u2_24 = (int64_t)(((uint64_t)uu60 * C24) >> 30);      // u^2/24
  const uint64_t u3 = ((uint64_t)uu60 * u46) >> 44;                   // u^3 at 2^62
  const int64_t u3_720 = (int64_t)((u3 * C720) >> 32);               // u^3/720
  *sfac_m1 = -(int64_t)umulhi(u, SIXTH64) + u2_120;
  *cm1 = -(int64_t)(u >> 1) + u2_24 - u3_720;
}

template <class T>
__host__ __device__ __forceinline__ double sin_fix(double x, const T& tb) {
  const uint64_t xb = bits(x);
  const uint32_t hx = (uint32_t)(xb >> 32 & 0x7fffffffu);
  if (hx >= 0x41300000u) {  // |x| >= 2^20, inf, NaN
#ifdef __CUDA_ARCH__
    return sin(x);
#else
    return std::sin(x);
#endif
  }
  int k;
  double kd;
  if (hx < 0x40B00000u) {  // |x| < 4096
    k = k_f32(x, 81.4873275756836f, &kd);  // 256/pi
  } else {
    const double t = fma(x, 81.48733086305042, 6755399441055744.0);
    k = (int)(uint32_t)bits(t);
    kd = t - 6755399441055744.0;
  }
  const double r1 = fma(-kd, A1, x);  // exact
  const int q = (k >> 7) & 3;
  if ((k & 255) == 0) {
    // +-sin r, r possibly tiny: r in FP64 with pi/256 in four parts, then r * (1 - u/6 + u^2/120)
    double rd = r1;  // k = 0: r = x exactly (keeps the sign of -0)
    if (k != 0) {
      rd = fma(-kd, A2, rd);
      rd = fma(-kd, A3, rd);
      rd = fma(-kd, A4, rd);
    }
    const uint64_t rb = bits(rd) ^ ((uint64_t)(q >> 1) << 63);  // sin(r + pi) = -sin r
    const int er = (int)((rb >> 52) & 0x7ff);
    if (er < 1023 - 26) return from_bits(rb);                   // |r| < 2^-26: sin r = r
    const uint64_t ra = uabs(to_fix(rd));
    int64_t sm1, cm1;
    sin_cos_poly(umulq(ra, ra), &sm1, &cm1);
    const uint64_t s = (uint64_t)(ONE + sm1);                   // 1 - u/6 + u^2/120 <= 2^62
    const uint64_t mr = ((rb & 0xfffffffffffffULL) | 0x10000000000000ULL) << 11;  // top bit 63
    const uint64_t pr = umulhi(mr, s << 1);                    // top bit at 61..63
    const int lz = clz64(pr);
    const uint64_t pn = pr << lz;
    const uint64_t m = (pn >> 11) + ((pn >> 10) & 1);
    // sin r = (pn / 2^63) * 2^(er - 1022 - lz); m's implicit bit adds one to the exponent field
    return from_bits((rb & 0x8000000000000000ULL) | (((uint64_t)(er - lz) << 52) + m));
  }
  const int64_t r = to_fix(r1) - mul_k<32>(k, A23_FIX94);
  int64_t sm1, cm1;
  sin_cos_poly(ssq(r), &sm1, &cm1);
  const int64_t sr = r + smulx(r, sm1);  // sin r
  const int j = k & 127;
  const int64_t sj = tb.s(j), cj = tb.c(j);
  int64_t sk = (q & 1) ? cj : sj, ck = (q & 1) ? sj : cj;
  if (q & 2) sk = -sk;
  if ((q ^ (q >> 1)) & 1) ck = -ck;
  const int64_t v = sk + smulx(sk, cm1) + smulx(ck, sr);
  const uint64_t sign = (uint64_t)v & 0x8000000000000000ULL;
  return from_bits(sign | fix_to_bits(uabs(v), 0));
}


// Host copy of the tables.
static const int64_t h_exp2j[256] = NEBO_FIX_EXP2J;
static const int64_t h_sinj[128] = NEBO_FIX_SINJ;
static const int64_t h_cosj[128] = NEBO_FIX_COSJ;
struct HostTables {
  int64_t e(int j) const { return h_exp2j[j]; }
  int64_t s(int j) const { return h_sinj[j]; }
  int64_t c(int j) const { return h_cosj[j]; }
};

#ifdef __CUDACC__
// Device copy of the tables, statically initialised (each translation unit holds its own), read
// through the read-only data cache.
static __device__ const int64_t d_exp2j[256] = NEBO_FIX_EXP2J;
static __device__ const int64_t d_sinj[128] = NEBO_FIX_SINJ;
static __device__ const int64_t d_cosj[128] = NEBO_FIX_COSJ;

struct DeviceTables {
  __device__ __forceinline__ int64_t e(int j) const { return __ldg(&d_exp2j[j]); }
  __device__ __forceinline__ int64_t s(int j) const { return __ldg(&d_sinj[j]); }
  __device__ __forceinline__ int64_t c(int j) const { return __ldg(&d_cosj[j]); }
};

__device__ __forceinline__ double exp_i(double x) { return exp_fix(x, DeviceTables()); }
__device__ __forceinline__ double sin_i(double x) { return sin_fix(x, DeviceTables()); }
#endif

}  // namespace fixmath
}  // namespace nebo
#endif
