// Host run of the integer-pipe exp and sin (include/spatialops/NeboFixMath.h): the
// same fixed-point arithmetic compiled for the CPU, checked against long double expl / sinl.
// Prints one line per range: "<name> <max ulp> <worst x>".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include <spatialops/NeboFixMath.h>

using namespace nebo::fixmath;

// the literal tables against long double: each entry within one unit of 2^-62 (long double
// rounding of the reference value)
static long table_mismatch() {
  const long double s62 = 4611686018427387904.0L;
  const long double pi = 3.141592653589793238462643383279502884L;
  long bad = 0;
  for (int j = 0; j < 256; ++j) bad += std::llabs(h_exp2j[j] - (long long)llroundl(exp2l(j / 256.0L) * s62)) > 1;
  for (int j = 0; j < 128; ++j) {
    bad += std::llabs(h_sinj[j] - (long long)llroundl(sinl(j * pi / 256.0L) * s62)) > 1;
    bad += std::llabs(h_cosj[j] - (long long)llroundl(cosl(j * pi / 256.0L) * s62)) > 1;
  }
  return bad;
}

static double ulp_err(double got, long double ref) {
  if (ref == 0) return got == 0 ? 0 : 1e9;
  int e;
  frexpl(fabsl(ref), &e);
  long double ulp = ldexpl(1.0L, e - 53);
  return (double)(fabsl((long double)got - ref) / ulp);
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 200000;
  const HostTables T;
  std::printf("table_mismatch %ld 0\n", table_mismatch());
  std::mt19937_64 g(12345);
  struct Range { const char* name; double lo, hi; int fn; } rs[] = {
      {"exp_unit", -1, 1, 0},     {"exp_full", -707.9, 707.9, 0}, {"exp_tiny", -1e-6, 1e-6, 0},
      {"sin_unit", -1, 1, 1},     {"sin_100", -100, 100, 1},      {"sin_1e5", -1e5, 1e5, 1},
      {"sin_tiny", -1e-8, 1e-8, 1}, {"sin_2p20", -1048575, 1048575, 1}};
  for (const Range& r : rs) {
    std::uniform_real_distribution<double> d(r.lo, r.hi);
    double mx = 0, worst = 0;
    for (long i = 0; i < n; ++i) {
      const double x = d(g);
      const double y = r.fn == 0 ? exp_fix(x, T) : sin_fix(x, T);
      const double e = ulp_err(y, r.fn == 0 ? expl((long double)x) : sinl((long double)x));
      if (e > mx) { mx = e; worst = x; }
    }
    std::printf("%s %.4f %.17g\n", r.name, mx, worst);
  }
  double mx = 0, worst = 0;  // doubles at and next to j*pi
  for (int j = 1; j < 333000; j += 7) {
    const double x = (double)((long double)j * 3.141592653589793238462643383279502884L);
    const double xs[3] = {x, std::nextafter(x, INFINITY), std::nextafter(x, -INFINITY)};
    for (double v : xs) {
      const double e = ulp_err(sin_fix(v, T), sinl((long double)v));
      if (e > mx) { mx = e; worst = v; }
    }
  }
  std::printf("sin_near_jpi %.4f %.17g\n", mx, worst);
  // conversions built from the bits: against the C casts on random bit patterns and edge values
  long bad_d2f = 0, bad_f2d = 0;
  std::uniform_int_distribution<uint64_t> bits64;
  for (long i = 0; i < 4 * n; ++i) {
    const uint64_t b = bits64(g);
    double v;
    std::memcpy(&v, &b, 8);
    const double av = std::fabs(v);
    if (std::isnan(v) || (av >= 1.1754943508222875e-38 && av < 3.4028234663852886e38) || av == 0.0) {
      const float want = (float)v, got = f64_to_f32_rn(v);
      if (std::memcmp(&want, &got, 4) != 0 && !(std::isnan(want) && std::isnan(got))) ++bad_d2f;
    }
    const uint32_t fb = (uint32_t)b;
    float f;
    std::memcpy(&f, &fb, 4);
    const double wd = (double)f, gd = f32_to_f64(f);
    if (std::memcmp(&wd, &gd, 8) != 0 && !(std::isnan(wd) && std::isnan(gd))) ++bad_f2d;
  }
  for (uint32_t fb : {0u, 0x80000000u, 1u, 0x80000001u, 0x007fffffu, 0x00400000u, 0x00800000u, 0x7f7fffffu,
                      0x7f800000u, 0xff800000u, 0x7fc00000u}) {
    float f;
    std::memcpy(&f, &fb, 4);
    const double wd = (double)f, gd = f32_to_f64(f);
    if (std::memcmp(&wd, &gd, 8) != 0 && !(std::isnan(wd) && std::isnan(gd))) ++bad_f2d;
  }
  std::printf("conv_d2f_mismatch %ld 0\nconv_f2d_mismatch %ld 0\n", bad_d2f, bad_f2d);
  return 0;
}
