// Host run of the integer-pipe exp and sin (spatialops-threadfix_gb300/csrc/fp64_int.cuh): the
// same fixed-point arithmetic compiled for the CPU, checked against long double expl / sinl.
// Prints one line per range: "<name> <max ulp> <worst x>".
#include <cmath>
#include <cstdio>
#include <random>

#include "../../spatialops-threadfix_gb300/csrc/fp64_int.cuh"

using namespace nebo::fixmath;

static double ulp_err(double got, long double ref) {
  if (ref == 0) return got == 0 ? 0 : 1e9;
  int e;
  frexpl(fabsl(ref), &e);
  long double ulp = ldexpl(1.0L, e - 53);
  return (double)(fabsl((long double)got - ref) / ulp);
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 200000;
  static Tables tables;
  fill_tables(&tables);
  const HostTables T{&tables};
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
  return 0;
}
