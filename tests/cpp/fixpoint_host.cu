// Host build of the 128-bit fixed-point helpers of the box filter (fixmath::to_units,
// units_to_double, units_to_double0 in spatialops-threadfix_gb300/csrc/fp64_int.cuh): prints
// random inputs with the helpers' outputs so that tests/test_fixpoint_host.py can check them
// against exact rational arithmetic.  Runs on the CPU only (no CUDA call).
//   U <x bits> <E> <hi> <lo>      to_units(x, E) = hi * 2^64 + lo (two's complement)
//   D <hi> <lo> <u> <bits>        units_to_double(hi * 2^64 + lo, u)
//   Z <bits>                      units_to_double0(0, 5)
#include <cstdio>
#include <cstdlib>
#include <random>

#include "fp64_int.cuh"

using nebo::fixmath::fix128;

int main(int argc, char** argv) {
  const long count = argc > 1 ? std::atol(argv[1]) : 20000;
  std::mt19937_64 g(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 7);
  auto emit128 = [](fix128 v) {
    std::printf("%016llx %016llx", (unsigned long long)((unsigned __int128)v >> 64), (unsigned long long)v);
  };
  for (long i = 0; i < count; ++i) {
    // to_units: x with biased exponent <= E (subnormals and zeros included), E in [130, 2040]
    const int E = 130 + (int)(g() % 1911);
    const int span = (int)(g() % 4);  // how far below E the value sits: 0..2, or far
    int e = span == 3 ? (int)(g() % (E + 1)) : E - (int)(g() % 75);
    if (e < 0) e = 0;
    unsigned long long b = (g() & 0xFFFFFFFFFFFFFull) | ((unsigned long long)e << 52) | (g() & (1ull << 63));
    if (i % 97 == 0) b &= 1ull << 63;  // +-0
    const double x = nebo::fixmath::from_bits(b);
    std::printf("U %016llx %d ", b, E);
    emit128(nebo::fixmath::to_units(x, E));
    std::printf("\n");
    // units_to_double: nonzero t of 1..126 bits, a scale whose result is a normal double
    const int nb = 1 + (int)(g() % 126);
    unsigned __int128 m = ((unsigned __int128)g() << 64) | g();
    m &= (((unsigned __int128)1) << nb) - 1;
    m |= ((unsigned __int128)1) << (nb - 1);
    if (i % 13 == 0 && nb > 54) {  // an exact tie: 53 leading bits, then one half unit, then zeros
      m = (m >> (nb - 53)) << (nb - 53);
      m |= ((unsigned __int128)1) << (nb - 54);
    }
    fix128 t = (fix128)m;
    if (g() & 1) t = -t;
    const int lo_u = -1022 - (nb - 1) + 1, hi_u = 1023 - nb;
    const int u = lo_u + (int)(g() % (unsigned)(hi_u - lo_u + 1));
    std::printf("D ");
    emit128(t);
    std::printf(" %d %016llx\n", u, (unsigned long long)nebo::fixmath::bits(nebo::fixmath::units_to_double(t, u)));
  }
  std::printf("Z %016llx\n", (unsigned long long)nebo::fixmath::bits(nebo::fixmath::units_to_double0(0, 5)));
  return 0;
}
