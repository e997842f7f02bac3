// Deterministic inputs shared by every program that runs the expression catalog.
//
// Values come from a counter-based splitmix64 hash, so the same (type, index, cell) gives the
// same double on any machine and in numpy (tests/nebo_inputs.py restates it).  Only names that
// both the reference's headers and the drop-in headers define are used here.
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace catalog {

static const double CATALOG_SENTINEL_VALUE = -7777.25;

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

// uniform in [-1, 1): 53 random bits scaled exactly
inline double uniform_pm1(uint64_t stream, uint64_t i) {
  const uint64_t h = splitmix64(splitmix64(stream) + i);
  return (double)(h >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

inline uint64_t field_stream(int type_code, int k, int domain) {
  return (uint64_t)(1000003 * type_code + 7919 * k + 104729 * domain + 17);
}

// Mask k over a window of glob dims g with `ghost` ghost layers: every cell whose hash
// falls below 1/5, in interior-relative coordinates (ghost cells included).
inline std::vector<int> mask_points(int k, int domain, const int n[3], int ghost) {
  std::vector<int> pts;
  const uint64_t stream = field_stream(99, k, domain);
  int idx = 0;
  for (int z = -ghost; z < n[2] + ghost; ++z)
    for (int y = -ghost; y < n[1] + ghost; ++y)
      for (int x = -ghost; x < n[0] + ghost; ++x, ++idx) {
        if (uniform_pm1(stream, (uint64_t)idx) < -0.6) {
          pts.push_back(x);
          pts.push_back(y);
          pts.push_back(z);
        }
      }
  return pts;
}

}  // namespace catalog
