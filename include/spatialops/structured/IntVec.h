// IntVec: a triple of ints (drop-in for spatialops/structured/IntVec.h).
#ifndef SpatialOps_IntVec_h
#define SpatialOps_IntVec_h

#include <ostream>

#ifdef __CUDACC__
#define NEBO_HD __host__ __device__
#else
#define NEBO_HD
#endif

namespace SpatialOps {

class IntVec {
  int ijk_[3];

 public:
  NEBO_HD IntVec() : ijk_{0, 0, 0} {}
  NEBO_HD IntVec(int i, int j, int k) : ijk_{i, j, k} {}
  NEBO_HD IntVec(const int v[3]) : ijk_{v[0], v[1], v[2]} {}
  NEBO_HD int operator[](int i) const { return ijk_[i]; }
  NEBO_HD int& operator[](int i) { return ijk_[i]; }
  NEBO_HD bool operator==(const IntVec& o) const { return ijk_[0] == o[0] && ijk_[1] == o[1] && ijk_[2] == o[2]; }
  NEBO_HD bool operator!=(const IntVec& o) const { return !(*this == o); }
  NEBO_HD IntVec operator+(const IntVec& o) const { return IntVec(ijk_[0] + o[0], ijk_[1] + o[1], ijk_[2] + o[2]); }
  NEBO_HD IntVec operator-(const IntVec& o) const { return IntVec(ijk_[0] - o[0], ijk_[1] - o[1], ijk_[2] - o[2]); }
  NEBO_HD IntVec operator*(const IntVec& o) const { return IntVec(ijk_[0] * o[0], ijk_[1] * o[1], ijk_[2] * o[2]); }
  NEBO_HD IntVec operator/(const IntVec& o) const { return IntVec(ijk_[0] / o[0], ijk_[1] / o[1], ijk_[2] / o[2]); }
  NEBO_HD IntVec operator-() const { return IntVec(-ijk_[0], -ijk_[1], -ijk_[2]); }
  NEBO_HD IntVec& operator+=(const IntVec& o) { for (int i = 0; i < 3; ++i) ijk_[i] += o[i]; return *this; }
  NEBO_HD IntVec& operator-=(const IntVec& o) { for (int i = 0; i < 3; ++i) ijk_[i] -= o[i]; return *this; }
  NEBO_HD int prod() const { return ijk_[0] * ijk_[1] * ijk_[2]; }
};

NEBO_HD inline IntVec min(const IntVec& a, const IntVec& b) {
  return IntVec(a[0] < b[0] ? a[0] : b[0], a[1] < b[1] ? a[1] : b[1], a[2] < b[2] ? a[2] : b[2]);
}
NEBO_HD inline IntVec max(const IntVec& a, const IntVec& b) {
  return IntVec(a[0] > b[0] ? a[0] : b[0], a[1] > b[1] ? a[1] : b[1], a[2] > b[2] ? a[2] : b[2]);
}
inline std::ostream& operator<<(std::ostream& os, const IntVec& v) {
  return os << "[" << v[0] << "," << v[1] << "," << v[2] << "]";
}

}  // namespace SpatialOps
#endif
