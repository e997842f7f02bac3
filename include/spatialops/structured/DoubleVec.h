// DoubleVec: a triple of doubles (drop-in for spatialops/structured/DoubleVec.h, the
// Numeric3Vec<double> of spatialops/structured/Numeric3Vec.h).
#ifndef SpatialOps_DoubleVec_h
#define SpatialOps_DoubleVec_h

#include <cmath>
#include <limits>
#include <ostream>

#include <spatialops/structured/IntVec.h>

namespace SpatialOps {

class DoubleVec {
  double ijk_[3];

 public:
  DoubleVec() : ijk_{0, 0, 0} {}
  DoubleVec(double x, double y, double z) : ijk_{x, y, z} {}
  double operator[](int i) const { return ijk_[i]; }
  double& operator[](int i) { return ijk_[i]; }
  DoubleVec operator/(const IntVec& n) const { return DoubleVec(ijk_[0] / n[0], ijk_[1] / n[1], ijk_[2] / n[2]); }
  DoubleVec operator*(const DoubleVec& o) const { return DoubleVec(ijk_[0] * o[0], ijk_[1] * o[1], ijk_[2] * o[2]); }
  DoubleVec operator+(const DoubleVec& o) const { return DoubleVec(ijk_[0] + o[0], ijk_[1] + o[1], ijk_[2] + o[2]); }
  DoubleVec operator-(const DoubleVec& o) const { return DoubleVec(ijk_[0] - o[0], ijk_[1] - o[1], ijk_[2] - o[2]); }
  // equal within two machine epsilons per component, as the reference's specialisation
  bool operator==(const DoubleVec& o) const {
    const double eps = 2.0 * std::numeric_limits<double>::epsilon();
    return std::abs(o[0] - ijk_[0]) < eps && std::abs(o[1] - ijk_[1]) < eps && std::abs(o[2] - ijk_[2]) < eps;
  }
  bool operator!=(const DoubleVec& o) const { return !(*this == o); }
};

inline std::ostream& operator<<(std::ostream& os, const DoubleVec& v) {
  return os << "[" << v[0] << "," << v[1] << "," << v[2] << "]";
}

}  // namespace SpatialOps
#endif
