// GhostData: ghost-cell counts per face with Nebo's "infinite" marker for scalars
// (drop-in for spatialops/structured/GhostData.h; same algebra, GHOST_MAX = 9001).
#ifndef SpatialOps_GhostData_h
#define SpatialOps_GhostData_h

#include <ostream>
#include <stdexcept>

#include <spatialops/structured/IntVec.h>

#define GHOST_MAX 9001

namespace SpatialOps {

class GhostData {
  IntVec minus_, plus_;
  bool isInf_;
  static bool all_inf(const IntVec& v) { return v[0] >= GHOST_MAX && v[1] >= GHOST_MAX && v[2] >= GHOST_MAX; }

 public:
  GhostData(int nx, int px, int ny, int py, int nz, int pz)
      : minus_(nx, ny, nz), plus_(px, py, pz), isInf_(all_inf(minus_) && all_inf(plus_)) {}
  GhostData(const IntVec& minus, const IntVec& plus) : minus_(minus), plus_(plus), isInf_(all_inf(minus) && all_inf(plus)) {}
  GhostData(int n = 0) : minus_(n, n, n), plus_(n, n, n), isInf_(all_inf(minus_) && all_inf(plus_)) {}

  IntVec get_minus() const { return minus_; }
  int get_minus(int i) const { return minus_[i]; }
  IntVec get_plus() const { return plus_; }
  int get_plus(int i) const { return plus_[i]; }
  void set_minus(const IntVec& m) { minus_ = m; isInf_ = all_inf(minus_) && all_inf(plus_); }
  void set_plus(const IntVec& p) { plus_ = p; isInf_ = all_inf(minus_) && all_inf(plus_); }
  bool is_infinite() const { return isInf_; }

  GhostData& operator+=(const GhostData& r) {
    if (!isInf_) {
      if (r.isInf_) {
        *this = r;
      } else {
        minus_ += r.minus_;
        plus_ += r.plus_;
      }
    }
    return *this;
  }
  GhostData operator+(const GhostData& r) const { GhostData g(*this); g += r; return g; }
  GhostData& operator-=(const GhostData& r) {
    if (r.isInf_) throw std::runtime_error("Cannot use infinite ghost data on the right-hand side of subtraction.");
    minus_ -= r.minus_;
    plus_ -= r.plus_;
    return *this;
  }
  GhostData operator-(const GhostData& r) const { GhostData g(*this); g -= r; return g; }
  bool operator==(const GhostData& r) const { return minus_ == r.minus_ && plus_ == r.plus_; }
  bool operator!=(const GhostData& r) const { return !(*this == r); }

  GhostData limit_by_extent(const IntVec& e) const {
    return GhostData(e[0] <= 1 ? 0 : minus_[0], e[0] <= 1 ? 0 : plus_[0], e[1] <= 1 ? 0 : minus_[1],
                     e[1] <= 1 ? 0 : plus_[1], e[2] <= 1 ? 0 : minus_[2], e[2] <= 1 ? 0 : plus_[2]);
  }
};

inline GhostData min(const GhostData& a, const GhostData& b) {
  return GhostData(min(a.get_minus(), b.get_minus()), min(a.get_plus(), b.get_plus()));
}
inline GhostData point_to_ghost(const IntVec& v) {
  return GhostData(v[0] < 0 ? -v[0] : 0, v[0] > 0 ? v[0] : 0, v[1] < 0 ? -v[1] : 0, v[1] > 0 ? v[1] : 0,
                   v[2] < 0 ? -v[2] : 0, v[2] > 0 ? v[2] : 0);
}
inline GhostData reductive_point_to_ghost(const IntVec& v) {
  return GhostData(v[0] < 0 ? v[0] : 0, v[0] > 0 ? -v[0] : 0, v[1] < 0 ? v[1] : 0, v[1] > 0 ? -v[1] : 0,
                   v[2] < 0 ? v[2] : 0, v[2] > 0 ? -v[2] : 0);
}
inline GhostData additive_point_to_ghost(const IntVec& v) {
  return GhostData(v[0] > 0 ? v[0] : 0, v[0] < 0 ? -v[0] : 0, v[1] > 0 ? v[1] : 0, v[1] < 0 ? -v[1] : 0,
                   v[2] > 0 ? v[2] : 0, v[2] < 0 ? -v[2] : 0);
}
inline GhostData additive_reductive_point_to_ghost(const IntVec& v) {
  return additive_point_to_ghost(v) + reductive_point_to_ghost(v);
}
inline std::ostream& operator<<(std::ostream& os, const GhostData& g) {
  return os << "{" << g.get_minus() << " " << g.get_plus() << "}";
}

}  // namespace SpatialOps
#endif
