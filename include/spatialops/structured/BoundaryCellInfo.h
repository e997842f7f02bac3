// Boundary-cell information (drop-in for spatialops/structured/BoundaryCellInfo.h): which +
// faces carry a physical boundary, and how many extra cells the location adds there.
#ifndef SpatialOps_BoundaryCellInfo_h
#define SpatialOps_BoundaryCellInfo_h

#include <cassert>

#include <spatialops/structured/IntVec.h>

namespace SpatialOps {

class BoundaryCellInfo {
  IntVec isbc_, nExtra_;
  BoundaryCellInfo(bool bcx, bool bcy, bool bcz, const IntVec& nExtra)
      : isbc_(bcx, bcy, bcz), nExtra_(IntVec(bcx, bcy, bcz) * nExtra) {}

 public:
  template <typename FieldT> static BoundaryCellInfo build(bool bcx, bool bcy, bool bcz) {
    return BoundaryCellInfo(bcx, bcy, bcz, FieldT::Location::BCExtra::int_vec());
  }
  template <typename FieldT> static BoundaryCellInfo build(const IntVec& bc) {
    return BoundaryCellInfo(bc[0] != 0, bc[1] != 0, bc[2] != 0, FieldT::Location::BCExtra::int_vec());
  }
  template <typename FieldT> static BoundaryCellInfo build() {
    return BoundaryCellInfo(false, false, false, FieldT::Location::BCExtra::int_vec());
  }
  bool has_bc(int d) const { return isbc_[d] != 0; }
  IntVec has_bc() const { return isbc_; }
  int num_extra(int d) const { return nExtra_[d]; }
  IntVec num_extra() const { return nExtra_; }
  int has_extra(int d) const { return has_bc(d) ? num_extra(d) : 0; }
  IntVec has_extra() const { return IntVec(has_extra(0), has_extra(1), has_extra(2)); }
  BoundaryCellInfo limit_by_extent(const IntVec& e) const {
    return BoundaryCellInfo(has_bc(0), has_bc(1), has_bc(2),
                            IntVec(e[0] == 1 ? 0 : has_extra(0), e[1] == 1 ? 0 : has_extra(1),
                                   e[2] == 1 ? 0 : has_extra(2)));
  }
  bool operator==(const BoundaryCellInfo& o) const { return isbc_ == o.isbc_ && nExtra_ == o.nExtra_; }
};

}  // namespace SpatialOps
#endif
