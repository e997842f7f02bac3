// Ghost bookkeeping of an assignment (drop-in for spatialops/NeboBasic.h:56-100):
// calculate_actual_ghost returns the ghost layers an assignment may write, given the left-hand
// side's ghosts and BC cells and the right-hand side's ghosts_with_bc().
#ifndef SpatialOps_NeboBasic_h
#define SpatialOps_NeboBasic_h

#include <sstream>
#include <stdexcept>

#include <spatialops/structured/BoundaryCellInfo.h>
#include <spatialops/structured/GhostData.h>

namespace SpatialOps {

inline GhostData calculate_actual_ghost(bool const useGhost, GhostData const& lhs, BoundaryCellInfo const& bc,
                                        GhostData const& rhs) {
  static const char* axis[3] = {"X", "Y", "Z"};
  for (int i = 0; i < 3; ++i) {
    if (bc.has_bc(i) && rhs.get_plus(i) < bc.has_extra(i)) {
      std::ostringstream msg;
      msg << "Nebo error in Nebo Ghost Checking:\nNot enough valid extra cells to validate all interior cells in the "
          << axis[i] << " direction";
      throw std::runtime_error(msg.str());
    }
  }
  const GhostData pe = point_to_ghost(bc.has_extra());
  return (useGhost ? min(lhs + pe, rhs) : GhostData(IntVec(0, 0, 0), bc.has_extra())) - pe;
}

}  // namespace SpatialOps
#endif
