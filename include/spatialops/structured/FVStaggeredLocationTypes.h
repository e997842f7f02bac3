// Staggered-mesh location types: offsets of each field type relative to the scalar volume and
// the extra cell it carries on a + boundary (drop-in for
// spatialops/structured/FVStaggeredLocationTypes.h:63-126; the table is the finite-volume
// staggering itself, so its entries are the same).
#ifndef SpatialOps_FVStaggeredLocationTypes_h
#define SpatialOps_FVStaggeredLocationTypes_h

#include <spatialops/structured/IndexTriplet.h>

namespace SpatialOps {

#define NEBO_LOCATION(NAME, DIR, OX, OY, OZ, EX, EY, EZ) \
  struct NAME {                                          \
    typedef DIR FaceDir;                                 \
    typedef IndexTriplet<OX, OY, OZ> Offset;             \
    typedef IndexTriplet<EX, EY, EZ> BCExtra;            \
  };

NEBO_LOCATION(SVol, NODIR, 0, 0, 0, 0, 0, 0)
NEBO_LOCATION(SSurfX, XDIR, -1, 0, 0, 1, 0, 0)
NEBO_LOCATION(SSurfY, YDIR, 0, -1, 0, 0, 1, 0)
NEBO_LOCATION(SSurfZ, ZDIR, 0, 0, -1, 0, 0, 1)
NEBO_LOCATION(XVol, NODIR, -1, 0, 0, 1, 0, 0)
NEBO_LOCATION(XSurfX, XDIR, 0, 0, 0, 0, 0, 0)
NEBO_LOCATION(XSurfY, YDIR, -1, -1, 0, 0, 1, 0)
NEBO_LOCATION(XSurfZ, ZDIR, -1, 0, -1, 0, 0, 1)
NEBO_LOCATION(YVol, NODIR, 0, -1, 0, 0, 1, 0)
NEBO_LOCATION(YSurfX, XDIR, -1, -1, 0, 1, 0, 0)
NEBO_LOCATION(YSurfY, YDIR, 0, 0, 0, 0, 0, 0)
NEBO_LOCATION(YSurfZ, ZDIR, 0, -1, -1, 0, 0, 1)
NEBO_LOCATION(ZVol, NODIR, 0, 0, -1, 0, 0, 1)
NEBO_LOCATION(ZSurfX, XDIR, -1, 0, -1, 1, 0, 0)
NEBO_LOCATION(ZSurfY, YDIR, 0, -1, -1, 0, 1, 0)
NEBO_LOCATION(ZSurfZ, ZDIR, 0, 0, 0, 0, 0, 0)
NEBO_LOCATION(SingleValue, NODIR, 0, 0, 0, 0, 0, 0)
#undef NEBO_LOCATION

}  // namespace SpatialOps
#endif
