// Operator type tags (drop-in for spatialops/SpatialOpsDefs.h:44-137).
#ifndef SpatialOps_SpatialOpsDefs_h
#define SpatialOps_SpatialOpsDefs_h

#include <spatialops/structured/IndexTriplet.h>

namespace SpatialOps {

struct Interpolant {};
struct Gradient {};
struct Divergence {};
struct Filter {};
struct Restriction {};
struct InterpolantX { typedef XDIR DirT; typedef InterpolantX type; };
struct InterpolantY { typedef YDIR DirT; typedef InterpolantY type; };
struct InterpolantZ { typedef ZDIR DirT; typedef InterpolantZ type; };
struct GradientX { typedef XDIR DirT; typedef GradientX type; };
struct GradientY { typedef YDIR DirT; typedef GradientY type; };
struct GradientZ { typedef ZDIR DirT; typedef GradientZ type; };

}  // namespace SpatialOps
#endif
