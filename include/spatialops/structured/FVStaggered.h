// Umbrella of the structured finite-volume API (drop-in for spatialops/structured/FVStaggered.h).
#ifndef SpatialOps_FVStaggered_h
#define SpatialOps_FVStaggered_h

#include <spatialops/Nebo.h>
#include <spatialops/OperatorDatabase.h>
#include <spatialops/structured/FVStaggeredFieldTypes.h>
#include <spatialops/structured/SpatialMask.h>
#include <spatialops/structured/stencil/FVStaggeredOperatorTypes.h>
#include <spatialops/structured/stencil/StencilBuilder.h>

#endif
