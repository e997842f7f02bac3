// Nebo: the field-expression language of SpatialOps, evaluated on sm_103a
// (drop-in umbrella for spatialops/Nebo.h).  Compile the including translation unit with nvcc
// for sm_103a and link libnebo_gb300.so.
#ifndef SpatialOps_Nebo_h
#define SpatialOps_Nebo_h

#include <spatialops/NeboApplyPointwise.h>
#include <spatialops/NeboAssignment.h>
#include <spatialops/NeboBasic.h>
#include <spatialops/NeboCore.h>
#include <spatialops/NeboOperators.h>
#include <spatialops/NeboReductions.h>
#include <spatialops/NeboStencilBuilder.h>
#include <spatialops/SpatialOpsDefs.h>

#endif
