// Particle fields: one value per particle, no mesh structure (drop-in for
// spatialops/particles/ParticleFieldTypes.h:33-66; the location traits are the reference's:
// no face direction, no staggering offset, no boundary-cell extra).
#ifndef ParticleFieldTypes_h
#define ParticleFieldTypes_h

#include <spatialops/structured/IndexTriplet.h>
#include <spatialops/structured/SpatialField.h>

namespace SpatialOps {
namespace Particle {

struct ParticleFieldTraits {
  typedef NODIR FaceDir;
  typedef IndexTriplet<0, 0, 0> Offset;
  typedef IndexTriplet<0, 0, 0> BCExtra;
};

typedef SpatialField<ParticleFieldTraits> ParticleField;

}  // namespace Particle
}  // namespace SpatialOps
#endif
