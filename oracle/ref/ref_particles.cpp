// Golden-vector generator for the particle <-> cell operators, built from the reference's own
// headers (spatialops/particles/ParticleOperators.h) around the scenes of
// tests/cpp/particles_scene.h.
//
// oracle/Makefile compiles this file with the reference tree on the include path, serial, with
// NDEBUG (the reference asserts that a particle's weights sum to one, which is false by design
// for the clipped boxes the fixtures include).  tests/golden/make_golden.py runs the binary,
// oracle/_ref/ref_particles, and stores inputs and outputs under tests/golden/.  Test
// infrastructure only: the product never links or runs it.

#include <spatialops/structured/FVStaggered.h>
#include <spatialops/structured/Grid.h>
#include <spatialops/particles/ParticleOperators.h>

#include "../../tests/cpp/particles_scene.h"

int main(int argc, char** argv) {
  const int rc = particles_main(argc, argv);
  std::fflush(NULL);
  std::_Exit(rc);
}
