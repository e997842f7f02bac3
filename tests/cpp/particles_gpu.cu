// The particle <-> cell scenes (tests/cpp/particles_scene.h) compiled against the drop-in
// headers: CellToParticle / ParticleToCell run on the GPU through nebo_cell_to_particle /
// nebo_particle_to_cell.  tests/test_gpu_particles.py compares its output files with the
// reference-built ones bit for bit and runs the reference's own test scene.
#include <spatialops/structured/FVStaggered.h>
#include <spatialops/structured/Grid.h>
#include <spatialops/particles/ParticleOperators.h>

#include "particles_scene.h"

int main(int argc, char** argv) { return particles_main(argc, argv); }
