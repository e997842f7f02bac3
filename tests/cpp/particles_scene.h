// The particle <-> cell scenes shared by the reference-built golden generator
// (oracle/ref/ref_particles.cpp, reference headers) and the GPU program
// (tests/cpp/particles_gpu.cu, drop-in headers).  It uses only names both sets of headers
// define, so the same code drives both.  The including file includes its SpatialOps headers
// (structured/FVStaggered.h, structured/Grid.h, particles/ParticleOperators.h) first.
//
//   <prog> scene <field> <nx> <ny> <nz> <ghost> <bcx> <np> <axes> <dx> <xlo> <dy> <ylo> <dz> <zlo>
//                <cell.bin> <px.bin> <py.bin> <pz.bin> <psize.bin> <pval.bin> <out.bin>
//       field 0 = SVolField, 1 = XVolField; axes bit a set: coordinate a is passed (else NULL).
//       cell.bin holds the cell field's whole allocation, the particle files np doubles each.
//       out.bin receives CellToParticle(cell) (np doubles), then ParticleToCell(pval) (the
//       allocation; cells outside the window keep -7777.25).
//   <prog> reftest
//       the reference's own test scene (spatialops/particles/test/TestParticleOperators.cpp:22-99):
//       Grid coordinates, one particle, its known answers; exit status 0 when all hold.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

using namespace SpatialOps;
using Particle::ParticleField;

static std::vector<double> particle_read_doubles(const char* path, size_t n) {
  std::vector<double> v(n);
  FILE* f = std::fopen(path, "rb");
  if (!f) { std::perror(path); std::exit(2); }
  if (n && std::fread(v.data(), 8, n, f) != n) { std::fprintf(stderr, "short read %s\n", path); std::exit(2); }
  std::fclose(f);
  return v;
}

// argv[1] is <field>; the scene's arguments follow as in the usage above.
template <typename CellField>
static int particle_scene(char** argv) {
  const IntVec n(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]));
  const int g = std::atoi(argv[5]);
  const bool bcx = std::atoi(argv[6]) != 0;
  const size_t np = (size_t)std::atol(argv[7]);
  const int axes = std::atoi(argv[8]);
  const double dx = std::strtod(argv[9], NULL), xlo = std::strtod(argv[10], NULL);
  const double dy = std::strtod(argv[11], NULL), ylo = std::strtod(argv[12], NULL);
  const double dz = std::strtod(argv[13], NULL), zlo = std::strtod(argv[14], NULL);

  const GhostData cg(g);
  const BoundaryCellInfo cbc = BoundaryCellInfo::build<CellField>(bcx, false, false);
  const MemoryWindow mw = get_window_with_ghost(n, cg, cbc);
  CellField cell(mw, cbc, cg, NULL);
  CellField ctmp(mw, cbc, cg, NULL);
  const size_t ncell = mw.glob_npts();
  const std::vector<double> cv = particle_read_doubles(argv[15], ncell);
  double* cp = cell.field_values(CPU_INDEX);
  double* tp = ctmp.field_values(CPU_INDEX);
  for (size_t i = 0; i < ncell; ++i) {
    cp[i] = cv[i];
    tp[i] = -7777.25;
  }

  const GhostData pg(0);
  const BoundaryCellInfo pbc = BoundaryCellInfo::build<ParticleField>();
  const MemoryWindow pmw(IntVec((int)np, 1, 1));
  ParticleField px(pmw, pbc, pg, NULL), py(pmw, pbc, pg, NULL), pz(pmw, pbc, pg, NULL);
  ParticleField psize(pmw, pbc, pg, NULL), pval(pmw, pbc, pg, NULL), ptmp(pmw, pbc, pg, NULL);
  ParticleField* fs[5] = {&px, &py, &pz, &psize, &pval};
  for (int a = 0; a < 5; ++a) {
    const std::vector<double> v = particle_read_doubles(argv[16 + a], np);
    double* d = fs[a]->field_values(CPU_INDEX);
    for (size_t i = 0; i < np; ++i) d[i] = v[i];
  }

  typedef Particle::CellToParticle<CellField> C2P;
  typedef Particle::ParticleToCell<CellField> P2C;
  C2P c2p(dx, xlo, dy, ylo, dz, zlo);
  P2C p2c(dx, xlo, dy, ylo, dz, zlo);
  c2p.set_coordinate_information((axes & 1) ? &px : NULL, (axes & 2) ? &py : NULL, (axes & 4) ? &pz : NULL, &psize);
  p2c.set_coordinate_information((axes & 1) ? &px : NULL, (axes & 2) ? &py : NULL, (axes & 4) ? &pz : NULL, &psize);
  c2p.apply_to_field(cell, ptmp);
  p2c.apply_to_field(pval, ctmp);

  FILE* f = std::fopen(argv[21], "wb");
  if (!f) { std::perror(argv[21]); return 2; }
  std::fwrite(ptmp.field_values(CPU_INDEX), 8, np, f);
  std::fwrite(ctmp.field_values(CPU_INDEX), 8, ncell, f);
  std::fclose(f);
  return 0;
}

// The reference test's scene and checks, written against the public API only.
static int particle_reftest() {
  const IntVec dim(10, 1, 1);
  const Grid grid(dim, DoubleVec(10, 1, 1));
  const GhostData cg(3);
  const BoundaryCellInfo cbc = BoundaryCellInfo::build<SVolField>();
  const MemoryWindow mw = get_window_with_ghost(dim, cg, BoundaryCellInfo::build<SVolField>(false, false, false));
  SVolField xcoord(mw, cbc, cg, NULL), f(mw, cbc, cg, NULL), ctmp(mw, cbc, cg, NULL);
  const GhostData pg(0);
  const BoundaryCellInfo pbc = BoundaryCellInfo::build<ParticleField>();
  const MemoryWindow pmw(IntVec(1, 1, 1));
  ParticleField pCoord(pmw, pbc, pg, NULL), pSize(pmw, pbc, pg, NULL), pfield(pmw, pbc, pg, NULL),
      ptmp(pmw, pbc, pg, NULL);
  grid.set_coord<XDIR>(xcoord);
  f <<= 10 * xcoord;
  pCoord[0] = 3.25;
  pSize[0] = 5;
  pfield[0] = 20;
  Particle::CellToParticle<SVolField> c2p(xcoord[1] - xcoord[0], xcoord[cg.get_minus(0)]);
  c2p.set_coordinate_information(&pCoord, NULL, NULL, &pSize);
  Particle::ParticleToCell<SVolField> p2c(xcoord[1] - xcoord[0], xcoord[cg.get_minus(0)]);
  p2c.set_coordinate_information(&pCoord, NULL, NULL, &pSize);
  c2p.apply_to_field(f, ptmp);
  p2c.apply_to_field(pfield, ctmp);
  int bad = 0;
  if (ptmp[0] != 32.5) { std::printf("c2p: %.17g\n", ptmp[0]); ++bad; }
  const double want[10] = {1, 4, 4, 4, 4, 3, 0, 0, 0, 0};
  const size_t ishift = cg.get_minus(0);
  for (int i = 0; i < 10; ++i)
    if (ctmp[ishift + i] != want[i]) { std::printf("p2c [%d]: %.17g\n", i, ctmp[ishift + i]); ++bad; }
  std::printf("%s\n", bad ? "FAIL" : "PASS");
  return bad ? 1 : 0;
}

static int particles_main(int argc, char** argv) {
  const std::string cmd = argc > 1 ? argv[1] : "";
  if (cmd == "reftest") return particle_reftest();
  if (cmd == "scene" && argc >= 23) {
    char** a = argv + 1;
    return std::atoi(a[1]) == 0 ? particle_scene<SVolField>(a) : particle_scene<XVolField>(a);
  }
  std::fprintf(stderr, "usage: %s reftest | scene field nx ny nz ghost bcx np axes dx xlo dy ylo dz zlo "
                       "cell px py pz psize pval out\n", argv[0]);
  return 1;
}
