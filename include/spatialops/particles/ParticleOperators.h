// Particle <-> cell interpolation operators (drop-in for
// spatialops/particles/ParticleOperators.h:45-403: ParticleToCell, CellToParticle).
//
// Same constructor, set_coordinate_information and apply_to_field as the reference; the work
// runs on the GPU through nebo_particle_to_cell / nebo_cell_to_particle and gives the
// reference's serial results bit for bit.  A particle is a cube of edge psize centred at its
// coordinates; a null coordinate field switches that axis off.  Differences from the reference:
//   * a box that reaches outside the cell field's window is clipped at both ends (the
//     reference clips the high end only; its low end is undefined behaviour);
//   * a missing size field or particle fields of different lengths throw std::runtime_error
//     ("Nebo error in ...") where the reference asserts or reads past the end.
#ifndef ParticleOperators_h
#define ParticleOperators_h

#include <stdexcept>
#include <string>

#include <nebo_gb300.h>
#include <spatialops/Nebo.h>
#include <spatialops/particles/ParticleFieldTypes.h>

namespace SpatialOps {
namespace Particle {

namespace detail {

// Device values of one particle field, after checking that its window is its whole allocation
// (the reference iterates begin()..end() of the window).
inline const double* particle_values(const ParticleField* f, size_t np, const char* who, const char* what) {
  if (!f) return nullptr;
  const MemoryWindow& w = f->window_with_ghost();
  if (w.local_npts() != w.glob_npts())
    throw std::runtime_error(std::string("Nebo error in ") + who + ": " + what + " is a sub-window of its field");
  if (w.local_npts() < np)
    throw std::runtime_error(std::string("Nebo error in ") + who + ": " + what + " has fewer values than particles");
  return f->device_values_for_read();
}

struct MeshState {
  double d[3], lo[3];
  MeshState(double dx, double xlo, double dy, double ylo, double dz, double zlo)
      : d{dx <= 0 ? 1.0 : dx, dy <= 0 ? 1.0 : dy, dz <= 0 ? 1.0 : dz},
        lo{dx <= 0 ? 0.0 : xlo, dy <= 0 ? 0.0 : ylo, dz <= 0 ? 0.0 : zlo} {}
  template <typename CellField>
  nebo_particle_mesh mesh(const CellField& cell) const {
    nebo_particle_mesh m;
    const IntVec ngm = cell.get_ghost_data().get_minus();
    for (int a = 0; a < 3; ++a) {
      m.spacing[a] = d[a];
      m.low[a] = lo[a];
      m.ghost_minus[a] = ngm[a];
    }
    return m;
  }
};

}  // namespace detail

// Interpolates an extensive particle quantity onto the mesh (ParticleOperators.h:45-88).
template <typename CellField>
class ParticleToCell {
 public:
  typedef ParticleField SrcFieldType;
  typedef CellField DestFieldType;

  ParticleToCell(const double dx, const double xlo, const double dy = -1, const double ylo = 0, const double dz = -1,
                 const double zlo = 0)
      : m_(dx, xlo, dy, ylo, dz, zlo) {}

  void set_coordinate_information(const ParticleField* const pxcoord, const ParticleField* const pycoord,
                                  const ParticleField* const pzcoord, const ParticleField* const psize) {
    px_ = pxcoord;
    py_ = pycoord;
    pz_ = pzcoord;
    psize_ = psize;
  }

  void apply_to_field(const SrcFieldType& src, DestFieldType& dest) const {
    const char* who = "ParticleToCell::apply_to_field";
    if (!psize_) throw std::runtime_error(std::string("Nebo error in ") + who + ": no particle size field");
    const size_t np = src.window_with_ghost().local_npts();
    const double* s = detail::particle_values(&src, np, who, "the source");
    const double* x = detail::particle_values(px_, np, who, "the x coordinate");
    const double* y = detail::particle_values(py_, np, who, "the y coordinate");
    const double* z = detail::particle_values(pz_, np, who, "the z coordinate");
    const double* sz = detail::particle_values(psize_, np, who, "the particle size");
    const nebo_particle_mesh m = m_.mesh(dest);
    nebo_field d = dest.descriptor();
    d.data = dest.device_values_for_write();
    nebo_detail::throw_status(nebo_particle_to_cell(&m, x, y, z, sz, (int64_t)np, s, &d, dest.get_stream()), who);
  }

 private:
  detail::MeshState m_;
  const ParticleField *px_ = nullptr, *py_ = nullptr, *pz_ = nullptr, *psize_ = nullptr;
};

// Interpolates a mesh quantity onto the particles (ParticleOperators.h:96-140).
template <typename CellField>
class CellToParticle {
 public:
  typedef CellField SrcFieldType;
  typedef ParticleField DestFieldType;

  CellToParticle(const double dx, const double xlo, const double dy = -1, const double ylo = 0, const double dz = -1,
                 const double zlo = 0)
      : m_(dx, xlo, dy, ylo, dz, zlo) {}

  void set_coordinate_information(const ParticleField* pxcoord, const ParticleField* pycoord,
                                  const ParticleField* pzcoord, const ParticleField* psize) {
    px_ = pxcoord;
    py_ = pycoord;
    pz_ = pzcoord;
    psize_ = psize;
  }

  void apply_to_field(const SrcFieldType& src, DestFieldType& dest) const {
    const char* who = "CellToParticle::apply_to_field";
    if (!psize_) throw std::runtime_error(std::string("Nebo error in ") + who + ": no particle size field");
    const MemoryWindow& dw = dest.window_with_ghost();
    if (dw.local_npts() != dw.glob_npts())
      throw std::runtime_error(std::string("Nebo error in ") + who + ": the destination is a sub-window of its field");
    const size_t np = dw.local_npts();
    const double* x = detail::particle_values(px_, np, who, "the x coordinate");
    const double* y = detail::particle_values(py_, np, who, "the y coordinate");
    const double* z = detail::particle_values(pz_, np, who, "the z coordinate");
    const double* sz = detail::particle_values(psize_, np, who, "the particle size");
    const nebo_particle_mesh m = m_.mesh(src);
    nebo_field c = src.descriptor();
    c.data = const_cast<typename SrcFieldType::value_type*>(src.device_values_for_read());
    double* out = dest.device_values_for_write();
    nebo_detail::throw_status(nebo_cell_to_particle(&m, x, y, z, sz, (int64_t)np, &c, out, dest.get_stream()), who);
  }

 private:
  detail::MeshState m_;
  const ParticleField *px_ = nullptr, *py_ = nullptr, *pz_ = nullptr, *psize_ = nullptr;
};

}  // namespace Particle
}  // namespace SpatialOps
#endif
