// nebo_oracle.cpp -- CPU restatement of the reference's serial Nebo evaluation.
//
// TEST INFRASTRUCTURE ONLY (the oracle).  See nebo_oracle.h for what it restates and where
// its parity is pinned.  Compiled with -ffp-contract=off so that no multiply-add is fused and
// every operation rounds as in the reference's serial build.

#include "nebo_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

// ------------------------------------------------------------------------------------------
// GhostData (spatialops/structured/GhostData.h:54-257).  GHOST_MAX marks "infinite" ghosts,
// which scalars carry; '+' keeps an infinite left side, '-' refuses an infinite right side.
const int GHOST_MAX = 9001;

struct GD {
  int m[3], p[3];
  bool inf;
  GD(int n = 0) {
    for (int i = 0; i < 3; ++i) m[i] = p[i] = n;
    fix();
  }
  GD(int mx, int px, int my, int py, int mz, int pz) {
    m[0] = mx; p[0] = px; m[1] = my; p[1] = py; m[2] = mz; p[2] = pz;
    fix();
  }
  void fix() {
    inf = m[0] >= GHOST_MAX && m[1] >= GHOST_MAX && m[2] >= GHOST_MAX && p[0] >= GHOST_MAX &&
          p[1] >= GHOST_MAX && p[2] >= GHOST_MAX;
  }
  GD operator+(const GD& r) const {
    GD g(*this);
    if (!g.inf) {
      if (r.inf) return r;
      for (int i = 0; i < 3; ++i) { g.m[i] += r.m[i]; g.p[i] += r.p[i]; }
    }
    return g;
  }
  GD operator-(const GD& r) const {
    if (r.inf) throw std::runtime_error("Cannot use infinite ghost data on the right-hand side of subtraction.");
    GD g(*this);
    for (int i = 0; i < 3; ++i) { g.m[i] -= r.m[i]; g.p[i] -= r.p[i]; }
    return g;  // isInf_ is kept from the left side, as in the reference's operator-=
  }
  GD limit_by_extent(const int e[3]) const {
    return GD(e[0] <= 1 ? 0 : m[0], e[0] <= 1 ? 0 : p[0], e[1] <= 1 ? 0 : m[1], e[1] <= 1 ? 0 : p[1],
              e[2] <= 1 ? 0 : m[2], e[2] <= 1 ? 0 : p[2]);
  }
};

GD gmin(const GD& a, const GD& b) {
  return GD(std::min(a.m[0], b.m[0]), std::min(a.p[0], b.p[0]), std::min(a.m[1], b.m[1]),
            std::min(a.p[1], b.p[1]), std::min(a.m[2], b.m[2]), std::min(a.p[2], b.p[2]));
}
GD point_to_ghost(const int v[3]) {
  return GD(v[0] < 0 ? -v[0] : 0, v[0] > 0 ? v[0] : 0, v[1] < 0 ? -v[1] : 0, v[1] > 0 ? v[1] : 0,
            v[2] < 0 ? -v[2] : 0, v[2] > 0 ? v[2] : 0);
}
GD reductive_point_to_ghost(const int v[3]) {
  return GD(v[0] < 0 ? v[0] : 0, v[0] > 0 ? -v[0] : 0, v[1] < 0 ? v[1] : 0, v[1] > 0 ? -v[1] : 0,
            v[2] < 0 ? v[2] : 0, v[2] > 0 ? -v[2] : 0);
}
GD additive_point_to_ghost(const int v[3]) {
  return GD(v[0] > 0 ? v[0] : 0, v[0] < 0 ? -v[0] : 0, v[1] > 0 ? v[1] : 0, v[1] < 0 ? -v[1] : 0,
            v[2] > 0 ? v[2] : 0, v[2] < 0 ? -v[2] : 0);
}
GD additive_reductive_point_to_ghost(const int v[3]) {
  return additive_point_to_ghost(v) + reductive_point_to_ghost(v);
}

// ------------------------------------------------------------------------------------------
// Boundary-cell info (spatialops/structured/BoundaryCellInfo.h:45-159) of a field or mask.
struct Layout {
  int glob[3];
  GD valid;       // valid ghosts (limited by extent)
  int has_bc[3];
  int extra[3];   // has_extra(): bc extra cells present on this axis
  Layout() {}
  template <typename D> explicit Layout(const D& d) {
    for (int i = 0; i < 3; ++i) glob[i] = d.glob[i];
    valid = GD(d.ghost_minus[0], d.ghost_plus[0], d.ghost_minus[1], d.ghost_plus[1], d.ghost_minus[2],
               d.ghost_plus[2])
                .limit_by_extent(glob);
    for (int i = 0; i < 3; ++i) {
      has_bc[i] = d.has_bc[i] ? 1 : 0;
      extra[i] = (has_bc[i] && glob[i] != 1) ? d.bc_extra[i] : 0;
    }
  }
  int index(int x, int y, int z) const {  // interior-relative -> flat (NeboRhs.h:283-285)
    return (x + valid.m[0]) + glob[0] * ((y + valid.m[1]) + glob[1] * (z + valid.m[2]));
  }
  void extents(int e[3]) const {
    for (int i = 0; i < 3; ++i) e[i] = glob[i] - valid.m[i] - valid.p[i];
  }
};

// ------------------------------------------------------------------------------------------
// Expression nodes.  eval() returns the value at interior-relative (x,y,z); check() the
// boolean of a comparison, logical operator or mask.
struct Node {
  virtual ~Node() {}
  virtual GD ghosts_with_bc() const = 0;
  virtual GD ghosts_without_bc() const = 0;
  virtual bool has_extents() const = 0;
  virtual void extents(int e[3]) const = 0;
  virtual void has_bc(int b[3]) const = 0;
  virtual double eval(int, int, int) const { throw std::runtime_error("oracle: boolean used as value"); }
  virtual bool check(int, int, int) const { throw std::runtime_error("oracle: value used as boolean"); }
};
typedef std::unique_ptr<Node> P;

struct FieldLeaf : Node {
  Layout L;
  const double* d;
  FieldLeaf(const orc_field& f) : L(f), d(f.data) {}
  GD ghosts_with_bc() const override { return L.valid + point_to_ghost(L.extra); }
  GD ghosts_without_bc() const override { return L.valid; }
  bool has_extents() const override { return true; }
  void extents(int e[3]) const override { L.extents(e); }
  void has_bc(int b[3]) const override { for (int i = 0; i < 3; ++i) b[i] = L.has_bc[i]; }
  double eval(int x, int y, int z) const override { return d[L.index(x, y, z)]; }
};

struct MaskLeaf : Node {
  Layout L;
  const uint32_t* bits;
  MaskLeaf(const orc_mask& m) : L(m), bits(m.bits) {}
  GD ghosts_with_bc() const override { return L.valid + point_to_ghost(L.extra); }
  GD ghosts_without_bc() const override { return L.valid; }
  bool has_extents() const override { return true; }
  void extents(int e[3]) const override { L.extents(e); }
  void has_bc(int b[3]) const override { GD g = point_to_ghost(L.has_bc); for (int i = 0; i < 3; ++i) b[i] = g.m[i]; }
  bool check(int x, int y, int z) const override {
    const int pos = L.index(x, y, z);
    return (bits[pos / 32] >> (pos % 32)) & 1u;
  }
};

struct ScalarLeaf : Node {
  double v;
  explicit ScalarLeaf(double v_) : v(v_) {}
  GD ghosts_with_bc() const override { return GD(GHOST_MAX); }
  GD ghosts_without_bc() const override { return GD(GHOST_MAX); }
  bool has_extents() const override { return false; }
  void extents(int e[3]) const override { e[0] = e[1] = e[2] = 0; }
  void has_bc(int b[3]) const override { b[0] = b[1] = b[2] = 0; }
  double eval(int, int, int) const override { return v; }
};

// Nodes whose ghosts are the min over children and whose extents come from the first child
// that has extents (SumOp et al., spatialops/NeboOperators.h:56-100).
struct Composite : Node {
  std::vector<P> kids;
  GD ghosts_with_bc() const override {
    GD g = kids[0]->ghosts_with_bc();
    for (size_t i = 1; i < kids.size(); ++i) g = gmin(g, kids[i]->ghosts_with_bc());
    return g;
  }
  GD ghosts_without_bc() const override {
    GD g = kids[0]->ghosts_without_bc();
    for (size_t i = 1; i < kids.size(); ++i) g = gmin(g, kids[i]->ghosts_without_bc());
    return g;
  }
  bool has_extents() const override {
    for (const P& k : kids) if (k->has_extents()) return true;
    return false;
  }
  const Node* first_with_extents() const {
    for (const P& k : kids) if (k->has_extents()) return k.get();
    return kids.back().get();
  }
  void extents(int e[3]) const override { first_with_extents()->extents(e); }
  void has_bc(int b[3]) const override { first_with_extents()->has_bc(b); }
};

struct Bin : Composite {
  int op;
  double eval(int x, int y, int z) const override {
    const double a = kids[0]->eval(x, y, z);
    const double b = kids[1]->eval(x, y, z);
    switch (op) {
      case ORC_ADD: return a + b;
      case ORC_SUB: return a - b;
      case ORC_MUL: return a * b;
      case ORC_DIV: return a / b;
      case ORC_POW: return std::pow(a, b);
      case ORC_MAX: return (a > b) ? a : b;
      case ORC_MIN: return (a < b) ? a : b;
    }
    throw std::runtime_error("oracle: bad binary op");
  }
};

struct Un : Composite {
  int fn;
  double eval(int x, int y, int z) const override {
    const double a = kids[0]->eval(x, y, z);
    switch (fn) {
      case ORC_NEG: return -a;
      case ORC_SIN: return std::sin(a);
      case ORC_COS: return std::cos(a);
      case ORC_TAN: return std::tan(a);
      case ORC_EXP: return std::exp(a);
      case ORC_TANH: return std::tanh(a);
      case ORC_ABS: return std::abs(a);
      case ORC_SQRT: return std::sqrt(a);
      case ORC_LOG: return std::log(a);
      case ORC_LOG10: return std::log10(a);
      case ORC_ERF: return std::erf(a);
      case ORC_ERFC: return std::erfc(a);
      case ORC_SQUARE: { const double r = a; return r * r; }
      case ORC_CUBE: { const double r = a; return r * r * r; }
    }
    throw std::runtime_error("oracle: bad unary fn");
  }
};

struct PowInt : Composite {
  int e;
  double eval(int x, int y, int z) const override { return std::pow(kids[0]->eval(x, y, z), (double)e); }
};

struct Cmp : Composite {
  int op;
  bool check(int x, int y, int z) const override {
    const double a = kids[0]->eval(x, y, z);
    const double b = kids[1]->eval(x, y, z);
    switch (op) {
      case ORC_EQ: return a == b;
      case ORC_NE: return a != b;
      case ORC_LT: return a < b;
      case ORC_LE: return a <= b;
      case ORC_GT: return a > b;
      case ORC_GE: return a >= b;
    }
    throw std::runtime_error("oracle: bad comparison");
  }
};

struct Logic : Composite {
  int op;
  bool check(int x, int y, int z) const override {
    switch (op) {
      case ORC_AND: return kids[0]->check(x, y, z) && kids[1]->check(x, y, z);
      case ORC_OR: return kids[0]->check(x, y, z) || kids[1]->check(x, y, z);
      case ORC_NOT: return !kids[0]->check(x, y, z);
    }
    throw std::runtime_error("oracle: bad logical op");
  }
};

// cond(t0, v0)(t1, v1)...(default): kids = t0 v0 t1 v1 ... default.  Ghosts are the min over
// all clause tests, values and the default (NeboCond.h:86-92, 284-290).
struct Cond : Composite {
  double eval(int x, int y, int z) const override {
    const size_t n = (kids.size() - 1) / 2;
    for (size_t i = 0; i < n; ++i)
      if (kids[2 * i]->check(x, y, z)) return kids[2 * i + 1]->eval(x, y, z);
    return kids.back()->eval(x, y, z);
  }
};

// Stencils: value = ((arg(p0)*c0 + arg(p1)*c1) + arg(p2)*c2) + ...; the first listed point is
// innermost (NeboStencils.h:407-448).  Ghosts: arg ghosts + min over points of
// additive_reductive_point_to_ghost (NeboStencils.h:222-239).
struct Stencil : Node {
  P arg;
  std::vector<int> pts;  // 3 per point
  std::vector<double> coefs;  // empty for a sum stencil
  GD possible(const GD& g) const {
    GD m = additive_reductive_point_to_ghost(&pts[0]);
    for (size_t i = 3; i < pts.size(); i += 3) m = gmin(m, additive_reductive_point_to_ghost(&pts[i]));
    return g + m;
  }
  GD ghosts_with_bc() const override { return possible(arg->ghosts_with_bc()); }
  GD ghosts_without_bc() const override { return possible(arg->ghosts_without_bc()); }
  bool has_extents() const override { return arg->has_extents(); }
  void extents(int e[3]) const override { arg->extents(e); }
  void has_bc(int b[3]) const override { arg->has_bc(b); }
  double eval(int x, int y, int z) const override {
    const size_t n = pts.size() / 3;
    if (coefs.empty()) {
      double r = arg->eval(x + pts[0], y + pts[1], z + pts[2]);
      for (size_t i = 1; i < n; ++i) r = r + arg->eval(x + pts[3 * i], y + pts[3 * i + 1], z + pts[3 * i + 2]);
      return r;
    }
    double r = arg->eval(x + pts[0], y + pts[1], z + pts[2]) * coefs[0];
    for (size_t i = 1; i < n; ++i)
      r = r + arg->eval(x + pts[3 * i], y + pts[3 * i + 1], z + pts[3 * i + 2]) * coefs[i];
    return r;
  }
};

struct Parser {
  const orc_expr* e;
  int pos = 0;
  explicit Parser(const orc_expr* e_) : e(e_) {}
  int next() {
    if (pos >= e->prog_len) throw std::runtime_error("oracle: truncated program");
    return e->prog[pos++];
  }
  P parse() {
    const int kind = next();
    switch (kind) {
      case ORC_FIELD: {
        const int i = next();
        if (i < 0 || i >= e->nfields) throw std::runtime_error("oracle: bad field index");
        return P(new FieldLeaf(e->fields[i]));
      }
      case ORC_SCALAR: return P(new ScalarLeaf(e->imms[next()]));
      case ORC_MASK: {
        const int i = next();
        if (i < 0 || i >= e->nmasks) throw std::runtime_error("oracle: bad mask index");
        return P(new MaskLeaf(e->masks[i]));
      }
      case ORC_BIN: { Bin* n = new Bin; n->op = next(); n->kids.push_back(parse()); n->kids.push_back(parse()); return P(n); }
      case ORC_UN: { Un* n = new Un; n->fn = next(); n->kids.push_back(parse()); return P(n); }
      case ORC_POWINT: { PowInt* n = new PowInt; n->e = next(); n->kids.push_back(parse()); return P(n); }
      case ORC_CMP: { Cmp* n = new Cmp; n->op = next(); n->kids.push_back(parse()); n->kids.push_back(parse()); return P(n); }
      case ORC_LOGIC: {
        Logic* n = new Logic;
        n->op = next();
        n->kids.push_back(parse());
        if (n->op != ORC_NOT) n->kids.push_back(parse());
        return P(n);
      }
      case ORC_COND: {
        Cond* n = new Cond;
        const int nc = next();
        for (int i = 0; i < 2 * nc + 1; ++i) n->kids.push_back(parse());
        return P(n);
      }
      case ORC_STENCIL:
      case ORC_SUMSTENCIL: {
        Stencil* n = new Stencil;
        const int np = next();
        for (int i = 0; i < 3 * np; ++i) n->pts.push_back(next());
        if (kind == ORC_STENCIL) {
          const int c0 = next();
          for (int i = 0; i < np; ++i) n->coefs.push_back(e->imms[c0 + i]);
        }
        n->arg = parse();
        return P(n);
      }
    }
    throw std::runtime_error("oracle: bad node kind");
  }
};

P parse_all(const orc_expr* e) {
  Parser p(e);
  P root = p.parse();
  if (p.pos != e->prog_len) throw std::runtime_error("oracle: trailing program words");
  return root;
}

// calculate_actual_ghost (spatialops/NeboBasic.h:61-100)
GD calculate_actual_ghost(bool useGhost, const GD& lhs, const Layout& bc, const GD& rhs) {
  static const char* axis[3] = {"X", "Y", "Z"};
  for (int i = 0; i < 3; ++i) {
    if (bc.has_bc[i] && rhs.p[i] < bc.extra[i]) {
      std::string msg = "Nebo error in Nebo Ghost Checking:\n";
      msg += "Not enough valid extra cells to validate all interior cells in the ";
      msg += axis[i];
      msg += " direction";
      throw std::runtime_error(msg);
    }
  }
  const GD pe = point_to_ghost(bc.extra);
  return (useGhost ? gmin(lhs + pe, rhs) : GD(0, bc.extra[0], 0, bc.extra[1], 0, bc.extra[2])) - pe;
}

// NeboField<Initial>::assign (spatialops/NeboLhs.h:67-98): the write region in
// interior-relative coordinates, [lo, hi) per axis.
bool write_limits(const Node& rhs, const Layout& L, bool useGhost, int lim[6]) {
  const GD ghosts = calculate_actual_ghost(useGhost, L.valid, L, rhs.ghosts_with_bc());
  int e[3];
  L.extents(e);
  for (int i = 0; i < 3; ++i) {
    lim[2 * i] = -ghosts.m[i];
    lim[2 * i + 1] = e[i] + ghosts.p[i];
  }
  return lim[1] - lim[0] > 0 && lim[3] - lim[2] > 0 && lim[5] - lim[4] > 0;
}

void set_err(char* err, int errlen, const char* msg) {
  if (err && errlen > 0) {
    std::strncpy(err, msg, (size_t)errlen - 1);
    err[errlen - 1] = 0;
  }
}

inline int wrap(int i, int n) { return ((i % n) + n) % n; }

}  // namespace

// ==========================================================================================
extern "C" {

int orc_write_limits(const orc_expr* e, const orc_field* lhs, int use_ghost, int32_t limits[6],
                     char* err, int errlen) {
  try {
    P root = parse_all(e);
    Layout L(*lhs);
    int lim[6];
    const bool any = write_limits(*root, L, use_ghost != 0, lim);
    for (int i = 0; i < 6; ++i) limits[i] = lim[i];
    return any ? 0 : 2;
  } catch (std::exception& ex) {
    set_err(err, errlen, ex.what());
    return 1;
  }
}

int orc_assign(const orc_expr* e, const orc_field* lhs, int use_ghost, char* err, int errlen) {
  try {
    P root = parse_all(e);
    Layout L(*lhs);
    int lim[6];
    if (!write_limits(*root, L, use_ghost != 0, lim)) return 0;
    for (int z = lim[4]; z < lim[5]; ++z)  // seqwalk_assign (NeboLhs.h:611-619)
      for (int y = lim[2]; y < lim[3]; ++y)
        for (int x = lim[0]; x < lim[1]; ++x) lhs->data[L.index(x, y, z)] = root->eval(x, y, z);
    return 0;
  } catch (std::exception& ex) {
    set_err(err, errlen, ex.what());
    return 1;
  }
}

int orc_masked_assign(const orc_expr* e, const orc_field* lhs, const int32_t* points, int npoints,
                      char* err, int errlen) {
  try {
    P root = parse_all(e);
    Layout L(*lhs);
    for (int i = 0; i < npoints; ++i) {
      const int x = points[3 * i], y = points[3 * i + 1], z = points[3 * i + 2];
      lhs->data[L.index(x, y, z)] = root->eval(x, y, z);
    }
    return 0;
  } catch (std::exception& ex) {
    set_err(err, errlen, ex.what());
    return 1;
  }
}

int orc_reduce(const orc_expr* e, int op, int use_ghost, double* result, char* err, int errlen) {
  try {
    P root = parse_all(e);
    // nebo_fold (NeboReductions.h:45-97): valid ghosts without BC when useGhost, else interior.
    const GD ghosts = use_ghost ? root->ghosts_without_bc() : GD(0);
    int ext[3];
    root->extents(ext);
    double r = op == ORC_RED_MAX ? -std::numeric_limits<double>::infinity()
               : op == ORC_RED_MIN ? std::numeric_limits<double>::infinity() : 0.0;
    for (int z = -ghosts.m[2]; z < ext[2] + ghosts.p[2]; ++z)
      for (int y = -ghosts.m[1]; y < ext[1] + ghosts.p[1]; ++y)
        for (int x = -ghosts.m[0]; x < ext[0] + ghosts.p[0]; ++x) {
          const double v = root->eval(x, y, z);
          switch (op) {
            case ORC_RED_SUM: r = r + v; break;
            case ORC_RED_MAX: r = (r < v) ? v : r; break;
            case ORC_RED_MIN: r = (r > v) ? v : r; break;
            case ORC_RED_NORM: r = r + std::pow(v, 2.0); break;
          }
        }
    if (op == ORC_RED_NORM) r = std::sqrt(r);
    *result = r;
    return 0;
  } catch (std::exception& ex) {
    set_err(err, errlen, ex.what());
    return 1;
  }
}

int orc_ghosts(const orc_expr* e, int with_bc, int32_t minus[3], int32_t plus[3]) {
  try {
    P root = parse_all(e);
    const GD g = with_bc ? root->ghosts_with_bc() : root->ghosts_without_bc();
    for (int i = 0; i < 3; ++i) { minus[i] = g.m[i]; plus[i] = g.p[i]; }
    return 0;
  } catch (std::exception&) {
    return 1;
  }
}

void orc_mask_from_points(uint32_t* bits, const int32_t glob[3], const int32_t offset[3],
                          const int32_t* points, int npoints) {
  for (int i = 0; i < npoints; ++i) {  // BitField::add_point (BitField.h:291-333)
    const int x = offset[0] + points[3 * i], y = offset[1] + points[3 * i + 1], z = offset[2] + points[3 * i + 2];
    const int pos = x + glob[0] * (y + glob[1] * z);
    bits[pos / 32] |= (1u << (pos % 32));
  }
}

// Every ghost cell takes its wrapped interior image.  Rows are visited once: a ghost row copies
// from its source row, an interior row only its ghost columns.  Sources are interior cells,
// which no iteration writes, so the rows may run on several threads in any order.
static void fill_periodic_threads(double* f, const int32_t n[3], int32_t g, int threads) {
  const int gx = n[0] + 2 * g, gy = n[1] + 2 * g, gz = n[2] + 2 * g;
#pragma omp parallel for num_threads(threads > 1 ? threads : 1) schedule(static)
  for (int zz = 0; zz < gz; ++zz) {
    const int z = zz - g;
    const bool zin = z >= 0 && z < n[2];
    const long szz = wrap(z, n[2]) + g;
    for (int yy = 0; yy < gy; ++yy) {
      const int y = yy - g;
      double* row = f + (long)gx * (yy + (long)gy * zz);
      const double* src = f + (long)gx * ((wrap(y, n[1]) + g) + (long)gy * szz);
      if (zin && y >= 0 && y < n[1]) {
        for (int x = -g; x < 0; ++x) row[x + g] = src[wrap(x, n[0]) + g];
        for (int x = n[0]; x < n[0] + g; ++x) row[x + g] = src[wrap(x, n[0]) + g];
      } else {
        for (int x = -g; x < n[0] + g; ++x) row[x + g] = src[wrap(x, n[0]) + g];
      }
    }
  }
}

static void copy_threads(double* dst, const double* src, size_t n, int threads) {
  const long chunk = 1 << 16;
  const long nchunks = (long)((n + chunk - 1) / chunk);
#pragma omp parallel for num_threads(threads > 1 ? threads : 1) schedule(static)
  for (long c = 0; c < nchunks; ++c) {
    const size_t lo = (size_t)c * chunk, hi = lo + chunk < n ? lo + chunk : n;
    std::memcpy(dst + lo, src + lo, (hi - lo) * sizeof(double));
  }
}

void orc_fill_periodic(double* f, const int32_t n[3], int32_t g) { fill_periodic_threads(f, n, g, 1); }

double orc_reduce_field(const double* f, const int32_t glob[3], int32_t g, int op, int interior) {
  const int lo = interior ? g : 0;
  double r = op == ORC_RED_MAX ? -std::numeric_limits<double>::infinity()
             : op == ORC_RED_MIN ? std::numeric_limits<double>::infinity() : 0.0;
  for (int z = lo; z < glob[2] - lo; ++z)
    for (int y = lo; y < glob[1] - lo; ++y)
      for (int x = lo; x < glob[0] - lo; ++x) {
        const double v = f[x + glob[0] * (y + glob[1] * z)];
        switch (op) {
          case ORC_RED_SUM: r = r + v; break;
          case ORC_RED_MAX: r = (r < v) ? v : r; break;
          case ORC_RED_MIN: r = (r > v) ? v : r; break;
          case ORC_RED_NORM: r = r + std::pow(v, 2.0); break;
        }
      }
  return op == ORC_RED_NORM ? std::sqrt(r) : r;
}

// ------------------------------------------------------------------------------------------
// Heat equation, explicit Euler, periodic ghosts, one ghost layer, unit spacing:
//   T' = T + dt*( DivX(InterpX(lam)*GradX(T)) + DivY(..) + DivZ(..) )
// with the reference's coefficients (StencilBuilder.cpp:60-72: interp {1/2,1/2},
// grad/div {-1/dx, 1/dx}, dx = L/n = 1) and its evaluation order (low point first, then
// (DivX + DivY) + DivZ).  Each step fills T's ghosts, writes the interior of Ttmp and swaps;
// after the last step T's ghosts are filled again.  The result ends in T.
void orc_heat_run(double* T, double* Ttmp, const double* lam, const int32_t n[3], int32_t steps,
                  double dt, int32_t threads) {
  const int gx = n[0] + 2, gy = n[1] + 2;
  const long sy = gx, sz = (long)gx * gy;
  const double c0 = -1.0 / 1.0, c1 = 1.0 / 1.0, h0 = 0.5, h1 = 0.5;
  double* cur = T;
  double* nxt = Ttmp;
  // uninitialised: the threads' copy touches the pages first
  const size_t npts = (size_t)gx * gy * (n[2] + 2);
  std::unique_ptr<double[]> lamf(new double[npts]);
  copy_threads(lamf.get(), lam, npts, threads);
  fill_periodic_threads(lamf.get(), n, 1, threads);
  const double* L = lamf.get();
  for (int s = 0; s < steps; ++s) {
    fill_periodic_threads(cur, n, 1, threads);
#pragma omp parallel for num_threads(threads > 1 ? threads : 1) schedule(static)
    for (int z = 0; z < n[2]; ++z)
      for (int y = 0; y < n[1]; ++y)
        for (int x = 0; x < n[0]; ++x) {
          const long i = (x + 1) + sy * (y + 1) + sz * (z + 1);
          // one direction: Div(Interp(lam)*Grad(T)) at cell i, faces i (low) and i+s (high)
          auto dir = [&](long s_) {
            const double flo = (L[i - s_] * h0 + L[i] * h1) * (cur[i - s_] * c0 + cur[i] * c1);
            const double fhi = (L[i] * h0 + L[i + s_] * h1) * (cur[i] * c0 + cur[i + s_] * c1);
            return flo * c0 + fhi * c1;
          };
          const double rhs = (dir(1) + dir(sy)) + dir(sz);
          nxt[i] = cur[i] + dt * rhs;
        }
    std::swap(cur, nxt);
  }
  fill_periodic_threads(cur, n, 1, threads);
  if (cur != T) copy_threads(T, cur, (size_t)gx * gy * (n[2] + 2), threads);
}

// Deep fused chain (one ghost layer, no BC):
//   out <<= 0; out <<= cond(mask, 0)(I(G(I(a))) * exp(b) + sin(c)); filt <<= 0; filt <<= Box(out)
// with I = Interp SVol->XVol {1/2,1/2} at points (-1,0), G = Grad XVol->SVol {-1/dx,1/dx} at
// points (0,+1), Box = 27-point sum (z outer, then y, then x, from -1) times 1/27.
// The write region of the cond is x in [1, n), y,z in [-1, n+1) (negative x ghost after the
// three stencils); Box writes the interior.
void orc_deep_run(const double* a, const double* b, const double* c, const uint32_t* maskbits,
                  double* out, double* filt, const int32_t n[3], double dx, int32_t threads) {
  const int gx = n[0] + 2, gy = n[1] + 2, gz = n[2] + 2;
  const long N = (long)gx * gy * gz;
  const long sy = gx, sz = (long)gx * gy;
  const double g0 = -1.0 / dx, g1 = 1.0 / dx;
#pragma omp parallel for num_threads(threads > 1 ? threads : 1) schedule(static)
  for (long i = 0; i < N; ++i) { out[i] = 0.0; filt[i] = 0.0; }
#pragma omp parallel for num_threads(threads > 1 ? threads : 1) schedule(static)
  for (int z = -1; z < n[2] + 1; ++z)
    for (int y = -1; y < n[1] + 1; ++y)
      for (int x = 1; x < n[0]; ++x) {
        const long i = (x + 1) + sy * (y + 1) + sz * (z + 1);
        double v;
        if ((maskbits[i / 32] >> (i % 32)) & 1u) {
          v = 0.0;
        } else {
          // I(a)[j] = a[j-1]*0.5 + a[j]*0.5 ; G(X)[k] = X[k]*g0 + X[k+1]*g1 ; I(S)[i] = S[i-1]*.5 + S[i]*.5
          auto Ia = [&](long j) { return a[j - 1] * 0.5 + a[j] * 0.5; };
          auto GIa = [&](long k) { return Ia(k) * g0 + Ia(k + 1) * g1; };
          const double igi = GIa(i - 1) * 0.5 + GIa(i) * 0.5;
          v = igi * std::exp(b[i]) + std::sin(c[i]);
        }
        out[i] = v;
      }
  const double w = 1.0 / 27.0;
#pragma omp parallel for num_threads(threads > 1 ? threads : 1) schedule(static)
  for (int z = 0; z < n[2]; ++z)
    for (int y = 0; y < n[1]; ++y)
      for (int x = 0; x < n[0]; ++x) {
        const long i = (x + 1) + sy * (y + 1) + sz * (z + 1);
        double s = out[i - 1 - sy - sz];
        bool first = true;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int ddx = -1; ddx <= 1; ++ddx) {
              if (first) { first = false; continue; }
              s = s + out[i + ddx + sy * dy + sz * dz];
            }
        filt[i] = s * w;
      }
}

// Scalar transport (two ghost layers, periodic, unit spacing).  Per direction d:
//   F_d = nu*I_d(lam)*G4_d(phi) - u_d*cond(u_d > 0, phi[i-1])(phi[i])     (on XVol/YVol/ZVol)
//   rhs = D_x(F_x) + D_y(F_y) + D_z(F_z),  D = Grad_{X->S} {-1, +1}
// G4 = {1, -27, 27, -1}/24 at points (-2,-1,0,+1); Heun's RK2:
//   phi1 = phi + dt*rhs(phi);  phin = 0.5*phi + 0.5*(phi1 + dt*rhs(phi1));  phi = phin
// Ghosts of phi/phi1 are filled before each stage.  Evaluation order follows the Nebo tree
// (nu*I)*G4, then minus u*cond, each stencil low point first.
namespace {
void transport_stage(const double* p, const double* base, double* dst, const double* u, const double* v,
                     const double* w, const double* lam, int n, double dt, double nu, int threads,
                     bool second) {
  const int G = 2, gx = n + 2 * G;
  const long sy = gx, sz = (long)gx * gx;
  const double h = 1.0 / 24.0;
  const double q0 = h, q1 = -27.0 * h, q2 = 27.0 * h, q3 = -h;
#pragma omp parallel for num_threads(threads > 1 ? threads : 1) schedule(static)
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        const long i = (x + G) + sy * (y + G) + sz * (z + G);
        auto flux = [&](long f, long s, const double* vel) {  // face f (between f-s and f)
          const double il = lam[f - s] * 0.5 + lam[f] * 0.5;
          const double g4 = ((p[f - 2 * s] * q0 + p[f - s] * q1) + p[f] * q2) + p[f + s] * q3;
          const double up = (vel[f] > 0.0) ? p[f - s] * 1.0 : p[f] * 1.0;
          return nu * il * g4 - vel[f] * up;
        };
        auto div = [&](long s, const double* vel) {
          return flux(i, s, vel) * -1.0 + flux(i + s, s, vel) * 1.0;
        };
        const double rhs = (div(1, u) + div(sy, v)) + div(sz, w);
        if (!second)
          dst[i] = p[i] + dt * rhs;
        else
          dst[i] = 0.5 * base[i] + 0.5 * (p[i] + dt * rhs);
      }
}
}  // namespace

void orc_transport_run(double* phi, double* phi1, double* phin, const double* u, const double* v,
                       const double* w, const double* lam, int32_t n, int32_t steps, double dt,
                       double nu, int32_t threads) {
  const int G = 2;
  const int32_t nn[3] = {n, n, n};
  const size_t N = (size_t)(n + 2 * G) * (n + 2 * G) * (n + 2 * G);
  std::vector<double> U(u, u + N), V(v, v + N), W(w, w + N), Lm(lam, lam + N);
  orc_fill_periodic(U.data(), nn, G);
  orc_fill_periodic(V.data(), nn, G);
  orc_fill_periodic(W.data(), nn, G);
  orc_fill_periodic(Lm.data(), nn, G);
  for (int s = 0; s < steps; ++s) {
    orc_fill_periodic(phi, nn, G);
    transport_stage(phi, phi, phi1, U.data(), V.data(), W.data(), Lm.data(), n, dt, nu, threads, false);
    orc_fill_periodic(phi1, nn, G);
    transport_stage(phi1, phi, phin, U.data(), V.data(), W.data(), Lm.data(), n, dt, nu, threads, true);
    // phi <<= phin copies the whole window; only the interior of phin was written this step
    std::memcpy(phi, phin, N * sizeof(double));
  }
  orc_fill_periodic(phi, nn, G);
}

// Adjoint of orc_heat_run.  Forward step k:  T_{k+1} = T_k + dt*R(lam, fill(T_k)) on the
// interior, with R(lam,T)[i] = sum_d (F_d[i+s_d] - F_d[i]),  F_d[f] = lamf_d[f]*(T[f]-T[f-s_d]),
// lamf_d[f] = 0.5*(lam[f-s_d] + lam[f]) after lam's periodic fill.  Reverse sweep with every
// state stored: gT_k = gT_{k+1} + dt*R(lam, gT_{k+1}) (R is self-adjoint on the periodic
// grid), glam += dt * dR/dlam^T gT_{k+1}.  The ghost fill's transpose folds each ghost
// contribution back onto its interior image, which the periodic wrap below expresses directly.
void orc_heat_adjoint(const double* T0, const double* lam, double* gT, double* glam,
                      const int32_t n[3], int32_t steps, double dt) {
  const int nx = n[0], ny = n[1], nz = n[2];
  const size_t NI = (size_t)nx * ny * nz;
  auto I = [&](int x, int y, int z) { return (size_t)wrap(x, nx) + nx * ((size_t)wrap(y, ny) + ny * (size_t)wrap(z, nz)); };
  const int gx = nx + 2, gy = ny + 2;
  std::vector<double> L(NI), Tin(NI);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const size_t gi = (x + 1) + gx * ((y + 1) + (size_t)gy * (z + 1));
        L[I(x, y, z)] = lam[gi];
        Tin[I(x, y, z)] = T0[gi];
      }
  // forward, storing states (interior only; periodic wrap replaces the ghost fill)
  std::vector<std::vector<double>> st(steps + 1, std::vector<double>(NI));
  st[0] = Tin;
  const int sx[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int k = 0; k < steps; ++k) {
    const std::vector<double>& T = st[k];
    std::vector<double>& Tn = st[k + 1];
    for (int z = 0; z < nz; ++z)
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
          double r[3];
          for (int d = 0; d < 3; ++d) {
            const int ax = sx[d][0], ay = sx[d][1], az = sx[d][2];
            const size_t c = I(x, y, z), lo = I(x - ax, y - ay, z - az), hi = I(x + ax, y + ay, z + az);
            const double flo = (L[lo] * 0.5 + L[c] * 0.5) * (T[lo] * -1.0 + T[c] * 1.0);
            const double fhi = (L[c] * 0.5 + L[hi] * 0.5) * (T[c] * -1.0 + T[hi] * 1.0);
            r[d] = flo * -1.0 + fhi * 1.0;
          }
          Tn[I(x, y, z)] = T[I(x, y, z)] + dt * ((r[0] + r[1]) + r[2]);
        }
  }
  // reverse
  std::vector<double> a(NI), an(NI), gl(NI, 0.0);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) a[I(x, y, z)] = gT[(x + 1) + gx * ((y + 1) + (size_t)gy * (z + 1))];
  for (int k = steps - 1; k >= 0; --k) {
    const std::vector<double>& T = st[k];
    for (int z = 0; z < nz; ++z)
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
          const size_t c = I(x, y, z);
          double r = 0.0, g = 0.0;
          for (int d = 0; d < 3; ++d) {
            const int ax = sx[d][0], ay = sx[d][1], az = sx[d][2];
            const size_t lo = I(x - ax, y - ay, z - az), hi = I(x + ax, y + ay, z + az);
            const double lf_lo = 0.5 * (L[lo] + L[c]), lf_hi = 0.5 * (L[c] + L[hi]);
            r += lf_hi * (a[hi] - a[c]) - lf_lo * (a[c] - a[lo]);
            // dJ/dlam[c]: both faces touching c use 0.5*lam[c]
            g += 0.5 * (T[c] - T[lo]) * (a[lo] - a[c]) + 0.5 * (T[hi] - T[c]) * (a[c] - a[hi]);
          }
          an[c] = a[c] + dt * r;
          gl[c] += dt * g;
        }
    std::swap(a, an);
  }
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const size_t gi = (x + 1) + gx * ((y + 1) + (size_t)gy * (z + 1));
        gT[gi] = a[I(x, y, z)];
        glam[gi] += gl[I(x, y, z)];
      }
}

}  // extern "C"

// ---------------------------------------------------------------- particle <-> cell operators
namespace {

struct PartBox {
  long lo[3], hi[3];
  double plo[3], phi[3], face[3];
  double pvol;
};

// The box of window cells particle p touches (ParticleOperators.h:214-238 / 337-361).
void part_box(PartBox& b, const double d[3], const double low[3], const int32_t ngm[3], const int32_t glob[3],
              const int32_t nmax[3], const double* const pos[3], const double* psize, int64_t p) {
  const double rp = psize[p] * 0.5;
  for (int a = 0; a < 3; ++a) {
    b.face[a] = low[a] - d[a] * ngm[a] - d[a] / 2;
    b.plo[a] = pos[a] ? pos[a][p] - rp : 0;
    b.phi[a] = pos[a] ? b.plo[a] + psize[p] : 0;
    const double ql = (b.plo[a] - b.face[a]) / d[a];
    // size_t conversion of the reference; a negative quotient clips to cell 0
    b.lo[a] = !(ql < (double)nmax[a]) ? nmax[a] : (ql > 0 ? (long)ql : 0);
    if (pos[a]) {
      const double qh = (b.phi[a] - b.face[a]) / d[a];
      if (!(qh > -1.0))
        b.hi[a] = 0;
      else
        b.hi[a] = qh >= (double)nmax[a] ? nmax[a] : std::min((long)nmax[a], (long)(int)qh + 1);
    } else if (glob[a] == 1) {
      b.lo[a] = 0;  // flat_index maps every index of an extent-1 axis to 0
      b.hi[a] = 1;
    } else {
      b.hi[a] = std::min((long)nmax[a], b.lo[a] + 1);
    }
  }
  b.pvol = (pos[0] ? 2 * rp : 1) * (pos[1] ? 2 * rp : 1) * (pos[2] ? 2 * rp : 1);
}

double part_cont(const PartBox& b, const double d[3], const double* const pos[3], int a, long i) {
  if (!pos[a]) return 1;
  const double cm = b.face[a] + i * d[a];
  const double cp = cm + d[a];
  return std::min(cp, b.phi[a]) - std::max(cm, b.plo[a]);
}

size_t part_flat(const int32_t glob[3], const int32_t off[3], long i, long j, long k) {
  const long x = glob[0] > 1 ? i + off[0] : 0, y = glob[1] > 1 ? j + off[1] : 0, z = glob[2] > 1 ? k + off[2] : 0;
  return (size_t)x + (size_t)glob[0] * ((size_t)y + (size_t)glob[1] * (size_t)z);
}

}  // namespace

extern "C" {

void orc_cell_to_particle(const double spacing[3], const double low[3], const int32_t ngm[3], const int32_t glob[3],
                          const int32_t off[3], const int32_t nmax[3], const double* cell, const double* px,
                          const double* py, const double* pz, const double* psize, int64_t np, double* dest) {
  const double* const pos[3] = {px, py, pz};
  for (int64_t p = 0; p < np; ++p) {
    PartBox b;
    part_box(b, spacing, low, ngm, glob, nmax, pos, psize, p);
    dest[p] = 0.0;
    for (long k = b.lo[2]; k < b.hi[2]; ++k) {
      const double zc = part_cont(b, spacing, pos, 2, k);
      for (long j = b.lo[1]; j < b.hi[1]; ++j) {
        const double yc = part_cont(b, spacing, pos, 1, j);
        for (long i = b.lo[0]; i < b.hi[0]; ++i) {
          const double xc = part_cont(b, spacing, pos, 0, i);
          dest[p] += cell[part_flat(glob, off, i, j, k)] * (xc * yc * zc / b.pvol);
        }
      }
    }
  }
}

void orc_particle_to_cell(const double spacing[3], const double low[3], const int32_t ngm[3], const int32_t glob[3],
                          const int32_t off[3], const int32_t nmax[3], double* cell, const double* px,
                          const double* py, const double* pz, const double* psize, int64_t np, const double* src) {
  for (long k = 0; k < nmax[2]; ++k)
    for (long j = 0; j < nmax[1]; ++j)
      for (long i = 0; i < nmax[0]; ++i) cell[part_flat(glob, off, i, j, k)] = 0.0;
  const double* const pos[3] = {px, py, pz};
  for (int64_t p = 0; p < np; ++p) {
    PartBox b;
    part_box(b, spacing, low, ngm, glob, nmax, pos, psize, p);
    for (long k = b.lo[2]; k < b.hi[2]; ++k) {
      const double zc = part_cont(b, spacing, pos, 2, k);
      for (long j = b.lo[1]; j < b.hi[1]; ++j) {
        const double yc = part_cont(b, spacing, pos, 1, j);
        for (long i = b.lo[0]; i < b.hi[0]; ++i) {
          const double xc = part_cont(b, spacing, pos, 0, i);
          cell[part_flat(glob, off, i, j, k)] += src[p] * (xc * yc * zc / b.pvol);
        }
      }
    }
  }
}

}  // extern "C"
