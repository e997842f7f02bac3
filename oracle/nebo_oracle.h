/*
 * nebo_oracle.h -- CPU restatement of the reference's serial Nebo evaluation.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py load it as the checker.  The product (the CUDA library and
 * the drop-in headers) never links, includes or calls it, and has no CPU fallback.
 *
 * Parity: pinned.  tests/test_oracle_golden.py checks this restatement bit-for-bit against
 * golden vectors that the reference's own headers produced (tests/golden/, generated by
 * tests/golden/make_golden.py through oracle/_ref/ref_driver).
 *
 * What it restates (reference file:line):
 *   GhostData algebra ............ spatialops/structured/GhostData.h:54-257
 *   calculate_actual_ghost ........ spatialops/NeboBasic.h:61-100
 *   NeboField::assign / seqwalk ... spatialops/NeboLhs.h:67-162, 592-631
 *   masked_assign point loop ...... spatialops/NeboLhs.h:164-283
 *   leaves (field, scalar) ........ spatialops/NeboRhs.h:29-328
 *   pointwise operators ........... spatialops/NeboOperators.h (SumOp :32 ... PowInt :14598)
 *   cond clause chain ............. spatialops/NeboCond.h:253-445
 *   mask bit lookup ............... spatialops/NeboMask.h:130-197, structured/BitField.h:291-333
 *   stencil fold order ............ spatialops/NeboStencils.h:280-524, 826-1046
 *   reductions (nebo_fold) ........ spatialops/NeboReductions.h:45-240
 *   particle <-> cell operators ... spatialops/particles/ParticleOperators.h:186-273, 313-398
 *
 * Expressions arrive as a prefix-encoded int32 program plus a table of double immediates:
 *   ORC_FIELD  idx                 field leaf (index into the field table)
 *   ORC_SCALAR imm                 scalar leaf (index into the immediates)
 *   ORC_BIN    op  a b             + - * / pow max min
 *   ORC_UN     fn  a               neg sin cos tan exp tanh abs sqrt log log10 erf erfc square cube
 *   ORC_POWINT e   a               pow(a, int e)
 *   ORC_CMP    op  a b             == != < <= > >=          (boolean)
 *   ORC_LOGIC  op  a [b]           && || !                  (boolean)
 *   ORC_COND   n   (test value)*n default
 *   ORC_MASK   idx                 mask leaf                (boolean)
 *   ORC_STENCIL npts (dx dy dz)*npts coef_imm0  arg         weighted stencil
 *   ORC_SUMSTENCIL npts (dx dy dz)*npts  arg                unweighted stencil
 */
#ifndef NEBO_ORACLE_H
#define NEBO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_FIELD = 1, ORC_SCALAR = 2, ORC_BIN = 3, ORC_UN = 4, ORC_POWINT = 5, ORC_CMP = 6,
  ORC_LOGIC = 7, ORC_COND = 8, ORC_MASK = 9, ORC_STENCIL = 10, ORC_SUMSTENCIL = 11
};
enum { ORC_ADD = 0, ORC_SUB, ORC_MUL, ORC_DIV, ORC_POW, ORC_MAX, ORC_MIN };
enum {
  ORC_NEG = 0, ORC_SIN, ORC_COS, ORC_TAN, ORC_EXP, ORC_TANH, ORC_ABS, ORC_SQRT, ORC_LOG,
  ORC_LOG10, ORC_ERF, ORC_ERFC, ORC_SQUARE, ORC_CUBE
};
enum { ORC_EQ = 0, ORC_NE, ORC_LT, ORC_LE, ORC_GT, ORC_GE };
enum { ORC_AND = 0, ORC_OR, ORC_NOT };
enum { ORC_RED_SUM = 0, ORC_RED_MAX, ORC_RED_MIN, ORC_RED_NORM };

/* A field: one allocation covering the ghosted window (window offset 0, extent = glob). */
typedef struct {
  double* data;
  int32_t glob[3];
  int32_t ghost_minus[3]; /* ghosts the field was built with (before limit_by_extent) */
  int32_t ghost_plus[3];
  int32_t has_bc[3];
  int32_t bc_extra[3]; /* the location's BCExtra; counted only on axes with has_bc */
} orc_field;

/* A mask: bit-packed 32-bit words over the same ghosted window, x fastest. */
typedef struct {
  const uint32_t* bits;
  int32_t glob[3];
  int32_t ghost_minus[3];
  int32_t ghost_plus[3];
  int32_t has_bc[3];
  int32_t bc_extra[3];
} orc_mask;

typedef struct {
  const int32_t* prog;
  int32_t prog_len;
  const double* imms;
  const orc_field* fields;
  int32_t nfields;
  const orc_mask* masks;
  int32_t nmasks;
} orc_expr;

/* Return 0 on success; on a reference error, copy its message into err and return 1. */
int orc_assign(const orc_expr* e, const orc_field* lhs, int use_ghost, char* err, int errlen);
int orc_write_limits(const orc_expr* e, const orc_field* lhs, int use_ghost, int32_t limits[6],
                     char* err, int errlen);
int orc_masked_assign(const orc_expr* e, const orc_field* lhs, const int32_t* points, int npoints,
                      char* err, int errlen);
int orc_reduce(const orc_expr* e, int op, int use_ghost, double* result, char* err, int errlen);
int orc_ghosts(const orc_expr* e, int with_bc, int32_t minus[3], int32_t plus[3]);

/* Mask words from interior-relative points (ghost = -1 ...). */
void orc_mask_from_points(uint32_t* bits, const int32_t glob[3], const int32_t offset[3],
                          const int32_t* points, int npoints);

/* Periodic ghost fill: every ghost cell takes the value of its wrapped interior image. */
void orc_fill_periodic(double* f, const int32_t n[3], int32_t g);

/* Workload drivers, written as direct loops in the reference's evaluation order.
 * threads <= 1 runs the serial walk; threads > 1 splits z into slabs (the Threading
 * backend's partition of the write region, spatialops/NeboBasic.h:112-178). */
void orc_heat_run(double* T, double* Ttmp, const double* lam, const int32_t n[3], int32_t steps,
                  double dt, int32_t threads);
void orc_deep_run(const double* a, const double* b, const double* c, const uint32_t* maskbits,
                  double* out, double* filt, const int32_t n[3], double dx, int32_t threads);
void orc_transport_run(double* phi, double* phi1, double* phin, const double* u, const double* v,
                       const double* w, const double* lam, int32_t n, int32_t steps, double dt,
                       double nu, int32_t threads);

/* Adjoint of orc_heat_run (no counterpart in the reference): given T0, lam and dJ/dT_N,
 * returns dJ/dT0 (in gT, overwritten in place) and dJ/dlam (accumulated into glam),
 * by storing every forward state (small cases only). */
void orc_heat_adjoint(const double* T0, const double* lam, double* gT, double* glam,
                      const int32_t n[3], int32_t steps, double dt);

/* Serial left fold over the ghosted window of one field (nebo_sum/max/min/norm). */
double orc_reduce_field(const double* f, const int32_t glob[3], int32_t g, int op, int interior);

/* Particle <-> cell operators (spatialops/particles/ParticleOperators.h:186-273 ParticleToCell,
 * :313-398 CellToParticle), serial loops in the reference's order.  The cell field is one
 * allocation of glob points whose window (ghosts included) starts at off and spans nmax;
 * spacing / low are the operator's state after its constructor (:153-166), ngm the field's ghost
 * cells on the - faces.  px, py, pz may be NULL (axis off).  A box that leaves the window is
 * clipped to it at both ends (the reference clips only the high end; its low end is undefined).
 * orc_particle_to_cell first sets every window cell to +0 (the reference's dest <<= 0). */
void orc_cell_to_particle(const double spacing[3], const double low[3], const int32_t ngm[3],
                          const int32_t glob[3], const int32_t off[3], const int32_t nmax[3],
                          const double* cell, const double* px, const double* py, const double* pz,
                          const double* psize, int64_t np, double* dest);
void orc_particle_to_cell(const double spacing[3], const double low[3], const int32_t ngm[3],
                          const int32_t glob[3], const int32_t off[3], const int32_t nmax[3],
                          double* cell, const double* px, const double* py, const double* pz,
                          const double* psize, int64_t np, const double* src);

#ifdef __cplusplus
}
#endif
#endif
