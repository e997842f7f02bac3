/*
 * nebo_gb300.h -- C ABI of the GB300-native (sm_103a) Nebo field-expression evaluator.
 *
 * Everything here is plain C: device pointers, sizes, POD descriptors and an int status.
 * No exception crosses this boundary; the C++ drop-in headers (include/spatialops/...) turn a
 * non-zero status into std::runtime_error("Nebo error in ..."), as the reference does
 * (spatialops/NeboLhs.h:107-152, spatialops/NeboBasic.h:65-93).
 *
 * One process drives one GPU.  Every launching entry point takes the cudaStream_t on which it
 * enqueues its work (the reference's per-field stream, spatialops/structured/FieldInfo.h:264)
 * and returns without synchronising unless it says otherwise.  A null stream means the
 * per-thread default stream.
 *
 * Layout contract (spatialops/structured/MemoryWindow.h:63-321): a field is one allocation of
 * glob[0]*glob[1]*glob[2] elements, x fastest; interior-relative index (x,y,z) lives at
 *   (offset[0]+ghost_minus[0]+x) + glob[0]*((offset[1]+ghost_minus[1]+y) + glob[1]*(...z))
 * with glob = n + ghost_minus + ghost_plus (+ one BC cell on + faces that have a boundary and
 * whose location carries BCExtra), or 1 on an axis of extent 1.
 */
#ifndef NEBO_GB300_H
#define NEBO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* nebo_stream_t; /* == cudaStream_t */

/* ------------------------------------------------------------------ status */
enum nebo_status_code {
  NEBO_OK = 0,
  NEBO_ERR_INVALID = 1,   /* bad descriptor, size, pointer or argument */
  NEBO_ERR_GHOST = 2,     /* not enough valid ghost / BC cells (NeboBasic.h:65-93) */
  NEBO_ERR_ALLOC = 3,     /* device allocation failed */
  NEBO_ERR_LAUNCH = 4,    /* kernel launch or CUDA runtime error */
  NEBO_ERR_TIMEOUT = 5,   /* a bounded device-side wait gave up */
  NEBO_ERR_UNSUPPORTED = 6,
  NEBO_ERR_NO_DEVICE = 7
};

enum nebo_dtype { NEBO_F64 = 0, NEBO_F32 = 1, NEBO_F32X2 = 2 /* two-float state (patchsets only) */ };

enum nebo_reduction { NEBO_RED_SUM = 0, NEBO_RED_MAX = 1, NEBO_RED_MIN = 2, NEBO_RED_NORM = 3 };

/* Field descriptor: SpatialField's window/ghost/BC state (SpatialField.h:128-603). */
typedef struct nebo_field {
  void* data;              /* device pointer to glob element (0,0,0) */
  int32_t glob[3];         /* MemoryWindow::glob_dim */
  int32_t offset[3];       /* MemoryWindow::offset */
  int32_t extent[3];       /* MemoryWindow::extent (window incl. ghosts) */
  int32_t ghost_minus[3];  /* valid ghost cells on - faces */
  int32_t ghost_plus[3];   /* valid ghost cells on + faces */
  int32_t has_bc[3];       /* BoundaryCellInfo::has_bc */
  int32_t bc_extra[3];     /* BoundaryCellInfo::has_extra (0 or the location's BCExtra) */
  int32_t dtype;           /* nebo_dtype */
} nebo_field;

/* Human-readable text of a status code; the last error message of the calling thread. */
const char* nebo_status_string(int status);
const char* nebo_last_error(void);

/* ------------------------------------------------------------------ device and memory
 * Replace FieldInfo's device bookkeeping and the Pool<T> / CUDADeviceInterface allocator
 * (spatialops/structured/FieldInfo.h:92-415, MemoryPool.cpp:104-216,
 *  CudaMemoryAllocator.cu:28-240, 390-578).  Allocation is stream ordered
 * (cudaMallocAsync on the device's default memory pool). */
int nebo_device_init(int device);
int nebo_device_count(int* count);
int nebo_alloc(size_t bytes, void** ptr, nebo_stream_t stream);
int nebo_free(void* ptr, nebo_stream_t stream);
int nebo_memcpy_h2d(void* dst, const void* src, size_t bytes, nebo_stream_t stream);
int nebo_memcpy_d2h(void* dst, const void* src, size_t bytes, nebo_stream_t stream);
int nebo_memcpy_d2d(void* dst, const void* src, size_t bytes, nebo_stream_t stream);
int nebo_memset(void* dst, int byte, size_t bytes, nebo_stream_t stream);
/* nebo_stream_sync also reports NEBO_ERR_TIMEOUT when a bounded device-side wait of a kernel
 * (the FP32 heat step's bulk-copy barriers give up after about a second) gave up since the last
 * report; the kernel's results are then not valid. */
int nebo_stream_sync(nebo_stream_t stream);

/* ------------------------------------------------------------------ ghost bookkeeping (host)
 * calculate_actual_ghost (spatialops/NeboBasic.h:61-100) and the write region of
 * NeboField<Initial>::assign (spatialops/NeboLhs.h:67-98).  Integer host code, exact.
 * rhs_minus/rhs_plus: ghosts_with_bc() of the right-hand side.  limits = {xlo,xhi,ylo,yhi,
 * zlo,zhi} in interior-relative coordinates.  Returns NEBO_ERR_GHOST with the reference's
 * message when a BC axis lacks valid extra cells. */
int nebo_write_limits(const nebo_field* lhs, int use_ghost, const int32_t rhs_minus[3],
                      const int32_t rhs_plus[3], int32_t limits[6]);

/* ------------------------------------------------------------------ periodic ghost exchange
 * Every ghost cell of f takes the value of its wrapped interior image (the in-HBM stand-in for
 * a halo exchange on a single periodic patch).  f must have equal ghosts on both faces and no
 * BC cells. */
int nebo_fill_periodic(const nebo_field* f, nebo_stream_t stream);

/* ------------------------------------------------------------------ masks
 * SpatialMask / BitField (spatialops/structured/SpatialMask.h:99-181, BitField.h:291-333):
 * one bit per cell of the ghosted window, word = flat/32, bit = flat%32, x fastest.
 * points: device int32 triples in interior-relative coordinates (ghost = -1).  words must be
 * zeroed by the caller (nebo_memset) or hold an earlier mask to OR into. */
int nebo_mask_from_points(uint32_t* words, const int32_t glob[3], const int32_t offset[3],
                          const int32_t* points, int32_t npoints, nebo_stream_t stream);

/* ------------------------------------------------------------------ reductions
 * nebo_sum / nebo_max / nebo_min / nebo_norm and their _interior forms
 * (spatialops/NeboReductions.h:45-240) over one field: ghost-inclusive (valid ghosts) unless
 * interior != 0.  Accumulation is FP64 for both dtypes; sums use compensated (Neumaier)
 * partials.  nebo_reduce writes *result on the host and synchronises the stream (the reference
 * returns the value synchronously); nebo_reduce_async leaves it in device memory. */
int nebo_reduce(const nebo_field* f, int op, int interior, double* result, nebo_stream_t stream);
int nebo_reduce_async(const nebo_field* f, int op, int interior, double* d_result,
                      nebo_stream_t stream);

/* sum, max, min and norm of the same region in ONE pass (d_out4[0..3], device memory): each
 * element costs two FP64 operations; max/min compare order-preserving integer keys (NaNs are
 * skipped, as the reference's comparisons skip them). */
int nebo_reduce_all(const nebo_field* f, int interior, double* d_out4, nebo_stream_t stream);

/* Same reduction, same result as nebo_reduce_async, but it allocates nothing: no counterpart in
 * the reference.  For callers that must not enter the CUDA allocator at the call (a host
 * framework that reserved the device memory up front in its own pool, so another allocation
 * fails or breaks its accounting; code running where the allocator may not be entered).  The
 * block partials live in a fixed device array of 1024 slots (16 KiB, held on every GPU that
 * loads the library until exit); a reduction takes at most 1024 blocks, one slot each, whatever
 * the GPU's SM count.  A region of more than 2^31 - 1 rows (y * z extent) is rejected with
 * NEBO_ERR_INVALID before any CUDA call.  The first call on a device looks the array up
 * (cudaGetSymbolAddress) with that device current and should come before any stream capture;
 * the address is cached, and a cudaDeviceReset voids it.  All calls share the array: calls whose
 * kernels overlap on the GPU race on it.  The result is written to d_result. */
int nebo_reduce_noalloc(const nebo_field* f, int op, int interior, double* d_result,
                        nebo_stream_t stream);

/* ------------------------------------------------------------------ fused heat equation
 * One explicit Euler step of the reference's scalar heat RHS
 *   Tout <<= T + dt*( DivX(InterpX(lam)*GradX(T)) + DivY(...) + DivZ(...) )
 * (examples/heat_equation.cpp:216-220; operators of StencilBuilder.cpp:60-72 on SVolField)
 * as ONE kernel on a single periodic patch: reads T's ghosts, writes Tout's interior and, in
 * the same pass, Tout's ghost cells as periodic images (the next step's ghost fill).
 * T, Tout, lam: SVol, one ghost layer, same shape and dtype.  spacing = {dx,dy,dz}.
 * FP64: same operations and roundings as the reference's serial walk (bit-exact).
 * FP32: FP32 storage and arithmetic. */
int nebo_heat_step(const nebo_field* T, const nebo_field* Tout, const nebo_field* lam, double dt,
                   const double spacing[3], nebo_stream_t stream);

/* steps Euler steps, ping-ponging T and Ttmp; the result is left in T (ghosts filled).
 * use_graph != 0 captures the step sequence in a CUDA graph once and replays it. */
int nebo_heat_run(const nebo_field* T, const nebo_field* Ttmp, const nebo_field* lam, int steps,
                  double dt, const double spacing[3], int use_graph, nebo_stream_t stream);

/* nebo_heat_run with a choice of arithmetic (no graph):
 *   NEBO_HEAT_EXACT        the bit-exact FP64 form of nebo_heat_step;
 *   NEBO_HEAT_FIXED_POINT  FP64 storage; each face flux (lam_a + lam_b)(T_b - T_a) and the
 *                          divergence exact in 64/128-bit integers at a per-field scale (the
 *                          largest exponent of T, carried from step to step), then
 *                          T' = fma(dt/2, RN(divergence), T): one FP64 operation per cell, the
 *                          rest on the integer pipe.  Within a few 2^-60 of max|T| per step of
 *                          the exact form (not bit-identical).  FP64, unit spacing.
 *   NEBO_HEAT_FIXED_STATE  FP64 fields in and out; the run keeps T as signed 64-bit integers
 *                          (about 60 bits below the largest |T|, rescaled as the values grow or
 *                          decay) and (dt/2) lambda as 64-bit integers, so a step is integer
 *                          arithmetic only: face flux = high half of (lw_a + lw_b)(T_b - T_a),
 *                          T' = T + divergence.  Within a few 2^-60 of max|T| per step of the
 *                          exact form; one rounding back to FP64 at the end.  Needs scratch for
 *                          one FP64 field (the lambda weights).  FP64, unit spacing.
 * Both non-exact modes run the exact form (bit-identical) when T or lam holds an infinity or a
 * NaN, or when the scales leave the ranges the integer forms cover. */
enum { NEBO_HEAT_EXACT = 0, NEBO_HEAT_FIXED_POINT = 1, NEBO_HEAT_FIXED_STATE = 2 };
/* OR'd into mode: capture the call's launches (conversions and steps) in a CUDA graph the first
 * time and replay it for the same arguments, as nebo_heat_run's use_graph does (for small grids,
 * where launches bound the steps; the graph keeps its scratch in the stream-ordered pool). */
enum { NEBO_HEAT_GRAPH = 0x100 };
int nebo_heat_run_ex(const nebo_field* T, const nebo_field* Ttmp, const nebo_field* lam, int steps,
                     double dt, const double spacing[3], int mode, nebo_stream_t stream);

/* ------------------------------------------------------------------ deep fused chain
 *   out <<= cond(mask, 0.0)( Interp_{S->X}(Grad_{X->S}(Interp_{S->X}(a))) * exp(b) + sin(c) )
 *   filt <<= Filter_{X->X}(out)                       (27-point box, 1/27)
 * a: SVol, b, c, out, filt: XVol, one ghost layer, no BC, FP64; mask: XVol bit words.
 * Write regions follow calculate_actual_ghost: out is written on x in [1,n), y,z in [-1,n+1)
 * (the chain's negative x ghost); filt on the interior.  Cells outside keep their contents.
 * dx: the x spacing of the gradient (coefficients -1/dx, 1/dx). */
int nebo_deep_chain(const nebo_field* a, const nebo_field* b, const nebo_field* c,
                    const uint32_t* mask_words, const nebo_field* out, const nebo_field* filt,
                    double dx, nebo_stream_t stream);

/* nebo_deep_chain followed by nebo_sum, nebo_max, nebo_min and nebo_norm of filt
 * (spatialops/NeboReductions.h:114-240; interior != 0: the _interior variants), with the
 * reductions folded into the filter kernel as it writes filt (valid ghost cells of filt, which
 * the filter does not write, are reduced by a small extra pass).  d_out4 (device, 4 doubles)
 * receives {sum, max, min, norm} as nebo_reduce_all gives them; nothing is synchronised. */
int nebo_deep_chain_reduce(const nebo_field* a, const nebo_field* b, const nebo_field* c,
                           const uint32_t* mask_words, const nebo_field* out, const nebo_field* filt,
                           double dx, int interior, double* d_out4, nebo_stream_t stream);

/* filt <<= BoxFilter3D(src) alone (the filter of nebo_deep_chain; 27 points, coefficient 1/27,
 * spatialops/NeboStencilBuilder.h:454-465) over the interior, for any FP64 field with one
 * periodic-style ghost layer (window = allocation, no BC cells).  The 9-point sum of each plane
 * is exact in 128-bit fixed point and rounded once; the three plane sums add in FP64 (see
 * deep.cu); the value is within 1e-13 of the reference's FP64 sum, relative to the sum of the
 * 27 magnitudes.  d_out4 non-null: {sum, max, min, norm} of dst as nebo_reduce_all gives
 * them (ghost-inclusive unless interior), folded into the same pass. */
int nebo_box_filter(const nebo_field* src, const nebo_field* dst, int interior, double* d_out4,
                    nebo_stream_t stream);

/* Element-wise FP64 exp (fn 0) or sin (fn 1) with the functions nebo_deep_chain uses: the
 * argument reduction's one exact product in FP64, the rest in FP32, 32-bit and 64-bit fixed
 * point (Tang's 2^(j/256) table for exp; sin/cos(k pi/256) for sin).  Within 0.52 ulp (exp,
 * |x| < 708) and about 1.1 ulp (sin, |x| < 2^20) of the exact result; other arguments use
 * CUDA's exp and sin.  fn 2 and 3 take n pairs (a, b) in x (2n doubles) and write a / b:
 * fn 2 through the reciprocal-and-correction quotient the particle operators use, fn 3 by
 * plain division; both must agree bit for bit. */
int nebo_fastmath_eval(int fn, const double* x, double* y, size_t n, nebo_stream_t stream);

/* ------------------------------------------------------------------ batched patches
 * Many independent periodic heat-equation patches (one ghost layer, scalar lambda and dt per
 * patch) advanced together: each time step is ONE persistent launch over a device patch table
 * and a work list of (patch, tile or row strip, z-chunk) items; nebo_patchset_run captures the steps in a
 * CUDA graph.  The reference advances such patches one `<<=` at a time from the caller's patch
 * loop (one gpu_assign_kernel launch per expression and patch, spatialops/NeboLhs.h:29-41).
 *   create:   shapes = 3 ints per patch (interior nx, ny, nz >= 2); allocates two FP64 state
 *             arenas holding every patch window (x fastest), returned by nebo_patchset_arena(ps,
 *             0|1); the element offset of each window comes from nebo_patchset_info.  dtype
 *             NEBO_F32 keeps the working state in FP32 (storage and arithmetic: half the bytes);
 *             NEBO_F32X2 keeps it as two floats (hi + lo, ~48-bit significand) with FP32
 *             arithmetic only.  In both, results reach the FP64 arena through nebo_patchset_sync.
 *   fill_ghosts: periodic ghost images of an FP64 arena, then its FP32 / two-float working copy;
 *             call after loading the FP64 arena.
 *   sync:     after run, make the FP64 arena `which` hold the state (FP32: widened, FP32X2:
 *             hi + lo).
 *   autotune: times tile widths 16/32/64 per x-extent class and keeps the fastest; in NEBO_F32
 *             mode (row strips of up to 1024 cells, no tile width) it picks the z extent of the
 *             work items instead (whole patch, 32 or 16 planes).  Clobbers the arenas: call it
 *             before loading data.
 *   run:      `steps` steps from arena `start`; *final_arena says where the result is.  In
 *             NEBO_F32 mode the steps read their halos from the periodic sources and write no
 *             ghost cells; the run ends by filling the ghosts of the result arena (one launch,
 *             part of the graph), so the result is a full window as in the other modes.
 * FP64 results are bit-identical to the reference's serial walk on a constant lambda field. */
typedef struct nebo_patchset nebo_patchset;
int nebo_patchset_create(nebo_patchset** ps, int npatch, const int32_t* shapes, const double* lam,
                         const double* dt, int dtype);
int nebo_patchset_destroy(nebo_patchset* ps);
int nebo_patchset_info(const nebo_patchset* ps, int64_t* total_elems, int64_t* offsets,
                       int32_t* log2_tile_x, int32_t* nitems);
void* nebo_patchset_arena(const nebo_patchset* ps, int which);
int nebo_patchset_fill_ghosts(const nebo_patchset* ps, int which, nebo_stream_t stream);
int nebo_patchset_sync(const nebo_patchset* ps, int which, nebo_stream_t stream);
int nebo_patchset_autotune(nebo_patchset* ps, nebo_stream_t stream, int32_t* chosen_log2_tile_x);
int nebo_patchset_run(nebo_patchset* ps, int start, int steps, int use_graph, int* final_arena,
                      nebo_stream_t stream);

/* ------------------------------------------------------------------ scalar transport
 * Heun RK2 steps of  d(phi)/dt = sum_d Grad_{d->S}( nu*Interp(lambda)*G4_d(phi)
 *                                                  - u_d*cond(u_d > 0, phi[i-1])(phi[i]) )
 * on an n^3 periodic SVol patch with two ghost layers (G4: 4th-order staggered gradient
 * {1,-27,27,-1}/24 at (-2,-1,0,+1); unit spacing).  phi: FP64 state window, updated in place.
 * u, v, w (XVol/YVol/ZVol face velocities) and lambda: windows of the same shape in `dtype`.
 * dtype NEBO_F32: FP32 storage and stencil arithmetic, FP64 time accumulation (phi stays FP64);
 * dtype NEBO_F64: everything FP64.  work: device scratch of nebo_transport_work_bytes bytes.
 * Each RK stage is one kernel.  FP32 with n even: staged planes (8-byte copies), and with every
 * float field 8-byte aligned two cells per thread in packed FP32x2 arithmetic; odd n or
 * unaligned fields take a one-cell kernel (same results within FP32 rounding).  The coefficient
 * ghost fills and the FP32 copy of the state are made once per call: run many steps per call. */
size_t nebo_transport_work_bytes(int n, int dtype);
int nebo_transport_run(double* phi, const void* u, const void* v, const void* w, const void* lam,
                       int n, int steps, double dt, double nu, int dtype, void* work,
                       nebo_stream_t stream);

/* ------------------------------------------------------------------ adjoint (differentiation)
 * No counterpart in the reference (it has no differentiation).  Gradients of
 *   J = 1/2 * sum_interior (T_N - T_target)^2,   T_{k+1} = nebo_heat_step(T_k, lambda, dt)
 * (unit spacing, periodic, one ghost layer, FP64) with respect to T_0 and lambda.
 * nebo_heat_adjoint_step: one reverse step -- Aout = A_{k+1} + dt*R(lambda, A_{k+1}) (the
 *   heat operator is self-adjoint on the periodic grid; the ghost fill's transpose folds ghost
 *   contributions onto interior images) and glam -= (dt/2)*sum of face (dT*dA) terms at T_k.
 *   Inputs need periodic ghost images (T_k, A_{k+1}, lambda); Aout gets images.
 * nebo_heat_gradient: forward sweep keeping every L-th state (L = checkpoint_every, or
 *   ceil(sqrt(steps)) when <= 0), then the reverse sweep recomputing each segment from its
 *   checkpoint: device memory ~ (steps/L + L) fields.  checkpoint_every = NEBO_CHECKPOINT_AUTO
 *   keeps every state (L = 1, no recomputation: one forward sweep instead of two) when
 *   steps + 7 fields fit in 80 % of the free device memory, else takes ceil(sqrt(steps)).
 *   Writes gT0 = dJ/dT_0 (window with images), glam = dJ/dlambda (interior; ghosts zero)
 *   and *J; the results do not depend on L. */
enum { NEBO_CHECKPOINT_AUTO = -1 };
/* nebo_heat_gradient with a choice of face-product precision in the lambda gradient:
 *   NEBO_PRODUCTS_F64  as nebo_heat_gradient (every operation FP64);
 *   NEBO_PRODUCTS_F32  the per-face products (T_b - T_a)(A_b - A_a) of the lambda gradient are
 *                      FP32 products of the exactly computed FP64 differences, summed per cell in
 *                      FP32 and accumulated into glam in FP64 (relative error ~1e-7 in glam);
 *                      the adjoint state, dJ/dT_0 and J stay FP64.  Six FP64 operations per cell
 *                      and reverse step fewer. */
enum { NEBO_PRODUCTS_F64 = 0, NEBO_PRODUCTS_F32 = 1 };
/* OR'ed into `products`: the forward sweep in FP32 (storage and arithmetic of the states, their
 * checkpoints and the recomputed segments: half the checkpoint memory and HBM traffic of the
 * forward work), the adjoint state and every accumulation in FP64 on the widened FP32 states.
 * The gradient is that of the FP64 model evaluated along the FP32 trajectory; J comes from the
 * FP32 final state. */
enum { NEBO_FORWARD_F32 = 2 };
int nebo_heat_gradient_ex(const nebo_field* T0, const nebo_field* lam, const nebo_field* Ttarget,
                          int steps, double dt, int checkpoint_every, int products,
                          const nebo_field* gT0, const nebo_field* glam, double* J,
                          nebo_stream_t stream);
int nebo_heat_adjoint_step(const nebo_field* Tk, const nebo_field* Ain, const nebo_field* Aout,
                           const nebo_field* lam, const nebo_field* glam, double dt,
                           nebo_stream_t stream);
int nebo_heat_gradient(const nebo_field* T0, const nebo_field* lam, const nebo_field* Ttarget,
                       int steps, double dt, int checkpoint_every, const nebo_field* gT0,
                       const nebo_field* glam, double* J, nebo_stream_t stream);

/* Transposed stencil operator (reverse mode of a stencil assignment; no counterpart in the
 * reference).  For the forward assignment dst(i) = sum_k coefs[k] * src(i + p_k) over the write
 * region `limits` of dst ({xlo,xhi,ylo,yhi,zlo,zhi}, interior-relative, as nebo_write_limits
 * gives it) -- Interpolant, Gradient, Divergence, FD and box-filter stencils alike, their points
 * p_k (3 ints each, listed order) and coefficients as the operator defines them
 * (spatialops/NeboStencilBuilder.h:154-232, structured/stencil/StencilBuilder.cpp:52-220) --
 * every cell j of src_bar's window receives
 *     sum over the k with j - p_k in limits of coefs[k] * dst_bar(j - p_k)
 * (accumulate != 0: added to its value; else written, 0 where no point contributes).  FP64, up
 * to 32 points, deterministic (a gather in listed point order, no atomics). */
int nebo_stencil_transpose(const nebo_field* dst_bar, const int32_t limits[6], const nebo_field* src_bar,
                           int32_t npoints, const int32_t* points, const double* coefs, int accumulate,
                           nebo_stream_t stream);

/* ------------------------------------------------------------------ particle <-> cell operators
 * Replace Particle::CellToParticle<CellField>::apply_to_field and
 * Particle::ParticleToCell<CellField>::apply_to_field (spatialops/particles/ParticleOperators.h:
 * 313-398 and 186-273).  A particle is a cube of edge psize[p] centred at (px, py, pz)[p]; a null
 * coordinate array switches that axis off (the particle covers one cell along it, weight 1).
 * `mesh` holds the operator's state after its constructor (ParticleOperators.h:152-166 and 277-291): spacing
 * already with the "spacing <= 0 becomes 1, low 0" rule applied, and the cell field's ghost
 * cells on the - faces (GhostData::get_minus of get_ghost_data()).  Cell indices run over the
 * field's window including its ghost cells, as SpatialField::operator()(i,j,k) does.
 * Results equal the reference's serial loops bit for bit; boxes reaching outside the window are
 * clipped to it at both ends (the reference clips the high end; its low end is undefined).
 *   nebo_cell_to_particle  dest[p] = sum over the particle's cells of src(c) * weight, in the
 *                          reference's (k, j, i) order.  Asynchronous.
 *   nebo_particle_to_cell  every window cell of `cell` = sum over the particles that overlap it,
 *                          in particle order, of src[p] * weight (+0 where none does).  Reads a
 *                          64-bit overlap count back to size its entry list: synchronises the
 *                          stream once.  Deterministic: no floating-point atomics. */
typedef struct nebo_particle_mesh {
  double spacing[3];       /* dx_, dy_, dz_ (> 0) */
  double low[3];           /* xlo_, ylo_, zlo_: coordinate of the first interior cell's centre */
  int32_t ghost_minus[3];  /* the cell field's ghost cells on the - faces */
} nebo_particle_mesh;

int nebo_cell_to_particle(const nebo_particle_mesh* mesh, const double* px, const double* py, const double* pz,
                          const double* psize, int64_t nparticles, const nebo_field* cell, double* dest,
                          nebo_stream_t stream);
int nebo_particle_to_cell(const nebo_particle_mesh* mesh, const double* px, const double* py, const double* pz,
                          const double* psize, int64_t nparticles, const double* src, const nebo_field* cell,
                          nebo_stream_t stream);

/* ------------------------------------------------------------------ launch accounting
 * Every kernel launch of this library is counted; with profiling on, each launch (outside
 * graph capture) is also bracketed by CUDA events on its stream.  nebo_profile_report
 * synchronises those events and writes {"<kernel>": {"launches": n, "ms": total}, ...} as
 * JSON into buf (reset != 0 clears the totals).  Plays the part of NEBO_REPORT_BACKEND and
 * TimeLogger (spatialops/NeboLhs.h:321-392, util/TimeLogger.h:85-263). */
unsigned long long nebo_kernel_launch_count(void);
int nebo_profile_enable(int on);
int nebo_profile_report(char* buf, size_t len, int reset);

#ifdef __cplusplus
}
#endif
#endif /* NEBO_GB300_H */
