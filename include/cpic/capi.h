/* capi.h -- C ABI of the GB300 implementation of CabanaPIC's per-step hot path.
 *
 * Every entry point takes raw device pointers into the reference's own array
 * layouts (see layout.h), plain sizes and a CUDA stream.  Calls are
 * stream-ordered and asynchronous: none synchronises the host except
 * cpic_status_read().  The library allocates no device memory: where a kernel
 * needs scratch space, the caller passes it (see the *_scratch_bytes queries).
 *
 * Return codes: CPIC_OK (0); a negative CPIC_E* for a rejected argument or a
 * CUDA launch error.  Problems found on the device (a particle in a cell
 * outside the grid, a mover streak cap, a non-finite displacement) are OR-ed
 * into a caller-owned device status word, read back with cpic_status_read().
 *
 * Unlike the reference, which is a header-only template library with no error
 * reporting (push() is void, move_p's return is ignored, Reflect boundaries
 * call exit(1)), every entry point validates its arguments and returns a code.
 */
#ifndef CPIC_CAPI_H
#define CPIC_CAPI_H

#include <stddef.h>
#include <stdint.h>

#include "layout.h"

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without including the CUDA runtime headers */
typedef struct CUstream_st* cpic_stream_t;

/* ---------------------------------------------------------------- codes */
#define CPIC_OK 0
#define CPIC_EINVAL (-1)       /* null pointer, bad size or bad enum value */
#define CPIC_EUNSUPPORTED (-2) /* valid in the reference's types but not implemented
                                  there either (Reflect boundary, num_ghosts != 1) */
#define CPIC_ECUDA (-3)        /* a CUDA launch or copy returned an error */
#define CPIC_ESCRATCH (-4)     /* caller-provided scratch too small */

/* device status bits (cpic_status_read) */
#define CPIC_STATUS_CELL_RANGE 1  /* particle cell index outside [0, num_cells): skipped */
#define CPIC_STATUS_MOVER_CAP 2   /* move_p streak loop hit its iteration cap */
#define CPIC_STATUS_NONFINITE 4   /* non-finite displacement met in move_p */
#define CPIC_STATUS_PIPELINE 8    /* a bounded wait inside the tiled push kernel gave up
                                     (about a second); the push is incomplete */

/* Boundary, src/input/deck.h:9-12 */
#define CPIC_REFLECT 0
#define CPIC_PERIODIC 1

/* real_t selection: the byte size of real_t (src/types.h:4-8) */
#define CPIC_FLOAT 4
#define CPIC_DOUBLE 8

/* cpic_push_params.flags */
#define CPIC_PUSH_TRUE_SQRT 1  /* real_t=double only: use sqrt() for gamma where the
                                  reference calls sqrtf() (src/push.h:148,169) */
#define CPIC_PUSH_EXACT 2      /* the exact variant: every multiply and add rounded
                                  separately, IEEE division and sqrtf, so particle states
                                  are bit-identical to a CPU build of the reference without
                                  FMA contraction.  Default (0): fused multiply-adds and the
                                  hardware reciprocal square root, within 1e-5 relative. */
#define CPIC_PUSH_STREAMING 4  /* streaming kernel: per-particle global gathers, no
                                  shared-memory cell window.  Same results as the default
                                  tiled kernel, which is faster once particles are in cell
                                  order. */
#define CPIC_PUSH_ACC_F64 8    /* real_t = float only: `accumulators` holds double rows
                                  ([cell][3][4] of double, 96 B per cell).  Warps still
                                  reduce their deposits in float; the sum over warps, streaks
                                  and particles (the per-cell current sum, k terms at k
                                  particles per cell) runs in double, so its error no longer
                                  grows with k.  Unload with cpic_unload_accumulator_f64. */

#define CPIC_PUSH_ACC_LAYOUT_LEFT 16 /* `accumulators` in Kokkos' LayoutLeft, the default
                                  layout of accumulator_array_t = View<real_t*[3][4]> in a
                                  Kokkos-Cuda build (src/types.h:120): value (comp, q) of cell c
                                  at c + num_cells * (comp + 3 q), num_cells the grid's ghosted
                                  cell count (the extent example/example.cpp:137 allocates).
                                  Unload with cpic_unload_accumulator_left.  Not with
                                  CPIC_PUSH_ACC_F64. */

/* Grid of the run: interior cells nx*ny*nz plus num_ghosts ghost layers;
 * boundary is the deck's BOUNDARY_TYPE, which the reference's field code reads
 * from the global deck (src/fields.h:20,112). */
typedef struct cpic_grid {
  int64_t nx, ny, nz, num_ghosts;
  int32_t boundary;
  int32_t reserved;
} cpic_grid;

/* Scalar arguments of push() (src/push.h:7-23), in double; they are rounded to
 * real_t on entry, which is exact for values that were computed in real_t. */
typedef struct cpic_push_params {
  double qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp;
  int32_t precision;   /* CPIC_FLOAT or CPIC_DOUBLE */
  int32_t particle_vl; /* AoSoA vector length of the particle list: 16 or 32 */
  int32_t flags;       /* CPIC_PUSH_* */
  int32_t reserved;
} cpic_push_params;

/* ---------------------------------------------------------------- queries */
int cpic_version(void);
const char* cpic_strerror(int code);

/* ---------------------------------------------------------------- push
 * Replaces: template<class _accumulator> void push(particle_list_t& particles,
 *   interpolator_array_t& f0, real_t qdt_2mc, real_t cdt_dx, real_t cdt_dy,
 *   real_t cdt_dz, real_t qsp, _accumulator& a0, grid_t* g, size_t nx, ny, nz,
 *   num_ghosts, Boundary boundary)            -- src/push.h:7-300
 * together with the move_p it calls for cell-crossing particles
 *                                              -- src/move_p.h:9-374.
 * Gathers each particle's 18 interpolator coefficients, applies the Boris
 * push, moves the particle and scatter-adds its 12 current contributions (per
 * streak for crossers) into `accumulators`, in place.  Like the reference's
 * ScatterView, it ADDS to the accumulator: clear it first.  `d_status` is a
 * device int32 the caller owns; problems found are OR-ed into it. */
int cpic_push(void* particles, int64_t num_particles, const void* interpolators,
              void* accumulators, const cpic_grid* grid, const cpic_push_params* prm,
              int32_t* d_status, cpic_stream_t stream);

/* The same push out of place: particle p of `particles` (not modified) is
 * pushed into slot p of `out`, a distinct list of the same size, every member
 * written.  For callers that keep the state before the step (the adjoint's
 * segment recompute) without copying the list.  Tiled kernel only
 * (CPIC_PUSH_STREAMING: CPIC_EUNSUPPORTED). */
int cpic_push_into(const void* particles, void* out, int64_t num_particles, const void* interpolators,
                   void* accumulators, const cpic_grid* grid, const cpic_push_params* prm,
                   int32_t* d_status, cpic_stream_t stream);

/* ---------------------------------------------------------------- cells
 * Replaces: void load_interpolator_array(field_array_t fields,
 *   interpolator_array_t interpolators, size_t nx, ny, nz, ng)
 *                                              -- src/interpolator.h:14-21, interpolator.cpp:4-124 */
int cpic_load_interpolator(const void* fields, void* interpolators, const cpic_grid* grid,
                           int32_t precision, cpic_stream_t stream);

/* Replaces: void initialize_interpolator(interpolator_array_t& f0)
 *                                              -- src/interpolator.h:23, interpolator.cpp:125-172 */
int cpic_initialize_interpolator(void* interpolators, int64_t num_cells, int32_t precision,
                                 cpic_stream_t stream);

/* Replaces: void clear_accumulator_array(field_array_t& fields,
 *   accumulator_array_t& accumulators, size_t nx, ny, nz)
 *                                              -- src/accumulator.h:15-21, accumulator.cpp:5-43 */
int cpic_clear_accumulator(void* accumulators, int64_t num_cells, int32_t precision,
                           cpic_stream_t stream);

/* Replaces: void unload_accumulator_array(field_array_t& fields,
 *   accumulator_array_t& accumulators, size_t nx, ny, nz, ng, real_t dx, dy, dz, dt)
 *                                              -- src/accumulator.h:23-32, accumulator.cpp:45-122 */
int cpic_unload_accumulator(void* fields, const void* accumulators, const cpic_grid* grid,
                            double dx, double dy, double dz, double dt, int32_t precision,
                            cpic_stream_t stream);

/* Replaces: unload_accumulator_array (src/accumulator.cpp:45-122) for an
 * accumulator in Kokkos' LayoutLeft, the Kokkos-Cuda default of
 * src/types.h:120 (see CPIC_PUSH_ACC_LAYOUT_LEFT): the same sums in the same
 * order as cpic_unload_accumulator, so the same jf bits. */
int cpic_unload_accumulator_left(void* fields, const void* accumulators, const cpic_grid* grid,
                                 double dx, double dy, double dz, double dt, int32_t precision,
                                 cpic_stream_t stream);

/* unload_accumulator_array from the double accumulator rows of a push with
 * CPIC_PUSH_ACC_F64: the four-term sums and the scaling run in double, jf is
 * rounded once to the fields' real_t (precision). */
int cpic_unload_accumulator_f64(void* fields, const double* accumulators, const cpic_grid* grid,
                                double dx, double dy, double dz, double dt, int32_t precision,
                                cpic_stream_t stream);

/* Replaces: Field_Solver<EM_Field_Solver>::advance_b(field_array_t&, real_t px, py, pz,
 *   size_t nx, ny, nz, ng)                     -- src/fields.h:352-364, 668-719
 * (cB update over the interior, then the periodic ghost copy of cB). */
int cpic_advance_b(void* fields, double px, double py, double pz, const cpic_grid* grid,
                   int32_t precision, cpic_stream_t stream);

/* Replaces: Field_Solver<EM_Field_Solver>::advance_e(field_array_t&, real_t px, py, pz,
 *   size_t nx, ny, nz, ng, real_t dt_eps0)     -- src/fields.h:365-378, 618-665
 * (periodic fold of the jf ghosts, ghost copy of jf, then the E update). */
int cpic_advance_e(void* fields, double px, double py, double pz, const cpic_grid* grid,
                   double dt_eps0, int32_t precision, cpic_stream_t stream);

/* Replaces: EM_Field_Solver::e_energy and b_energy (src/fields.h:556-615), as
 * used by dump_energies (src/fields.h:722-763): writes {0.5*sum E^2,
 * 0.5*sum cB^2} over the interior, accumulated in double, to d_out[0..1]
 * (device memory).  The sum order is fixed (deterministic).  `d_scratch` must
 * hold cpic_energy_scratch_bytes() bytes of device memory; its contents on
 * entry do not matter. */
size_t cpic_energy_scratch_bytes(void);
int cpic_field_energies(const void* fields, const cpic_grid* grid, int32_t precision,
                        double* d_out, void* d_scratch, size_t scratch_bytes,
                        cpic_stream_t stream);

/* Energies without allocation -- no counterpart in the reference.  For
 * callers that cannot allocate device memory (device memory owned by their own
 * pool or arena, bindings with no CUDA allocator, per-step diagnostics that
 * must not allocate): the same result as cpic_field_energies, bit for bit, with
 * the scratch held in a static 9,480-byte device array inside this library
 * (592 block partial sums and a completion counter; every GPU that loads the
 * library keeps it until exit).  The scratch need does not grow with the grid;
 * grids beyond the library's limits (an axis above 2^20 cells, 2^31 ghosted
 * cells or more) return CPIC_EINVAL.  Every call looks up the array's device
 * address in the current device's context (so a context recreated after
 * cudaDeviceReset is served correctly); the first call on a device may load
 * the library's device code, so make that first call before any stream
 * capture.  All calls share the one array: calls that overlap on the GPU (concurrent
 * streams) race and must be serialised by the caller. */
int cpic_field_energies_noalloc(const void* fields, const cpic_grid* grid, int32_t precision,
                                double* d_out, cpic_stream_t stream);

/* Replaces: void uncenter_particles(particle_list_t particles,
 *   interpolator_array_t& f0, real_t qdt_2mc)          -- src/uncenter_p.h:4-105
 * The optional t = 0 back half-step of the momenta (example/example.cpp:204-213):
 * Boris rotation with -qdt_2mc/2, then the half E kick, in place.  `grid` is
 * used to check the particles' cell indices; a bad one sets
 * CPIC_STATUS_CELL_RANGE and leaves the particle unchanged. */
int cpic_uncenter_particles(void* particles, int64_t num_particles, const void* interpolators,
                            double qdt_2mc, const cpic_grid* grid, int32_t precision,
                            int32_t particle_vl, int32_t* d_status, cpic_stream_t stream);

/* Replaces: ES_Field_Solver_1D::advance_e (src/fields.h:511-544) with
 * fold_ghosts = 1 (the periodic jf fold, then E -= dt_eps0 * J) and
 * ES_Field_Solver::advance_e (src/fields.h:400-436) with fold_ghosts = 0; the
 * E update covers every cell of the array, ghosts included, as in the
 * reference.  (The ES solvers' advance_b is a no-op.) */
int cpic_es_advance_e(void* fields, const cpic_grid* grid, double dt_eps0, int32_t fold_ghosts,
                      int32_t precision, cpic_stream_t stream);

/* Replaces: ES e_energy (src/fields.h:438-463, 484-509): d_out[0] = 0.5 * sum
 * over every cell (ghosts included, as in the reference) of E^2, in double;
 * d_out[1] = 0.  Scratch as cpic_field_energies. */
int cpic_es_e_energy(const void* fields, const cpic_grid* grid, int32_t precision, double* d_out,
                     void* d_scratch, size_t scratch_bytes, cpic_stream_t stream);

/* ---------------------------------------------------------------- dumps */
/* Replaces the values printed by dump_particles (src/helpers.h:31-61):
 * d_out[2p] = xmin + (ix - 1 + (x_p + 1) * 0.5) * dx (computed in double,
 * stored as real_t), d_out[2p+1] = ux_p, for every particle p (2 * n real_t).
 * The caller copies d_out to the host (asynchronously) and prints each pair
 * as "%e  %e ", then one "\n". */
int cpic_particle_dump_values(const void* particles, int64_t num_particles, int32_t particle_vl,
                              const cpic_grid* grid, int32_t precision, double xmin, double dx,
                              void* d_out, cpic_stream_t stream);

/* Replaces the values printed by Field_Solver::dump_fields (src/fields.h:318-350):
 * d_out[2(i-1)] = xmin + (i - 0.5) * dx, d_out[2(i-1)+1] = ex of voxel (i,1,1),
 * i = 1..nx (2 * nx real_t); printed as "%e %e\n" per i, then "\n\n". */
int cpic_field_dump_values(const void* fields, const cpic_grid* grid, int32_t precision, double xmin,
                           double dx, void* d_out, cpic_stream_t stream);

/* ---------------------------------------------------------------- self-test
 * Self-test of the bounded device waits (no counterpart in the reference):
 * one warp waits on a shared-memory mbarrier phase that nothing completes,
 * with the tiled push's wait loop; after `limit_cycles` GPU cycles
 * (<= 2^31, the push's own limit) it gives up and OR-s
 * CPIC_STATUS_PIPELINE into `d_status`.  The device stays usable. */
int cpic_selftest_bounded_wait(int64_t limit_cycles, int32_t* d_status, cpic_stream_t stream);

/* ---------------------------------------------------------------- particle loading
 * Seeded uniform thermal plasma written on the device (no counterpart in the
 * reference, whose decks initialise particles on the host:
 * src/input/deck.h:79-158, decks/custom_init.cxx).  `ppc` particles per
 * interior cell, cells in VOXEL order with x fastest (particle p in interior
 * cell p / ppc); offsets uniform in [-1, 1); momenta Maxwellian with width
 * `uth` per component; every weight `weight`.  Particle p draws from the
 * counter-based generator Philox4x32-10 at counters (p, 0) and (p, 1) under
 * the key `seed`, so the list depends only on (seed, p).  Requires
 * num_particles <= ppc * nx * ny * nz. */
int cpic_thermal_particles(void* particles, int64_t num_particles, int32_t ppc, const cpic_grid* grid,
                           double uth, double weight, uint64_t seed, int32_t precision,
                           int32_t particle_vl, cpic_stream_t stream);

/* ---------------------------------------------------------------- sort
 * Counting sort of the particle list by cell index, in place.  The reference
 * leaves this step commented out (example/example.cpp:226-228, Cabana::sortByKey);
 * here it keeps the push's gathers and deposits local.  The order of particles
 * that share a cell is not specified.  `d_scratch` must hold
 * cpic_sort_scratch_bytes(...) bytes of device memory. */
size_t cpic_sort_scratch_bytes(int64_t num_particles, int64_t num_cells, int32_t precision,
                               int32_t particle_vl);
int cpic_sort_particles(void* particles, int64_t num_particles, int64_t num_cells,
                        int32_t precision, int32_t particle_vl, void* d_scratch,
                        size_t scratch_bytes, cpic_stream_t stream);

/* Out-of-place variant for callers that own two particle lists: the same
 * order, gathered from `particles` (unchanged) into `sorted` (distinct, same
 * size), without the in-place variant's copy of the list.  Scratch: the
 * counts and permutation only (cpic_sort_into_scratch_bytes). */
size_t cpic_sort_into_scratch_bytes(int64_t num_particles, int64_t num_cells, int32_t precision,
                                    int32_t particle_vl);
int cpic_sort_particles_into(const void* particles, void* sorted, int64_t num_particles,
                             int64_t num_cells, int32_t precision, int32_t particle_vl,
                             void* d_scratch, size_t scratch_bytes, cpic_stream_t stream);

/* Out-of-place sort on look-ahead keys: each particle is keyed by the interior
 * cell it reaches after `steps_ahead` free-streaming pushes at its current
 * momentum (displacement 2 u cdt_d / gamma per push, from prm's cdt_dx/dy/dz;
 * periodic wrap; a particle in a ghost cell keeps its cell as key).  Sorting
 * every S steps with steps_ahead = S/2 leaves the list in cell order midway
 * through the interval rather than at its start, so fewer of a warp's
 * particles sit outside its largest same-cell group, averaged over the
 * interval.  Any order is a valid particle list: the push's results do not
 * depend on it, only its speed.  prm supplies precision, particle_vl and the
 * cdt's (its other members are ignored); the grid must pass the push's grid
 * checks.  Scratch: cpic_sort_into_scratch_bytes(num_particles, cells of
 * grid, precision, particle_vl).  steps_ahead = 0 gives cell keys. */
int cpic_sort_particles_ahead_into(const void* particles, void* sorted, int64_t num_particles,
                                   const cpic_grid* grid, const cpic_push_params* prm,
                                   int32_t steps_ahead, void* d_scratch, size_t scratch_bytes,
                                   cpic_stream_t stream);

/* ---------------------------------------------------------------- diagnostics
 * FP64 diagnostics with no counterpart in the reference (its only diagnostic
 * is the field energy): what its scheme conserves, measured.
 *
 * cpic_charge_density overwrites d_rho (num_cells doubles, VOXEL-indexed
 * nodes; node (i,j,k) is the low corner of voxel (i,j,k)) with the charge
 * density of the particles: trilinear node weights (1 -/+ x)/2 (1 -/+ y)/2
 * (1 -/+ z)/2 of the cell offsets, times qsp * w / (dx dy dz), with the
 * periodic fold of the n+1 node layer into layer 1.  A particle whose cell
 * is outside the grid is skipped and sets bit 1 of *d_status. */
int cpic_charge_density(const void* particles, int64_t num_particles, const cpic_grid* grid,
                        int32_t precision, int32_t particle_vl, double qsp, double dx, double dy,
                        double dz, double* d_rho, int32_t* d_status, cpic_stream_t stream);

/* Discrete Gauss residual r = div E - rho/eps0 (- d_ref, if not null) at the
 * interior nodes, div E with backward differences of the edge fields
 * ((ex(i) - ex(i-1))/dx + ...; periodic images for index 0).  The push's
 * deposit and the Yee update keep r constant in time, so r(t) - r(0) measures
 * charge-conservation error.  d_out = {max |r|, sum r^2, sum (rho/eps0)^2};
 * d_resid (optional, num_cells doubles) receives r.  Deterministic. */
size_t cpic_diag_scratch_bytes(void);
int cpic_gauss_residual(const void* fields, const double* d_rho, const double* d_ref, double eps0,
                        double dx, double dy, double dz, const cpic_grid* grid, int32_t precision,
                        double* d_resid, double* d_out, void* d_scratch, size_t scratch_bytes,
                        cpic_stream_t stream);

/* Kinetic energy sum w * mc2 * (gamma - 1), gamma = sqrt(1 + u^2), in double
 * (gamma - 1 computed as u^2 / (1 + gamma)), into d_out[0].  Deterministic. */
int cpic_kinetic_energy(const void* particles, int64_t num_particles, int32_t precision,
                        int32_t particle_vl, double mc2, double* d_out, void* d_scratch,
                        size_t scratch_bytes, cpic_stream_t stream);

/* ---------------------------------------------------------------- adjoint
 * Reverse-mode (transposed) step kernels, no counterpart in the reference:
 * gradients of a loss on the state after K steps with respect to the initial
 * state.  Adjoint arrays use the forward layouts.  The field adjoints are the
 * transposed periodic stencils (the reference's ghost copies and jf fold make
 * the forward field maps periodic on the interior); ghost cells of adjoint
 * arrays are unused.
 *
 * cpic_adjoint_push: given the particles at the START of the step, the
 * step's interpolator, the adjoint accumulator array and, in
 * lambda_particles, the adjoint of (offsets, momenta) after the step,
 * overwrites lambda_particles with the adjoint before the step and adds the
 * adjoint of the gathered coefficients into lambda_interp (transpose of the
 * gather; the transpose of the deposit is a gather from lambda_acc).  Cell
 * indices are piecewise constant; weights are not differentiated. */
int cpic_adjoint_push(const void* particles, int64_t num_particles, const void* interpolators,
                      const void* lambda_acc, void* lambda_particles, void* lambda_interp,
                      const cpic_grid* grid, const cpic_push_params* prm, int32_t* d_status,
                      cpic_stream_t stream);

/* lambda_E -= Mb^T lambda_B: transpose of advance_b's cB update
 * (src/fields.h:668-719), same (px, py, pz). */
int cpic_adjoint_advance_b(void* d_lambda_fields, double px, double py, double pz,
                           const cpic_grid* grid, int32_t precision, cpic_stream_t stream);

/* lambda_B += Me^T lambda_E and lambda_J = -dt_eps0 lambda_E: transpose of
 * advance_e (src/fields.h:618-665), lambda_J in the jf members. */
int cpic_adjoint_advance_e(void* d_lambda_fields, double px, double py, double pz,
                           const cpic_grid* grid, double dt_eps0, int32_t precision,
                           cpic_stream_t stream);

/* lambda_acc = unload^T lambda_J: transpose of unload_accumulator_array with
 * its periodic fold (src/accumulator.cpp:45-122, src/fields.h:102-271).
 * d_lambda_acc ([cell][3][4], like the accumulator) must be 16-byte aligned. */
int cpic_adjoint_unload_accumulator(const void* d_lambda_fields, void* d_lambda_acc,
                                    const cpic_grid* grid, double dx, double dy, double dz,
                                    double dt, int32_t precision, cpic_stream_t stream);

/* lambda_(E, cB) += interp^T lambda_I: transpose of load_interpolator_array
 * (src/interpolator.cpp:4-124). */
int cpic_adjoint_load_interpolator(const void* d_lambda_interp, void* d_lambda_fields,
                                   const cpic_grid* grid, int32_t precision, cpic_stream_t stream);

/* The interpolator adjoint in cell-major rows (no counterpart in the
 * reference): cpic_adjoint_push with CPIC_ADJ_INTERP_ROWS in prm->flags adds
 * the adjoint of cell c's 18 coefficients (interpolator member order) into
 * values [c * CPIC_ADJ_INTERP_ROW, c * CPIC_ADJ_INTERP_ROW + 18) of
 * lambda_interp (num_cells rows, 16-byte aligned), instead of the
 * interpolator's AoSoA layout: a particle's 18 adjoints then land in one or
 * two 128-byte lines as vector reductions, where the AoSoA layout spreads them
 * over 18 lines.  cpic_adjoint_load_interpolator_rows is the transpose of the
 * interpolator load reading that layout; together they give the AoSoA pair's
 * result, summed in another order. */
#define CPIC_ADJ_INTERP_ROW 20
#define CPIC_ADJ_INTERP_ROWS 32
int cpic_adjoint_load_interpolator_rows(const void* d_lambda_interp_rows, void* d_lambda_fields,
                                        const cpic_grid* grid, int32_t precision, cpic_stream_t stream);

/* ---------------------------------------------------------------- status */
/* Clears the device status word (stream-ordered). */
int cpic_status_clear(int32_t* d_status, cpic_stream_t stream);
/* Synchronises `stream` and copies the status word to *h_status. */
int cpic_status_read(const int32_t* d_status, cpic_stream_t stream, int32_t* h_status);

#ifdef __cplusplus
}
#endif

#endif /* CPIC_CAPI_H */
