/*
 * igsolve.h -- C-ABI of libigsolve.so, the GB300 (sm_103a) implementation of
 * ion_gym's 3-D finite-difference Laplace field solve.
 *
 * Every solver entry point takes arrays in C order (nx, ny, nz), z
 * contiguous, is synchronous, and returns an int status (IG_OK or one of the
 * codes below).  ig_solve3d, ig_solve3d_mg and ig_cascadic_relres accept
 * host (pageable or pinned) or device pointers alike (the copies resolve the
 * direction by unified addressing); the V-cycle and basis entry points read
 * their masks on the host and need host arrays.  A failing call leaves a message for ig_last_error() (per
 * calling thread).  Masks are uint8 (0 / 1); potentials float64; theta, when
 * given, float32 (6, nx, ny, nz) in the order (-x, +x, -y, +y, -z, +z);
 * theta == NULL is the reference's theta=None.  stencil: 0 = "ghost_linear",
 * 1 = "sw".  The calling thread's current CUDA device runs the solve.
 *
 * The FP64 entry points return the reference's bits: the same sweep counts,
 * the same final delta and the same potential, node for node.
 *
 * Functions ending in _dev take DEVICE pointers and a cudaStream_t (as
 * void*, NULL = the legacy default stream); they enqueue on that stream and,
 * when they return a max, synchronize it.
 */
#ifndef IGSOLVE_H
#define IGSOLVE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
enum {
  IG_OK = 0,
  IG_NOT_CONVERGED = 1, /* SOR sweep cap (solver3d.py:287-293)               */
  IG_STAGNATED = 2,     /* V-cycle stagnation (multigrid3d.py:708-724)       */
  IG_CYCLE_CAP = 3,     /* V-cycle max_cycles (multigrid3d.py:726-731)       */
  IG_INTERRUPTED = 4,   /* stop requested (multigrid3d.py:255-260, 655, 669) */
  IG_BAD_ARG = 5,       /* invalid shape, stencil or pointer                 */
  IG_CUDA_ERROR = 6,    /* a CUDA call failed; see ig_last_error()           */
  IG_NO_DEVICE = 7      /* no CUDA device is visible                         */
};

/* Message of the last failing call on this thread ("" if none). */
const char *ig_last_error(void);
/* ABI version of this header (2: ig_mixed_open_ex takes gamma_levels). */
int ig_abi_version(void);
/* Number of visible CUDA devices (0 without a GPU; never fails). */
int ig_device_count(void);
/* Free bytes of the calling thread's current device (0 without a GPU; no
 * reference counterpart: sizes concurrent basis solves). */
long long ig_device_free_bytes(void);

/* ---- cooperative stop (multigrid3d.py:42, 61-79) ----------------------
 * Replaces the threading.Event _STOP: request_stop() / clear_stop() set and
 * clear it; the V-cycle polls it twice per cycle and the basis loop between
 * bases, exactly where the reference polls _STOP. */
void ig_request_stop(void);
void ig_clear_stop(void);
int ig_stop_requested(void);

/* ---- solvers (host arrays, synchronous) -------------------------------- */

/* solver3d.solve3d (solver3d.py:250-293): red-black SOR until the max
 * |update| of a sweep pair is < tol, at most max_sweeps pairs.
 * omega: the SOR factor (the caller passes optimal_omega(shape) for None).
 * phi0: NULL for a zero start.  Out: phi (n), sweep pairs, final delta.
 * IG_NOT_CONVERGED at the cap, with the last pair's delta. */
int ig_solve3d(const uint8_t *fixed, const double *val, const float *theta,
               long nx, long ny, long nz, double tol, long max_sweeps,
               double omega, const double *phi0, int stencil, double *phi_out,
               long *sweeps_out, double *delta_out);

/* multigrid3d.solve3d_mg (multigrid3d.py:175-230), cascadic multigrid:
 * levels by _coarsen_mask while min(shape) > min_coarse and the next level
 * keeps every axis >= 3 (at most max_levels), coarsest solved to tol,
 * intermediates to tol * level_tol_factor from the prolongated guess, fine
 * level to tol with theta.  level_omega[L] is the SOR factor of level L
 * (0 = fine); n_level_omega must be at least the number of levels.
 * Out: fine phi, fine sweep pairs, fine delta. */
int ig_solve3d_mg(const uint8_t *fixed, const double *val, const float *theta,
                  long nx, long ny, long nz, double tol, long max_sweeps,
                  int stencil, int min_coarse, int max_levels,
                  double level_tol_factor, const double *level_omega,
                  int n_level_omega, double *phi_out, long *sweeps_out,
                  double *delta_out);

/* multigrid3d.solve3d_vmg (multigrid3d.py:602-731), V-cycle multigrid with
 * the recursive error-equation solve of _solve_err (multigrid3d.py:553-599).
 * bottom_omega: optimal_omega() of the bottom error level's shape (<= 0:
 * computed here with libm).  Out: phi, fine sweep pairs, final cycle delta,
 * cycles run, and the previous cycle's delta (for the stagnation message).
 * IG_STAGNATED / IG_CYCLE_CAP / IG_INTERRUPTED as the reference raises;
 * accept_stagnation != 0 returns IG_OK with the stalled iterate. */
int ig_solve3d_vmg(const uint8_t *fixed, const double *val, const float *theta,
                   long nx, long ny, long nz, double tol, int max_cycles,
                   int nu1, int nu2, int stencil, const double *phi0,
                   int accept_stagnation, double bottom_omega, double *phi_out,
                   long *sweeps_out, double *delta_out, int *cycles_out,
                   double *prev_delta_out);

/* One basis of multigrid3d.solve_bases_mg (multigrid3d.py:265-269): the
 * V-cycle on the metal union with val = v_basis on `mask` and 0 elsewhere,
 * built on the device from the mask.  Same outputs and statuses as
 * ig_solve3d_vmg. */
int ig_solve_basis_vmg(const uint8_t *metal, const uint8_t *mask,
                       double v_basis, const float *theta, long nx, long ny,
                       long nz, double tol, int max_cycles, int nu1, int nu2,
                       int stencil, double bottom_omega, double *phi_out,
                       long *sweeps_out, double *delta_out, int *cycles_out,
                       double *prev_delta_out);

/* One basis of solver3d.solve_bases (solver3d.py:308-319): SOR on the metal
 * union with val = v_basis on `mask`.  Same outputs as ig_solve3d. */
int ig_solve_basis_sor(const uint8_t *metal, const uint8_t *mask,
                       double v_basis, const float *theta, long nx, long ny,
                       long nz, double tol, long max_sweeps, double omega,
                       int stencil, double *phi_out, long *sweeps_out,
                       double *delta_out);

/* Cascadic multigrid with a residual stopping rule (no reference
 * counterpart; the quadrupole benchmark's rule): the same level hierarchy as
 * ig_solve3d_mg, each level relaxed with red-black SOR at level_omega[L],
 * the relative residual max|r| / max|r(phi_D)| (r: multigrid3d._residual,
 * phi_D: the Dirichlet values, zero elsewhere) checked every check_every
 * pairs; the coarsest and fine levels stop below rel_tol, intermediates
 * below rel_tol * level_tol_factor.  Out: fine phi, fine pairs, fine
 * relative residual, total pairs on all levels, and (levels_out) the level
 * count. */
int ig_cascadic_relres(const uint8_t *fixed, const double *val, long nx,
                       long ny, long nz, double rel_tol, long max_sweeps,
                       int min_coarse, int max_levels, double level_tol_factor,
                       const double *level_omega, int n_level_omega,
                       int check_every, double *phi_out, long *sweeps_out,
                       double *relres_out, long *total_pairs_out,
                       int *levels_out);

/* Mixed-precision batched basis solve (the reference's solve_bases_mg
 * problem, multigrid3d.py:233-291, with a different method and stopping
 * rule): n_bases unit bases on the metal union `metal`, basis b at v_basis
 * on masks[b] (n_bases stacked (nx,ny,nz) uint8 masks) and 0 on the rest of
 * the metal.  Flexible conjugate gradients on the FP32 correction,
 * preconditioned by one FP32 red-black multigrid V-cycle (nu1/nu2
 * Gauss-Seidel pairs), refine the potential, held in 64-bit fixed point
 * (units of 2^-56 of the largest Dirichlet magnitude, |values| in
 * [2^-61, 2^60), else IG_BAD_ARG) and returned as float64 with the Dirichlet
 * values exact at the metal; its residual is the reference's fine operator
 * with theta None, an exact integer sum; a basis is
 * done when the geometric tail d * rho / (1 - rho) of its last refinement
 * step d is below `acc` (absolute, volts), rho being 3 x the larger of the
 * last two observed step ratios.  Out: phi (n_bases x n float64), refinement steps, and
 * each basis's last step.  IG_NOT_CONVERGED after max_steps. */
int ig_mixed_bases(const uint8_t *metal, const uint8_t *masks, int n_bases,
                   double v_basis, long nx, long ny, long nz, int stencil,
                   double acc, int max_steps, int nu1, int nu2, int vcycles,
                   double *phi_out, int *steps_out, double *dmax_out);

/* Resident mixed-precision sessions (no reference counterpart): one
 * geometry's multigrid hierarchy, potentials and captured CUDA graphs stay
 * on the device between solves, on the session's own stream, so sessions of
 * different geometries run concurrently.  ig_mixed_bytes: the device bytes a
 * session for up to max_problems problems holds (admission by HBM
 * footprint).  ig_mixed_solve_bases: as ig_mixed_bases on the session's
 * metal.  ig_mixed_solve_values: n_problems Dirichlet problems on the
 * session's metal, problem p with the values vals[p] (float64 (n) each) at
 * the metal nodes.  Arrays may be host or device memory. */
long ig_mixed_bytes(long nx, long ny, long nz, int max_problems);
/* Kernel launches the mixed path has issued (graph replays counted node by
 * node) since the library was loaded. */
long ig_mixed_launch_count(void);
int ig_mixed_open(const uint8_t *metal, long nx, long ny, long nz,
                  int max_problems, int stencil, int nu1, int nu2, int vcycles,
                  void **handle);
/* ig_mixed_open with the method and cycle shape.  method 1 (default of
 * ig_mixed_open): flexible conjugate gradients on the FP32 correction,
 * preconditioned by one multigrid cycle, cg_iters iterations per FP64
 * refinement (the correction is then added to the FP64 potential and the
 * carried residual replaced by the exact FP64 one); method 0: plain defect
 * correction with `vcycles` cycles per refinement.  gamma 1 = V-cycle,
 * 2 = W-cycle (coarse levels cycled twice per visit); gamma_levels: the
 * second visit only from the finest gamma_levels levels (1: a W-cycle at
 * the top level, V below; <= 0: every level); smooth_omega: the
 * relaxation factor of the red-black smoother (1 = Gauss-Seidel). */
int ig_mixed_open_ex(const uint8_t *metal, long nx, long ny, long nz,
                     int max_problems, int stencil, int nu1, int nu2,
                     int vcycles, int gamma, int gamma_levels,
                     double smooth_omega, int method, int cg_iters,
                     void **handle);
/* A session with one metal per problem (no reference counterpart): the
 * n_problems stacked (nx, ny, nz) uint8 masks in `metals`, problem p
 * solved on metal p by ig_mixed_solve_values (problems 0..P-1 of a call on
 * metals 0..P-1), so decks of one grid shape with different electrodes run
 * as one batch: every launch of a refinement step covers all of them.
 * ig_mixed_rebind then takes n_problems stacked masks; ig_mixed_solve_bases
 * is refused (IG_BAD_ARG).  ig_mixed_bytes_multi: its device bytes. */
int ig_mixed_open_multi(const uint8_t *metals, int n_problems, long nx, long ny,
                        long nz, int stencil, int nu1, int nu2, int vcycles,
                        int gamma, int gamma_levels, double smooth_omega,
                        int method, int cg_iters, void **handle);
long ig_mixed_bytes_multi(long nx, long ny, long nz, int n_problems);
int ig_mixed_solve_bases(void *handle, const uint8_t *masks, int n_bases,
                         double v_basis, double acc, int max_steps,
                         double *phi_out, int *steps_out, double *dmax_out);
/* ig_mixed_solve_bases returning the unit bases the field cache stores
 * (replaces the host-side (phi / V_BASIS).astype(float32) of
 * physics/build_stl3d.py:849 after the basis door): unit_out receives
 * n_bases float32 arrays, each RN32(phi / v_basis) of the float64
 * potential ig_mixed_solve_bases returns -- the same two roundings, so the
 * same bits -- formed on the device, so half the bytes come back.  v_basis
 * must be finite and nonzero. */
int ig_mixed_solve_unit_bases(void *handle, const uint8_t *masks, int n_bases,
                              double v_basis, double acc, int max_steps,
                              float *unit_out, int *steps_out,
                              double *dmax_out);
int ig_mixed_solve_values(void *handle, const double *vals, int n_problems,
                          double acc, int max_steps, double *phi_out,
                          int *steps_out, double *dmax_out);
/* ig_mixed_solve_values with one absolute accuracy per problem (acc[p]
 * volts for problem p; no reference counterpart). */
int ig_mixed_solve_values_acc(void *handle, const double *vals, int n_problems,
                              const double *acc, int max_steps, double *phi_out,
                              int *steps_out, double *dmax_out);
void ig_mixed_close(void *handle);
/* Changes a session's cycle (no reference counterpart): nu1 / nu2
 * smoothing pairs before / after the coarse correction and the flexible
 * CG's iterations per refinement step; the captured graphs are dropped and
 * recaptured at the next solve, the buffers kept.  The accuracy contract
 * of the solves is unchanged (their bits follow the cycle). */
int ig_mixed_set_cycle(void *handle, int nu1, int nu2, int cg_iters);
/* Gives a session another geometry of its shape (no reference
 * counterpart): the new metal union's masks replace the old ones on every
 * level; the buffers, the tuned smoother shape and the captured graphs stay,
 * so a solve on the rebound session costs no session build.  The results
 * are those of a session opened on the new metal.  IG_BAD_ARG when the
 * shape differs.  A session with one metal per problem takes its
 * n_problems masks stacked. */
int ig_mixed_rebind(void *handle, const uint8_t *metal, long nx, long ny,
                    long nz);
/* Times `pairs` red-black pairs of the session's fine-level FP32
 * Gauss-Seidel kernel for n_problems problems with CUDA events on the
 * session's stream: the average launch (one colour) and its algorithmic
 * bytes (6.5 B per node and problem). */
int ig_mixed_time_gs(void *handle, int n_problems, int pairs,
                     double *ms_per_launch, double *bytes_per_launch);
/* The smoother shape the session's tuner chose for n_problems problems
 * (tuning first if it has not run): float4 groups per thread and block
 * size of the separate half-sweeps; tb[0] = the temporal-block depth taken
 * for the finest level (half-sweeps per blocked pass; 0 = separate
 * launches), tb[1] = the fastest blocked depth timed (0 = none timed:
 * IG_MIXED_TB_LEVELS set, a size-1 axis or a single level); us[0] and
 * us[1] = their measured microseconds per half-sweep.  No reference
 * counterpart (a measurement aid). */
int ig_mixed_tuning(void *handle, int n_problems, int *ng, int *threads,
                    int tb[2], double us[2]);
/* Algorithmic DRAM bytes of one refinement step of the session for
 * n_problems problems: every kernel's inputs read once and outputs written
 * once, summed over the captured step (all levels).  A step's time over
 * this gives the whole step's achieved bandwidth.  No reference
 * counterpart (a measurement aid). */
int ig_mixed_step_bytes(void *handle, int n_problems, double *bytes_out);
/* The algorithmic bytes of every refinement step of the session's last
 * solve (ig_mixed_step_bytes times its steps).  No reference counterpart
 * (a measurement aid). */
int ig_mixed_solve_bytes(void *handle, double *bytes_out);
/* Checks the integer-pipe float -> int64 conversion (round to nearest
 * even) that the mixed path's update uses to add a correction to the
 * fixed-point potential against the GPU's own conversion instruction, bit
 * for bit, on n host values (copied to the device): *mismatches = the
 * number of values whose results differ, 0 when all agree.  No reference
 * counterpart (a self-check of this library). */
int ig_mixed_check_convert(const float *floats, long n, long long *mismatches);
/* Checks the fused kernels of the mixed path against the separate launches
 * they replace, on the state the session's last solve left (right-hand
 * sides, corrections, direction): mismatches[0] = the first Gauss-Seidel
 * pair from a zero correction vs a zeroed correction and two half-sweeps,
 * [1] = the float4 colour-0 residual vs the per-slot one, [2] = the
 * windowed prolongation vs the per-node gather, [3] = the direction update
 * fused into the operator apply vs the two kernels (direction, L p and the
 * block partials of the inner products), [4] = the four-node restriction
 * of the colour-0 residual vs the per-node one, [5] = the CG update of a
 * refinement step's first iteration (x = alpha p) vs a zeroed x and the
 * update, and the last iteration's x += alpha p folded into the FP64
 * update vs the two kernels (potentials and step maxima), [6] = the
 * temporally blocked pre-smoothing (1, 2 and 3 Gauss-Seidel pairs from a
 * zero correction in one pass) vs a zeroed correction and the separate
 * half-sweeps, [7] = the blocked post-smoothing (colours 1, 0, ... into a
 * second array) vs the separate half-sweeps on the same input -- each the
 * number of 32-bit words that differ over every multigrid level, 0 when
 * bit-identical.  Flexible-CG sessions only; no reference counterpart (a
 * self-check of this library's kernel fusion). */
int ig_mixed_check_fused(void *handle, int n_problems,
                         long long mismatches[8]);

/* ig_cascadic_relres for callers that cannot allocate device memory (no
 * counterpart in the reference).  Some callers may not call cudaMalloc, or
 * let a library call it for them, while they run: a serving process that
 * reserved its HBM up front and lends the solver only its own buffers, a
 * framework custom call that must not allocate outside its allocator, a
 * latency-bound loop where an allocation could stall on the driver.  This
 * entry point allocates nothing: fixed, val and phi_out are DEVICE arrays,
 * the solve iterates in phi_out, and the coarse levels live in one static
 * device array of IG_NOALLOC_SCRATCH_BYTES that every GPU loading the
 * library holds until exit.  A grid whose coarse levels (about 2.4 bytes per
 * fine node) do not fit is refused with IG_BAD_ARG.  All calls share that
 * array and it keeps the last call's contents: calls that overlap on the GPU
 * race, so serialise them.  Every call looks up the array's address on the
 * current device (no allocation), so a device reset between calls is safe.
 * The solve synchronises `stream` at every residual check.  stream: the
 * caller's cudaStream_t (NULL = legacy default stream).  Same results, bit
 * for bit, as ig_cascadic_relres. */
#define IG_NOALLOC_SCRATCH_BYTES (48u * 1024u * 1024u)
int ig_cascadic_relres_noalloc(const uint8_t *fixed, const double *val,
                               long nx, long ny, long nz, double rel_tol,
                               long max_sweeps, int min_coarse,
                               int max_levels, double level_tol_factor,
                               const double *level_omega, int n_level_omega,
                               int check_every, double *phi_out,
                               long *sweeps_out, double *relres_out,
                               long *total_pairs_out, int *levels_out,
                               void *stream);

/* ---- analytic scenes (physics/rasterize3d.py, physics/solver3d.py) ------
 * A scene is a primitive table in grid units, 16 doubles per row: kind
 * (0 z-cylinder, 1 box), electrode slot (rows in slot order), shape id,
 * role (0 within, 1 notin), six bounds with +1e-9 (inclusive) and six with
 * -1e-9 (strict): cylinder cx, cy, r^2+e, (z-length)-e, z+e, 0; box x1-e,
 * x2+e, y1-e, y2+e, z1-e, z2+e.
 * ig_rasterize (rasterize3d.py:45-109): int16 labels (electrode_index[slot]
 * inside, 0 vacuum), per slot the node count, the count of nodes it claims
 * from an earlier electrode and the lowest such flat index.
 * ig_theta_scene (solver3d.py:75-127): theta (6, nx, ny, nz) float32 of
 * every vacuum node whose neighbour along a direction is metal, by `iters`
 * bisections of the exact inside test; mirror_bits: bit a set = low mirror
 * plane on axis a. */
int ig_rasterize(const double *table, int n_prims, const int *electrode_index,
                 int n_electrodes, long nx, long ny, long nz,
                 int16_t *labels_out, unsigned long long *counts_out,
                 unsigned long long *clash_counts_out,
                 unsigned long long *clash_first_out);
int ig_theta_scene(const double *table, int n_prims, const uint8_t *metal,
                   long nx, long ny, long nz, int mirror_bits, int iters,
                   float *theta_out);

/* ---- extruded 2-D shapes (build_shapes3d.py:71-243, raster2d.py:113-230)
 * ig_shape_xsection: one shape's cross-section on in-plane node
 * coordinates a (na) x b (nb) -> out (na, nb) uint8, float64 throughout.
 * type 0 rect, params = cx, cy, cos, sin (of -rotation), x0-T, x0+w+T,
 * y0-T, y0+h+T, rotated (0/1); type 1 ellipse, params = cx, cy, rx+T, ry+T;
 * type 2 polygon (closed solid: even-odd interior or within sqrt(tol2) of
 * an edge), params = tol2, poly = 7 rows of n_points: x0, y0, x1, y1,
 * ex, ey, seg2 (edge j from point j to j+1, wrapping).
 * ig_shapes_label: the 3-D assembly.  table: 7 long longs per shape, in
 * electrode order: electrode slot, extrusion axis (0..2; in-plane axes
 * the next two cyclically), cutout (0/1), offset of its cross-section in
 * xs (n_a1 x n_a2 bytes), offset of its range in rng (one byte per node
 * of the axis), n_a1, n_a2.  Per node: additive shapes OR their volume
 * into the electrode, cutouts AND NOT theirs; labels_out = the last
 * electrode (electrode_index[slot]) claiming the node, 0 vacuum; per slot
 * the node count, the count of nodes already claimed by an earlier
 * electrode and the lowest such flat index. */
int ig_shape_xsection(int type, const double *params, int n_params,
                      const double *poly, int n_points, const double *a,
                      long na, const double *b, long nb, uint8_t *out);
int ig_shapes_label(const long long *table, int n_shapes, const uint8_t *xs,
                    long long xs_len, const uint8_t *rng, long long rng_len,
                    const int *electrode_index, int n_electrodes, long nx,
                    long ny, long nz, int16_t *labels_out,
                    unsigned long long *counts_out,
                    unsigned long long *clash_counts_out,
                    unsigned long long *clash_first_out);

/* ---- fields from solved bases ------------------------------------------ *
 * Unit bases, drive superposition and the electrode-aware E-field, the same
 * bits as the reference.
 * ig_unit_bases_dev (build_stl3d.py:849): out = float32(phi / v_basis),
 * float64 division rounded to float32.
 * ig_superpose_dev / the first half of ig_compose_fields (build_stl3d.py:
 * 547-568): a plan of n_steps steps in electrode order; step s reads the
 * device basis basis_ptrs[s] (a host array of n_steps device pointers; in
 * ig_compose_fields, row rows[s] of the host stack); channel c starts at +0
 * and adds mult[c*n_steps+s] times float32(weights[c*n_steps+s] * basis),
 * float32 round to nearest, no fused multiply-add.  The static drive A is a
 * channel with weights float32(dc_i) (mult 0 where dc_i is 0); a drive
 * group is a channel with weight 1 and mult = how often the electrode names
 * the group.  Launches of IG_FIELD_MAX_CHANNELS channels by
 * IG_FIELD_MAX_STEPS steps; longer plans continue the float32 sums.
 * ig_field_aware_3d / ig_field_aware_dev (tracer3d.py:55-117): E = -grad
 * phi on the node grid, numpy.gradient (central inside, first order at the
 * faces) and, where metal is given, the one-sided difference into the
 * vacuum at metal nodes with vacuum on exactly one side along an axis.
 * dtype 0: float32 potential and fields, 1: float64.  h_is_f64 = 0 when the
 * reference's spacing is a Python float (float32 potentials then divide in
 * float32 by float32(2h) and float32(h)), 1 when it is a numpy float64
 * (float64 division, rounded).  The metal rule divides in float64.  Every
 * axis needs at least 2 nodes.  The _dev form does n_channels potentials
 * phi_stride elements apart into fields out_stride apart.
 * ig_compose_fields: host buffers; bases (n_bases, nx, ny, nz) float32 ->
 * per channel its potential phi_out and ex/ey/ez_out (n_channels, nx, ny,
 * nz) float32. */
#define IG_FIELD_MAX_STEPS 64
#define IG_FIELD_MAX_CHANNELS 8
int ig_unit_bases_dev(const double *phi, long long n, double v_basis,
                      float *out, void *stream);
int ig_superpose_dev(const float *const *basis_ptrs, int n_steps,
                     int n_channels, const float *weights,
                     const uint8_t *mult, long long n, float *out,
                     long long out_stride, void *stream);
int ig_field_aware_dev(const void *phi, int dtype, long long phi_stride,
                       int n_channels, const uint8_t *metal, long nx, long ny,
                       long nz, double h, int h_is_f64, void *ex, void *ey,
                       void *ez, long long out_stride, void *stream);
int ig_field_aware_3d(const void *phi, int dtype, const uint8_t *metal,
                      long nx, long ny, long nz, double h, int h_is_f64,
                      void *ex, void *ey, void *ez);
/* Self-check (no reference counterpart): the field kernels divide without
 * the hardware division on their fast path (an FMA-corrected float32
 * quotient; a float32 emulation of the float64 quotient with an exact
 * fallback).  Compares them with the IEEE divisions for the spacing h:
 * every float32 numerator over float32(h) and float32(2h), and `samples`
 * hashed numerators over the float64 h and 2h.  *mismatches_out = the
 * number of differing results (0 expected). */
int ig_field_check_division(double h, unsigned long long samples,
                            unsigned seed, unsigned long long *mismatches_out);
int ig_compose_fields(const float *bases, int n_bases, int n_steps,
                      const int *rows, int n_channels, const float *weights,
                      const uint8_t *mult, const uint8_t *metal, long nx,
                      long ny, long nz, double h, int h_is_f64,
                      float *phi_out, float *ex_out, float *ey_out,
                      float *ez_out);

/* ---- single kernels on device arrays ----------------------------------- */

/* solver3d._sweep (solver3d.py:131-198); theta NULL = all ones.  The max
 * |update| goes to *dmax_out (host), after a stream synchronize. */
int ig_sweep_dev(double *phi, const uint8_t *fixed, const float *theta,
                 long nx, long ny, long nz, double omega, int colour,
                 int stencil, double *dmax_out, void *stream);
/* multigrid3d._residual (multigrid3d.py:305-354). */
int ig_residual_dev(const double *phi, const uint8_t *fixed,
                    const float *theta, long nx, long ny, long nz, int stencil,
                    double *out, void *stream);
/* multigrid3d._sweep_rhs (multigrid3d.py:357-391). */
int ig_sweep_rhs_dev(double *e, const uint8_t *fixed, const double *f,
                     long nx, long ny, long nz, double omega, int colour,
                     double *dmax_out, void *stream);
/* multigrid3d._residual_rhs (multigrid3d.py:394-417). */
int ig_residual_rhs_dev(const double *e, const uint8_t *fixed, const double *f,
                        long nx, long ny, long nz, double *out, void *stream);
/* multigrid3d._restrict_fw_njit (multigrid3d.py:420-455): out has the
 * ((n+1)/2) coarse shape. */
int ig_restrict_fw_dev(const double *fine, long nx, long ny, long nz,
                       double *out, void *stream);
/* multigrid3d._prolong_add_njit (multigrid3d.py:458-499). */
int ig_prolong_add_dev(const double *coarse, long cx, long cy, long cz,
                       double *out, const uint8_t *fixed, long nx, long ny,
                       long nz, void *stream);
/* multigrid3d._prolongate (multigrid3d.py:138-171). */
int ig_prolongate_dev(const double *coarse, long cx, long cy, long cz,
                      double *out, long nx, long ny, long nz, void *stream);
/* multigrid3d._coarsen_fixed_any (multigrid3d.py:507-526). */
int ig_coarsen_fixed_any_dev(const uint8_t *fixed, long nx, long ny, long nz,
                             uint8_t *out, void *stream);
/* multigrid3d._coarsen_mask (multigrid3d.py:85-135). */
int ig_coarsen_mask_dev(const uint8_t *fixed, const double *val, long nx,
                        long ny, long nz, uint8_t *fc, double *vc,
                        void *stream);
/* solver3d._residual_kernel (solver3d.py:366-386); every axis >= 2. */
int ig_residual_audit_dev(const double *u, const uint8_t *fixed,
                          const float *theta, long nx, long ny, long nz,
                          double *out, void *stream);
/* solver3d._err_sweep (solver3d.py:389-417); every axis >= 2. */
int ig_err_sweep_dev(double *e, const uint8_t *fixed, const float *theta,
                     const double *rhs, long nx, long ny, long nz,
                     double omega, int colour, double *dmax_out, void *stream);

/* ---- profiling of the timed sweep launches ----------------------------
 * When enabled, the SOR loops bracket each batch of sweep launches with CUDA
 * events on their own stream and accumulate the time and the number of
 * launches that did work. */
void ig_prof_enable(int on);
void ig_prof_reset(void);
void ig_prof_read(double *sweep_ms, long *sweep_launches, long *sweep_nodes);
/* Kernel launches this library has issued since it was loaded. */
long ig_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* IGSOLVE_H */
