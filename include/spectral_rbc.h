/*
 * spectral_rbc.h -- C ABI of the GB300 spectral Rayleigh-Benard library.
 *
 * Drop-in boundary for rustpde's pseudo-spectral RBC time step.  The
 * reference exposes Rust traits, not an FFI; every entry point below states
 * the reference item it replaces (paths relative to the rustpde repository).
 *
 * Conventions
 *  - Every function returns an int status: RBC_OK (0) or a negative error
 *    code; rbc_last_error() returns the message of the last failure on the
 *    calling thread.  No call aborts the process or traps on the device.
 *  - Arrays are row-major (x, y) with y contiguous, like the reference's
 *    ndarray default.  Complex spectral arrays are interleaved (re, im)
 *    doubles, the memory layout of num_complex::Complex<f64>.
 *  - A case handle is not thread-safe; different handles may be used from
 *    different threads.  Each case owns a CUDA stream; stepping calls are
 *    asynchronous and every state/diagnostic call synchronises that stream.
 *  - `stream` arguments are cudaStream_t values passed as void* (NULL: the
 *    legacy default stream).
 */
#ifndef SPECTRAL_RBC_H
#define SPECTRAL_RBC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define RBC_OK 0
#define RBC_ERR_INVALID (-1)     /* bad argument: size mismatch, null pointer, range */
#define RBC_ERR_CUDA (-2)        /* CUDA runtime failure */
#define RBC_ERR_NUMERIC (-3)     /* non-finite value detected in the state */
#define RBC_ERR_UNSUPPORTED (-4) /* valid request the library does not implement */
#define RBC_ERR_NOMEM (-5)       /* device allocation failed / budget exceeded */
#define RBC_ERR_CANCELLED (-6)   /* serving: the request was cancelled (rbc_server_cancel) */

/* ---- enums -------------------------------------------------------------- */
/* case kinds: Navier2D::new(adiabatic=true/false), Navier2D::new_periodic */
#define RBC_BOX_ADIABATIC 0
#define RBC_BOX_CONDUCTING 1
#define RBC_PERIODIC 2
/* arithmetic of the time step */
#define RBC_PREC_FP64 0
#define RBC_PREC_MIXED 1
/* fields (Navier2D public fields, src/navier/navier.rs:153-170) */
#define RBC_TEMP 0
#define RBC_UX 1
#define RBC_UY 2
#define RBC_PRES 3        /* pres[0] */
#define RBC_PSEUDO_PRES 4 /* pres[1] */
#define RBC_FIELDBC 5     /* fieldbc (read only) */
/* diagnostics */
#define RBC_NU 0       /* eval_nu       src/navier/functions.rs:12-36 */
#define RBC_NUVOL 1    /* eval_nuvol    functions.rs:42-75 */
#define RBC_RE 2       /* eval_re       functions.rs:82-101 */
#define RBC_KE 3       /* <(ux^2+uy^2)/2> with the volume weights of Field2::average */
#define RBC_DIV_NORM 4 /* ||divergence||_2, the quantity Navier2D::exit tests (navier.rs:855-862) */

typedef struct RbcParams {
  int nx, ny;       /* modes in x and y */
  double ra, pr;    /* Rayleigh and Prandtl numbers */
  double dt;        /* time step */
  double aspect;    /* aspect ratio L/H */
  int kind;         /* RBC_BOX_ADIABATIC / RBC_BOX_CONDUCTING / RBC_PERIODIC */
  int precision;    /* RBC_PREC_FP64, or RBC_PREC_MIXED: dense transforms on the tensor
                       cores (3xTF32), convection products in FP32, banded solves,
                       projection and state update in FP64 */
} RbcParams;

typedef struct RbcCase RbcCase;

const char* rbc_last_error(void);
/* library version string */
const char* rbc_version(void);

/* ---- case lifecycle ------------------------------------------------------
 * Replaces Navier2D::new (navier.rs:219-307) and Navier2D::new_periodic
 * (navier.rs:384-467).  The state starts at zero; the reference's unseeded
 * random_disturbance(0.1) is available seeded as rbc_random_disturbance.
 * Sizes: ny in [8, 4097], nx in [8, 4097] (box) or [8, 8192] (periodic), and
 * within those, what the step's passes can hold: a pass keeps the lanes it
 * transforms in a block's shared memory.  Where a Chebyshev axis's FFT form
 * would not fit, the dense transform is used (the same transform as an n x n
 * product); a case that fits in no form is refused at once with
 * RBC_ERR_INVALID, naming the pass and the bytes it needs.  On a GB300
 * (227 KB per block) the FP64 step runs periodic cases up to nx = 1208 and
 * ny = 631 and boxes up to nx = 906 (ny = 1707); the mixed form periodic
 * cases up to nx = 2418 and ny = 726, and boxes up to 1707 x 1707. */
int rbc_create(const RbcParams* params, RbcCase** out);
int rbc_destroy(RbcCase* c);
/* nu, ka, ra, pr, dt, scale_x, scale_y (navier.rs:46-55 get_nu/get_ka) */
int rbc_get_params(const RbcCase* c, double out[7]);

/* ---- initial conditions ---------------------------------------------------
 * set_velocity navier.rs:927-931, set_temperature :934-936,
 * random_disturbance :939-948 (seeded: splitmix64, row-major draws). */
int rbc_set_velocity(RbcCase* c, double amp, double m, double n);
int rbc_set_temperature(RbcCase* c, double amp, double m, double n);
int rbc_random_disturbance(RbcCase* c, double amp, uint64_t seed);
/* temperature = amp*(2u-1) at interior points (0 on walls), u ~ splitmix64(seed) */
int rbc_set_temperature_noise(RbcCase* c, double amp, uint64_t seed);

/* ---- solid obstacles (penalisation) ---------------------------------------
 * rbc_set_solid replaces `navier.solid = Some([mask, value])` (navier.rs:
 * 189-190): conv_ux, conv_uy and conv_temp subtract (-1/eta) mask w with
 * eta = 1e-2 and w = ux, uy, T + T_bc - value (navier.rs:551-560, 579-584,
 * 603-608).  mask, value: physical nx*ny arrays on the temperature grid
 * (value NULL = 0); mask NULL removes the solid.  FP64 cases, stepped on
 * their own or in a batch (the batch rebuilds the case's group plan and its
 * graphs; a batch case then steps bitwise as it does alone);
 * RBC_ERR_UNSUPPORTED for RBC_PREC_MIXED. */
int rbc_set_solid(RbcCase* c, const double* mask, const double* value, size_t n_doubles);
/* present = 1 with the mask and value (either may be NULL) when a solid is set */
int rbc_get_solid(const RbcCase* c, int* present, double* mask, double* value, size_t n_doubles);
/* Mask generators (src/navier/solid_masks.rs), host only: x (nx), y (ny) are
 * grid coordinates (e.g. rbc_get_coords of RBC_TEMP); mask, value: nx*ny.
 *   solid_cylinder_inner      solid_masks.rs:32-55
 *   solid_roughness_sinusoid  solid_masks.rs:58-98
 *   solid_porosity            solid_masks.rs:101-140 */
int rbc_solid_cylinder_inner(const double* x, int nx, const double* y, int ny, double x0, double y0, double radius,
                             double* mask, double* value);
int rbc_solid_roughness_sinusoid(const double* x, int nx, const double* y, int ny, double height, double wavenumber,
                                 double* mask, double* value);
int rbc_solid_porosity(const double* x, int nx, const double* y, int ny, double diameter, double porosity,
                       double* mask, double* value);
/* solid_porosity_interpolate (solid_masks.rs:144-174): the porosity mask on
 * the 513 x 513 Chebyshev grid, truncated in spectral space to (nx, ny) on
 * the GPU. */
int rbc_solid_porosity_interpolate(int nx, int ny, double diameter, double porosity, double* mask, double* value);

/* ---- stepping -------------------------------------------------------------
 * rbc_step: Integrate::update (src/lib.rs:137, navier.rs:737-765), nsteps
 * times, enqueued on the case stream (asynchronous). */
int rbc_step(RbcCase* c, int nsteps);
int rbc_synchronize(RbcCase* c);
int rbc_get_time(const RbcCase* c, double* t);   /* Integrate::get_time lib.rs:139 */
int rbc_set_time(RbcCase* c, double t);          /* Navier2D::reset_time navier.rs:951 */
int rbc_get_dt(const RbcCase* c, double* dt);    /* Integrate::get_dt lib.rs:141 */
/* Status word of the case (bits stay set until the case is destroyed; a
 * batch clears its cases' words when it is created):
 *   bit 0 (1): a non-finite value was written to the state;
 *   bit 1 (2): RBC_PREC_MIXED only -- a tensor-core completion wait of a lane
 *              GEMM timed out, so that step's results are incomplete (the
 *              kernel skipped its stores and returned instead of hanging). */
int rbc_status(RbcCase* c, int* status);
/* Integrate::exit (navier.rs:855-862): *stop = 1 if ||div|| is NaN */
int rbc_exit(RbcCase* c, int* stop);
/* integrate() (lib.rs:155-187): step until max_time; call cb(case, time, user)
 * whenever time % save_intervall is within dt/2 (save_intervall <= 0: never);
 * a non-zero return of cb stops the loop.  steps_done may be NULL.  Stops
 * after MAX_TIMESTEP (1e7) steps, or when exit() holds (the divergence norm is
 * NaN), as the reference does; returns RBC_ERR_CUDA when status bit 1 is set. */
typedef int (*rbc_callback)(RbcCase* c, double time, void* user);
int rbc_integrate(RbcCase* c, double max_time, double save_intervall, rbc_callback cb, void* user,
                  long* steps_done);

/* ---- state ----------------------------------------------------------------
 * The spectral arrays (Field2::vhat).  n_doubles must equal the array size
 * in doubles (complex arrays count 2 per element). */
int rbc_field_shape(const RbcCase* c, int field, int* n0, int* n1, int* is_complex);
int rbc_get_state(RbcCase* c, int field, double* host, size_t n_doubles);
int rbc_set_state(RbcCase* c, int field, const double* host, size_t n_doubles);
/* Field2::backward of a field (physical nx x ny values) */
int rbc_get_physical(RbcCase* c, int field, double* host, size_t n_doubles);
/* Field2 grid coordinates of a field (scaled by the aspect ratio as
 * Navier2D::_scale does for temp/ux/uy/pres) */
int rbc_get_coords(const RbcCase* c, int field, double* x, double* y);
/* diagnostics: RBC_NU, RBC_NUVOL, RBC_RE, RBC_KE, RBC_DIV_NORM */
int rbc_eval(RbcCase* c, int what, double* out);
int rbc_get_stream(RbcCase* c, void** stream);
/* device bytes held by the case (state, scratch, operators, step tables, solid mask) */
int rbc_device_bytes(const RbcCase* c, size_t* bytes);

/* Time the kernels of the step individually: runs nsteps steps launching each
 * stage on the case stream between CUDA events; stage_ms[k] receives the mean
 * duration of stage k (at most max_stages entries), *nstages the count. */
int rbc_profile_step(RbcCase* c, int nsteps, double* stage_ms, int max_stages, int* nstages);
/* name of stage k of the step (static string) */
const char* rbc_stage_name(const RbcCase* c, int k);
/* algorithmic HBM bytes of stage k (every array it must read or write, once) */
int rbc_stage_bytes(const RbcCase* c, int k, double* bytes);
/* name of a kernel id returned by rbc_batch_profile_step */
const char* rbc_kernel_name(int kernel);

/* ---- batches --------------------------------------------------------------
 * Many independent cases advanced together (no reference counterpart: the
 * reference advances one Navier2D at a time).  Cases are grouped by kind (box /
 * periodic) and precision, whatever their sizes; each pass of the step is one
 * launch per group whose work table covers the lanes of every case in the
 * group, groups run as parallel branches, and the whole batch step is one
 * CUDA graph.  Case handles
 * from rbc_batch_case are borrowed (do not destroy them); they share the batch
 * stream, so their state/diagnostic calls are ordered after rbc_batch_step.
 * Mixed-precision batches time the forms of each FP64 pass at creation and
 * keep the fastest (rbc_batch_tuning); the environment variable
 * RBC_BATCH_FORM pins the forms instead (profiling runs): the string
 * rbc_batch_tuning_forms returns, "<FP64 passes>[;<GEMM passes>[;<groups>]]",
 * each part one digit for all its entries or a comma-separated digit per
 * entry; an empty part is left to the autotuner.  FP64 passes: 0 a CTA per
 * lane, 1 128-thread CTAs, 2 one thread per sub-lane, 3 the same with the
 * periodic Y2 launches fused into one.  GEMM passes: 0 output tiles of up to
 * 64 columns, 4 up to 128, 5 64 in the warp-specialised form (producer, MMA
 * and flush warps; all 0 when the part is missing).  Groups: mixed-
 * precision cases whose Chebyshev lengths are all 2^p + 1 are grouped apart,
 * and each such group runs its transforms as tensor-core GEMMs (0) or as the
 * FP64 plan's FFT butterflies (1; at least as accurate), whichever its step
 * measured faster (all 0 when the part is missing).  The group
 * whose step takes longest runs on a high-priority branch, so its thread
 * blocks are dispatched first; RBC_BATCH_PRIORITY=0 gives every branch the
 * default priority. */
typedef struct RbcBatch RbcBatch;
int rbc_batch_create(const RbcParams* params, int ncases, RbcBatch** out);
int rbc_batch_destroy(RbcBatch* b);
int rbc_batch_size(const RbcBatch* b, int* ncases);
int rbc_batch_case(RbcBatch* b, int i, RbcCase** c);
int rbc_batch_step(RbcBatch* b, int nsteps);
int rbc_batch_synchronize(RbcBatch* b);
/* number of size buckets and of kernel launches per batch step */
int rbc_batch_layout(const RbcBatch* b, int* nbuckets, int* launches_per_step);
int rbc_batch_get_stream(RbcBatch* b, void** stream);
/* The spectral state of every case of a batch lives in one device region:
 * case after case, each as temp, ux, uy, pres[0], pres[1] (the rbc_get_state
 * layouts), every array padded to a multiple of 256 bytes.  These copy the
 * whole region in one transfer (host memory may be pinned for speed). */
/* Per-kernel timing of the batch step: every launch of every bucket runs
 * alone between two events; stage k aggregates one kernel (stage_kernel[k],
 * see rbc_kernel_name) over all buckets: mean ms per step and algorithmic
 * bytes per step (stage_bytes and stage_kernel may be NULL). */
int rbc_batch_profile_step(RbcBatch* b, int nsteps, double* stage_ms, double* stage_bytes, int* stage_kernel,
                           int max_stages, int* nstages);
/* every launch of the batch step timed alone, in step order: kernel id
 * (rbc_kernel_name), bucket, pass id, mean ms, algorithmic bytes (may be NULL) */
int rbc_batch_profile_launches(RbcBatch* b, int nsteps, int* kernel, int* bucket, int* pass, double* ms,
                               double* bytes, int max_launches, int* nlaunches);
/* Autotuner record of a batch: for the passes that have other forms beside
 * the one-CTA-per-lane form, rbc_batch_create timed every form on the batch
 * (ms per step) and kept the fastest.  *n = number of decisions; entry k (if
 * 0 <= k < *n) is written to the non-null outputs: the CTA form's kernel and
 * time, the fastest other form's kernel and time (kernel ids: see
 * rbc_kernel_name). */
int rbc_batch_tuning(const RbcBatch* b, int k, int* kernel_cta, int* kernel_lanes, double* ms_cta, double* ms_lanes,
                     int* n);
/* The forms kept, one digit per decision of rbc_batch_tuning, comma-separated,
 * the FP64 passes' first, then after a ';' the GEMM passes', then after a
 * second ';' (when the batch has groups of 2^p + 1 sizes) each such group's
 * transforms (FP64: 0 a CTA per lane, 1 128-thread CTAs, 2 a thread per
 * sub-lane, 3 the same with the periodic Y2 launches fused, timed for
 * one-group batches; GEMM: 0 64-output tiles, 4 128-output tiles, 5
 * warp-specialised; groups: 0 tensor-core GEMMs, 1 FP64 butterflies), NUL-
 * terminated in buf (len bytes).  Passed as RBC_BATCH_FORM it makes another
 * batch of the same cases keep the same forms, whatever its own timings say. */
int rbc_batch_tuning_forms(const RbcBatch* b, char* buf, size_t len);
int rbc_batch_state_bytes(const RbcBatch* b, size_t* bytes);
int rbc_batch_state_offset(const RbcBatch* b, int i, size_t* offset);
int rbc_batch_get_state_all(RbcBatch* b, void* host, size_t bytes);
int rbc_batch_set_state_all(RbcBatch* b, const void* host, size_t bytes);
/* rbc_batch_set_state_all(host_in), rbc_batch_step(nsteps) and
 * rbc_batch_get_state_all(host_out) in one call, with the same results, the
 * copies pipelined: each group's cases hold one contiguous range of the state
 * (rbc_batch_state_offset), which is copied in, stepped by that group's own
 * graph and copied back on the group's branch, so that one group's copies
 * overlap the other groups' steps.  Inputs are copied in the order of the
 * groups' step times, shortest first.  host_in and host_out (bytes =
 * rbc_batch_state_bytes each, page-locked for the copies to be asynchronous)
 * may be the same buffer; returns when host_out is written. */
int rbc_batch_step_io(RbcBatch* b, const void* host_in, void* host_out, size_t bytes, int nsteps);

/* ---- snapshots -----------------------------------------------------------------
 * Navier2D::write (navier.rs:975-1013) and Navier2D::read (navier.rs:961-972)
 * with the reference's dataset layout (groups temp, ux, uy, pres with v and
 * vhat / vhat_re / vhat_im; x, dx, y, dy; time, ra, pr, nu, kappa) in a
 * self-describing little-endian binary file ("RBCSNAP1") plus a JSON sidecar
 * (path + ".json").  Reading restores the spectral fields and the time; a
 * snapshot of another resolution is broadcast (overlapping low modes copied,
 * the rest zero), as field/read.rs:116-125. */
int rbc_write_snapshot(RbcCase* c, const char* path);
int rbc_read_snapshot(RbcCase* c, const char* path);

/* ---- statistics and diagnostics series ------------------------------------------
 * Statistics (src/navier/statistics.rs) on the device, in the `field` space
 * (ortho x ortho): rbc_stats_reset = Statistics::new (tot_time = current
 * time); rbc_stats_update = Statistics::update with the case's current state
 * (running mean of the temperature with the boundary field, the latest ux and
 * uy, and the Nusselt field (dT/dz / -s + uy T / kappa) 2 s); rbc_stats_write
 * = Statistics::write (groups temp, ux, uy, nusselt; scalars tot_time,
 * avg_time, num_save, ka) in the snapshot format.  which: 0 temp, 1 ux, 2 uy,
 * 3 nusselt. */
int rbc_stats_reset(RbcCase* c);
int rbc_stats_update(RbcCase* c);
int rbc_stats_info(const RbcCase* c, double* tot_time, double* avg_time, long* num_save);
int rbc_stats_get(RbcCase* c, int which, double* host, size_t n_doubles);
int rbc_stats_write(RbcCase* c, const char* path);
/* the diagnostics of Navier2D::callback (navier.rs:819-838): rbc_diag_record
 * appends (time, Nu, Nuvol, Re) evaluated on the device; rbc_diag_series
 * copies up to max_entries of them (*n = entries recorded; NULL outputs are
 * skipped). */
int rbc_diag_record(RbcCase* c);
int rbc_diag_series(const RbcCase* c, double* time, double* nu, double* nuvol, double* re, int max_entries, int* n);

/* ---- serving loop ------------------------------------------------------------
 * No reference counterpart (the reference runs one Navier2D per process).  A
 * request is one RBC solve: the case of `params` from the standard initial
 * fields (set_velocity(0.2, 1, 1) and seeded temperature noise 1e-3, see
 * rbc_set_temperature_noise) to `horizon` time units, i.e. round(horizon/dt)
 * steps.  Set-up threads build requested cases (operators, factorisations,
 * boundary field, initial fields) while memory is reserved within the budget;
 * a scheduler thread admits built cases while slots (max_active) allow, keeps
 * every admitted case's state and
 * factorised operators on the device, and advances all of them together in
 * batched steps (continuous batching: requests that arrive while others run
 * join at the next chunk of chunk_steps steps).  Each finished request yields
 * a result (Nu, KE at its horizon, timestamps on the server clock).  A case
 * computes exactly the same numbers alone or in any mix.  The FP64 passes run
 * as a CTA per lane; RBC_SERVER_FORM=1 to 5 (read when the active set
 * changes) selects another of the forms above for every case, which keeps
 * that property. */
typedef struct RbcServer RbcServer;
typedef struct RbcServerConfig {
  size_t hbm_budget_bytes; /* admission budget for the cases' device memory */
  int max_active;          /* cases advanced together at most */
  int chunk_steps;         /* steps launched per scheduling round */
  int setup_threads;       /* host threads building admitted cases */
} RbcServerConfig;
typedef struct RbcRequestResult {
  long long id;
  int status;      /* RBC_OK, RBC_ERR_NUMERIC (non-finite state), RBC_ERR_NOMEM (never fits),
                      RBC_ERR_CUDA (status bit 1, see rbc_status) or RBC_ERR_CANCELLED */
  int steps;       /* steps advanced (fewer than requested when cancelled) */
  double sim_time; /* simulated time reached */
  double t_submit, t_admit, t_done; /* server clock, seconds */
  double nu, ke;   /* eval_nu and kinetic energy at the horizon */
  long long grid_points;
} RbcRequestResult;
typedef struct RbcServerStats {
  double now;      /* server clock, seconds */
  int pending, active;
  long long completed;
  size_t bytes_in_use;
  double grid_point_steps; /* advanced so far */
  long long steps_launched, rebuilds;
  size_t peak_bytes_in_use; /* largest bytes_in_use so far (never above the budget but for a
                               single case admitted alone) */
} RbcServerStats;
int rbc_server_create(const RbcServerConfig* cfg, RbcServer** out);
/* params->precision selects the form of the case (RBC_PREC_FP64 / RBC_PREC_MIXED) */
int rbc_server_submit(RbcServer* s, const RbcParams* params, double horizon, uint64_t seed, long long* id);
/* Cancel a request: *found = 1 if it had not finished.  A request still
 * queued is answered at once; one being built, waiting for a slot or
 * advancing stops at the scheduler's next chunk boundary (no step of it is in
 * flight when its memory is freed).  Either way a result with status
 * RBC_ERR_CANCELLED and the steps it advanced is queued; the other requests'
 * numbers are unaffected.  No reference counterpart (the reference runs one
 * case to completion). */
int rbc_server_cancel(RbcServer* s, long long id, int* found);
/* completed results (at most max_results, *n of them; non-blocking) */
int rbc_server_poll(RbcServer* s, RbcRequestResult* out, int max_results, int* n);
/* wait until nothing is pending or running (or timeout); *idle = 1 when idle */
int rbc_server_wait_idle(RbcServer* s, double timeout_s, int* idle);
int rbc_server_stats(RbcServer* s, RbcServerStats* stats);
/* stops the scheduler; unfinished requests are dropped */
int rbc_server_destroy(RbcServer* s);

/* ---- device memory helpers (callers that do not link the CUDA runtime) ---- */
int rbc_host_alloc_pinned(void** ptr, size_t bytes);
int rbc_host_free_pinned(void* ptr);
int rbc_dev_alloc(void** ptr, size_t bytes);
int rbc_dev_free(void* ptr);
int rbc_memcpy_h2d(void* dst, const void* src, size_t bytes);
int rbc_memcpy_d2h(void* dst, const void* src, size_t bytes);
int rbc_device_synchronize(void);
/* The GPU this library's calls run on, for the calling thread (the library
 * links its own CUDA runtime, so a framework's device selection does not
 * reach it).  Handles are created on the device current at creation and must
 * be used with it current; a serving loop keeps the device of its creation.
 * No reference counterpart (the reference runs on the CPU). */
int rbc_set_device(int ordinal);
int rbc_get_device(int* ordinal);

/* ---- funspace primitives on device buffers ---------------------------------
 * Space2::new(base0, base1) (funspace/src/space2.rs:37-50) with bases
 * chebyshev / cheb_dirichlet / cheb_neumann / cheb_dirichlet_bc /
 * cheb_neumann_bc / fourier_r2c (funspace/src/lib.rs:230-345).  Fourier is
 * supported along axis 0 (the reference's R2c x R2r space). */
#define FS_CHEBYSHEV 0
#define FS_CHEB_DIRICHLET 1
#define FS_CHEB_NEUMANN 2
#define FS_CHEB_DIRICHLET_BC 3
#define FS_CHEB_NEUMANN_BC 4
#define FS_FOURIER_R2C 5
/* shape selectors for fs_space_shape */
#define FS_PHYSICAL 0
#define FS_SPECTRAL 1
#define FS_ORTHO 2

typedef struct FsSpace FsSpace;
/* Lengths n0, n1 in [4, 8192]; a space whose lanes (with the transforms' work
 * elements) do not fit a block's shared memory is refused with
 * RBC_ERR_INVALID (on a GB300: Chebyshev lengths up to 3628, FourierR2c up
 * to 2902 even and 2419 odd). */
int fs_space_create(int base0, int n0, int base1, int n1, FsSpace** out);
int fs_space_destroy(FsSpace* s);
int fs_space_shape(const FsSpace* s, int which, int* n0, int* n1, int* is_complex);
/* Field2::forward / backward / to_ortho / from_ortho / gradient (src/field.rs:103-129) */
int fs_forward(FsSpace* s, const double* d_phys, double* d_spec, void* stream);
int fs_backward(FsSpace* s, const double* d_spec, double* d_phys, void* stream);
int fs_to_ortho(FsSpace* s, const double* d_spec, double* d_ortho, void* stream);
int fs_from_ortho(FsSpace* s, const double* d_ortho, double* d_spec, void* stream);
/* scale: two doubles or NULL (None) */
int fs_gradient(FsSpace* s, const double* d_spec, double* d_ortho, int deriv0, int deriv1, const double* scale,
                void* stream);

/* fs_forward_noalloc: the transform of fs_forward, computed by the same
 * kernels, for callers that must not allocate while they run -- a loop that
 * has handed all device memory to a fixed budget, or that cannot afford the
 * device-wide synchronisation cudaFree implies.  No counterpart in the
 * reference (Field2::forward, src/field.rs:103-107, allocates freely).
 *
 * The call allocates nothing, on the device or the host: the intermediate
 * array between the two axis passes (phys0 x spec1 doubles) lives in a fixed
 * device buffer of FS_NOALLOC_SCRATCH_BYTES that the library owns, one per
 * device.  A space whose intermediate needs more returns RBC_ERR_INVALID
 * before anything is enqueued.  Nothing in the buffer has to start at zero:
 * the first pass writes every element the second pass reads.
 *
 * The first call on a device looks the buffer's address up (this can load
 * the library's device code); make it before any stream capture, with the
 * space's device current.  All calls on one device share the buffer, so two
 * calls that may run at the same time (on different streams, or from
 * different threads without ordering) race on it; calls ordered on one
 * stream do not.  The looked-up address is kept per device ordinal for the
 * life of the process; after cudaDeviceReset it no longer names the buffer,
 * so do not call this entry point on a device that was reset. */
#define FS_NOALLOC_SCRATCH_BYTES (4u * 1024u * 1024u)
int fs_forward_noalloc(FsSpace* s, const double* d_phys, double* d_spec, void* stream);

/* ---- batched 1-D transforms and solves (precision microbenchmark) ----------
 * `lanes` contiguous lanes (row-major lanes x length) of one Chebyshev-family
 * basis (FS_CHEBYSHEV, FS_CHEB_DIRICHLET, FS_CHEB_NEUMANN) of length n, the
 * 1-D restriction of Space2's axis operations (funspace ortho.rs:235-312,
 * composite.rs:156-238) and of HholtzAdi::solve along one axis
 * (hholtz_adi.rs:92-131).  precision RBC_PREC_FP64 runs the FP64 lane
 * kernels; RBC_PREC_MIXED applies each operator as one dense matrix on the
 * tensor cores (3xTF32, FP32 accumulation) and keeps the banded Helmholtz
 * sweep in FP64.  Inputs and outputs are FP64 in both forms. */
#define FS_OP_FORWARD 0    /* physical (n) -> spectral (m) */
#define FS_OP_BACKWARD 1   /* spectral (m) -> physical (n) */
#define FS_OP_TO_ORTHO 2   /* spectral (m) -> ortho (n) */
#define FS_OP_FROM_ORTHO 3 /* ortho (n) -> spectral (m) */
#define FS_OP_HHOLTZ 4     /* ortho right-hand side (n) -> spectral solution (m) */
typedef struct FsLanes FsLanes;
int fs_lanes_create(int base, int n, int precision, FsLanes** out);
int fs_lanes_destroy(FsLanes* p);
/* n: physical / ortho length, m: spectral length */
int fs_lanes_shape(const FsLanes* p, int* n, int* m);
/* coefficient c of (I - c D2) for FS_OP_HHOLTZ (HholtzAdi::new(field, [c]) along this axis) */
int fs_lanes_set_hholtz(FsLanes* p, double c);
int fs_lanes_apply(FsLanes* p, int op, const double* d_in, double* d_out, int lanes, void* stream);
/* Waits for `stream`, then returns and clears the status word of the applies
 * enqueued so far: bit 1 (2) when a tensor-core completion wait of an
 * RBC_PREC_MIXED apply timed out (its output is incomplete); 0 otherwise. */
int fs_lanes_status(FsLanes* p, void* stream, unsigned int* status);

/* Test hook (no counterpart in the reference): the poll limit of the lane
 * GEMM's bounded completion waits on the current device; a negative value
 * restores the default (2^22 polls).  A limit of 0 makes every wait run out at
 * once, so that the time-out path -- status bit 1 set, stores skipped, the
 * MMAs in flight drained, tensor memory freed -- can be exercised without a
 * hung GPU.  It applies to every RBC_PREC_MIXED handle on the device. */
int rbc_set_gemm_wait_limit(long long polls);

/* ---- solvers ----------------------------------------------------------------
 * Hholtz::new (src/solver/hholtz.rs:42-76), HholtzAdi::new (hholtz_adi.rs:44-63),
 * Poisson::new (poisson.rs:50-90); Solve::solve (src/solver.rs:56-64) maps an
 * ortho-sized input to a spectral-sized output of the space. */
#define SV_HHOLTZ 0
#define SV_HHOLTZ_ADI 1
#define SV_POISSON 2
typedef struct SvSolver SvSolver;
int sv_create(FsSpace* s, int kind, const double c[2], SvSolver** out);
int sv_destroy(SvSolver* sv);
int sv_solve(SvSolver* sv, const double* d_in, double* d_out, void* stream);

/* ---- Navier2DAdjoint (src/navier/navier_adjoint.rs) -----------------------
 * rbc_adjoint_create replaces Navier2DAdjoint::new (navier_adjoint.rs:151-283,
 * kind BOX_*) and ::new_periodic (:287-409): params as rbc_create, dt is the
 * adjoint's pseudo time step, precision RBC_PREC_FP64.  rbc_adjoint_step is
 * Integrate::update (:767-800): one Navier2D step with dt = 1e-2 gives the
 * residual, (1 - D2) smooths it, the state advances with the adjoint
 * convection, diffusion and a projection; one CUDA graph per update.
 * Fields: RBC_TEMP, RBC_UX, RBC_UY, RBC_PRES, RBC_PSEUDO_PRES (the state,
 * spectral, as rbc_get_state) and the smoothed residuals below.
 * rbc_adjoint_eval: Nu, Nuvol, Re (:932-963), KE, |div|.  rbc_adjoint_residual:
 * the L2 norms of the unsmoothed and the smoothed residual of ux, uy, temp
 * (:866-874).  rbc_adjoint_exit: NaN divergence or smoothed residual < 1e-8
 * (:889-906). */
#define RBC_ADJ_TEMP_RES 10
#define RBC_ADJ_UX_RES 11
#define RBC_ADJ_UY_RES 12
typedef struct RbcAdjoint RbcAdjoint;
int rbc_adjoint_create(const RbcParams* params, RbcAdjoint** out);
int rbc_adjoint_destroy(RbcAdjoint* a);
int rbc_adjoint_set_velocity(RbcAdjoint* a, double amp, double m, double n);    /* :965-968 */
int rbc_adjoint_set_temperature(RbcAdjoint* a, double amp, double m, double n); /* :969-971 */
int rbc_adjoint_step(RbcAdjoint* a, int nsteps);
int rbc_adjoint_synchronize(RbcAdjoint* a);
int rbc_adjoint_get_time(const RbcAdjoint* a, double* t);
int rbc_adjoint_set_time(RbcAdjoint* a, double t); /* reset_time :973-976 */
int rbc_adjoint_field_shape(const RbcAdjoint* a, int field, int* n0, int* n1, int* is_complex);
int rbc_adjoint_get_state(RbcAdjoint* a, int field, double* host, size_t n_doubles);
int rbc_adjoint_set_state(RbcAdjoint* a, int field, const double* host, size_t n_doubles);
int rbc_adjoint_eval(RbcAdjoint* a, int what, double* out);
int rbc_adjoint_residual(RbcAdjoint* a, double out[6]);
int rbc_adjoint_exit(RbcAdjoint* a, int* stop);
int rbc_adjoint_get_stream(RbcAdjoint* a, void** stream);
/* Navier2DAdjoint::write / read (navier_adjoint.rs:991-1040) in the snapshot
 * format of rbc_write_snapshot; read restores temp, ux, uy and time */
int rbc_adjoint_write_snapshot(RbcAdjoint* a, const char* path);
int rbc_adjoint_read_snapshot(RbcAdjoint* a, const char* path);

/* ---- Diffusion2D (src/navier/diffusion.rs:113-238) ------------------------
 * df_create replaces Diffusion2D::new(field, kappa, dt) (diffusion.rs:140-153)
 * for a field on the space (base0, n0) x (base1, n1): composite or Fourier
 * bases (Fourier along axis 0 only), Hholtz solver with c = dt*kappa on both
 * axes.  df_step is Integrate::update (diffusion.rs:186-207): rhs =
 * to_ortho(vhat) + dt force + dt kappa (d2/dx2 + d2/dy2) fieldbc, vhat =
 * Hholtz.solve(rhs); one CUDA graph per update on the case stream.
 * df_impulse: diffusion.rs:156-163; df_add_force: :168-171 (real spaces:
 * the force has field.v's shape and is added in ortho space); df_add_fieldbc:
 * :176-179 with the boundary field's spectral coefficients on (base0, base1);
 * df_get_physical: field.backward() (+ fieldbc.v when with_bc, as callback
 * writes it, :214-225).  State arrays: spectral (spec0 x spec1), interleaved
 * re/im for a Fourier axis. */
typedef struct DfCase DfCase;
int df_create(int base0, int n0, int base1, int n1, double kappa, double dt, DfCase** out);
int df_destroy(DfCase* d);
int df_shape(const DfCase* d, int which, int* n0, int* n1, int* is_complex);
int df_get_state(DfCase* d, double* host, size_t n_doubles);
int df_set_state(DfCase* d, const double* host, size_t n_doubles);
int df_impulse(DfCase* d);
int df_add_force(DfCase* d, const double* force, size_t n_doubles);
int df_add_fieldbc(DfCase* d, int base0, int base1, const double* vhat, size_t n_doubles);
int df_step(DfCase* d, int nsteps);
int df_synchronize(DfCase* d);
int df_get_time(const DfCase* d, double* t);
int df_get_dt(const DfCase* d, double* dt);
int df_get_physical(DfCase* d, int with_bc, double* host, size_t n_doubles);
int df_get_stream(DfCase* d, void** stream);

#ifdef __cplusplus
}
#endif
#endif /* SPECTRAL_RBC_H */
