/*
 * fv3d_gb300.h -- C ABI of the GB300 (sm_103a) finite-volume hydro step.
 *
 * The entry points replace the reference fv3d's hot path, which sits behind
 * C++ classes taking `const Params&` and `Kokkos::View` handles:
 *
 *   fv_read_ini / fv_parse_ini   <- fv3d::readInifile            (SimInfo.h:169-306)
 *   fvgpu_set_prim / get_prim    <- fv3d::primToCons/consToPrim  (SimInfo.h:313-331)
 *   fvgpu_init_problem           <- InitFunctor::init(Q) + primToCons (Init.h:247-279,
 *                                   main.cpp:42-44); fvgpu_generate fills caller arrays
 *   fvgpu_compute_dt             <- ComputeDtFunctor::computeDt  (ComputeDt.h:17-63)
 *   fvgpu_step                   <- UpdateFunctor::update        (Update.h:180-206),
 *                                   which runs BoundaryManager::fillBoundaries
 *                                   (BoundaryConditions.h:146-215) inside euler_step
 *                                   (Update.h:164-178)
 *   fvgpu_advance                <- the time loop of main.cpp:51-74 (without I/O)
 *   fvgpu_batch_*                <- no counterpart: many independent problems
 *                                   advanced together, each with its own dt.
 *
 * Conventions
 *   - Every function returns an int status (FV_OK == 0).  No C++ exception
 *     crosses this boundary.
 *   - Field arrays passed in or out are HOST arrays of the interior cells only,
 *     in C order [Nz][Ny][Nx] (x fastest), i.e. element (i,j,k) of the
 *     reference's View Q(k+Ng, j+Ng, i+Ng, var).  A NULL pointer means "all
 *     zeros" on input and "do not copy" on output.
 *   - A handle is not thread-safe and owns all of its device memory.  Work is
 *     ordered on one CUDA stream per handle; fvgpu_step returns before the GPU
 *     has finished, every call that returns data synchronises.
 */
#ifndef FV3D_GB300_H
#define FV3D_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Enumerations.  Numeric values equal the reference's enums (SimInfo.h:32-69). */
enum fv_boundary   { FV_BC_ABSORBING = 0, FV_BC_REFLECTING = 1, FV_BC_PERIODIC = 2, FV_BC_C91 = 3 };
enum fv_riemann    { FV_HLL = 0, FV_HLLC = 1 };
enum fv_stepping   { FV_TS_EULER = 0, FV_TS_RK2 = 1 };
enum fv_recon      { FV_PCM = 0, FV_PCM_WB = 1, FV_PLM = 2 };
enum fv_tc_mode    { FV_TCM_CONSTANT = 0, FV_TCM_B02 = 1 };
enum fv_bctc_mode  { FV_BCTC_NONE = 0, FV_BCTC_FIXED_TEMPERATURE = 1, FV_BCTC_FIXED_GRADIENT = 2 };
enum fv_visc_mode  { FV_VSC_CONSTANT = 0 };
/* Storage/arithmetic of the GPU path (driver-only setting, no reference counterpart). */
enum fv_precision  { FV_PREC_FP64 = 0, FV_PREC_FP32_MIXED = 1 };
/* FV_PHYS_REFERENCE reproduces the reference's arithmetic, including its
 * viscous flux divergence without 1/d (Viscosity.h:151), its z-branch index
 * and field mix-ups (Viscosity.h:122-129) and HLLC's kinetic energy from two
 * velocities (RiemannSolvers.h:52-55).  FV_PHYS_CORRECTED divides the
 * viscous fluxes by the cell size, uses the mirror of the x / y branches
 * for z, and gives HLLC all three velocities (no reference counterpart). */
enum fv_physics    { FV_PHYS_REFERENCE = 0, FV_PHYS_CORRECTED = 1 };

/* Status codes. */
enum fv_status {
  FV_OK = 0,
  FV_ERR_PARAM = 1,        /* invalid argument or parameter set                  */
  FV_ERR_UNSUPPORTED = 2,  /* valid reference setting this build does not run    */
  FV_ERR_CUDA = 3,         /* a CUDA runtime call or kernel launch failed        */
  FV_ERR_NONFINITE = 4,    /* the dt reduction met NaN/Inf or rho<=0 / p<=0      */
  FV_ERR_NOMEM = 5,        /* device or pinned host allocation failed            */
  FV_ERR_IO = 6,           /* file could not be read                             */
  FV_ERR_TIMEOUT = 7,      /* a bounded device-side wait gave up                 */
  FV_ERR_STATE = 8         /* call order violated (e.g. step before set_prim)    */
};

/*
 * Run parameters.  Mirrors fv3d::Params (SimInfo.h:72-159) minus the Kokkos
 * ranges, plus driver-only fields (precision, physics, problem/filename
 * strings).
 * Fill it with fv_read_ini / fv_parse_ini (reference readInifile semantics,
 * including single-precision parsing of every GetFloat key) or by hand; dx,
 * dy, dz must then equal (max-min)/N as readInifile computes them.
 */
typedef struct fv_params {
  /* mesh */
  int Nx, Ny, Nz, Ng;
  double xmin, xmax, ymin, ymax, zmin, zmax;
  double dx, dy, dz;
  /* run */
  double save_freq, tend;
  int boundary_x, boundary_y, boundary_z;
  int reconstruction, riemann_solver, time_stepping;
  double CFL;
  /* physics */
  double epsilon, gamma0;
  int gravity, well_balanced_flux_at_z_bc;
  double g;
  int well_balanced, thermal_conductivity_active;
  /* thermal conduction */
  int thermal_conductivity_mode, bctc_zmin;
  double kappa;
  int bctc_zmax, viscosity_active;
  double bctc_zmin_value, bctc_zmax_value;
  /* viscosity */
  int viscosity_mode, seed;
  double mu;
  /* polytrope / H84 / C91 / B02 */
  double m1, theta1, m2, theta2, h84_pert, c91_pert;
  double b02_zmid, b02_kappa1, b02_kappa2, b02_thickness;
  /* misc */
  int log_frequency, precision;
  char problem[64];
  char filename_out[256];
  int physics;          /* fv_physics ([gpu] physics = reference | corrected) */
} fv_params;

/* Human-readable name of a status code (static storage). */
const char* fv_status_string(int status);

/* readInifile (SimInfo.h:169-306) on a file / on INI text held in memory.
 * Like the reference, a missing file or malformed line is not an error: the
 * affected keys take their defaults.  FV_ERR_PARAM only for NULL arguments. */
int fv_read_ini(const char* path, fv_params* out);
int fv_parse_ini(const char* text, fv_params* out);

/* IOManager::saveSolution (IOManager.h:88-192) for interior primitive arrays
 * ([Nz][Ny][Nx]): the reference's HDF5 snapshot file at `path` -- root
 * attributes Ntx..kend (int) and problem (string), vertex datasets x, y, z,
 * and a group ite_<iteration> with datasets rho, u, v, w, prs and a time
 * attribute.  iteration 0 creates (truncates) the file, later iterations
 * add their group to it.  Written without an HDF5 library, in the original
 * HDF5 format (superblock 0, symbol-table groups, contiguous datasets).
 * FV_ERR_IO when the file cannot be written or is not one this call made. */
int fv_h5_save(const fv_params* params, const char* path, int iteration, double t, const double* rho,
               const double* u, const double* v, const double* w, const double* prs);

/* ---- single problem --------------------------------------------------- */
typedef struct fv_sim fv_sim;

/* Allocate device state for one problem on the current CUDA device.
 * precision FV_PREC_FP64 (default) is the bit-exact form; FV_PREC_FP32_MIXED
 * runs the problem in the FP32-mixed form through the batch machinery (a
 * batch of one): every call below works except set_cons / get_cons and
 * per-kernel profiling (FV_ERR_UNSUPPORTED).  FV_ERR_UNSUPPORTED names
 * settings this build does not run (see fvgpu_last_error).  FP64 device
 * memory: 3 states of 5 fields (U^n, U*, scratch), plus a primitive copy
 * of U^n with RK2 time stepping; a state is 5 fields of pitch x rows
 * doubles (pitch: Nx rounded up to 16; each field rounded up to 256 bytes). */
int fvgpu_create(const fv_params* params, fv_sim** out);
int fvgpu_destroy(fv_sim* sim);
/* Message for the last failing call on this handle ("" if none). */
const char* fvgpu_last_error(const fv_sim* sim);

/* Set the state from primitive (rho,u,v,w,p) or conserved (rho,rhou,rhov,rhow,E)
 * host arrays; primToCons/consToPrim arithmetic as States.h:20-45. */
int fvgpu_set_prim(fv_sim* sim, const double* rho, const double* u, const double* v,
                   const double* w, const double* p);
int fvgpu_get_prim(fv_sim* sim, double* rho, double* u, double* v, double* w, double* p);
int fvgpu_set_cons(fv_sim* sim, const double* rho, const double* mx, const double* my,
                   const double* mz, const double* E);
int fvgpu_get_cons(fv_sim* sim, double* rho, double* mx, double* my, double* mz, double* E);

/* InitFunctor(params).init(Q) followed by primToCons (Init.h:228-279,
 * main.cpp:42-44), on the GPU: the generator named by params.problem
 * (sod_x, sod_y, sod_z, blast, rayleigh-taylor, diffusion, H84, C91) writes
 * the state directly.  Positions and operation order are the reference's
 * (sod / blast / diffusion bit for bit; cos and pow may differ in the last
 * place).  H84 / C91 perturbations come from a counter-based splitmix64
 * stream of params.seed (cell (k*Ny + j)*Nx + i, stream 31 / 32) in place of
 * Kokkos' XorShift64 pool, whose draws depend on the thread schedule.
 * FV_ERR_PARAM for an unknown problem (where Init.h:241-242 throws). */
int fvgpu_init_problem(fv_sim* sim);
/* The same generator into caller arrays of primitives (rho, u, v, w, p;
 * [Nz][Ny][Nx]; any memory, NULL skips a field), without a handle: the
 * state init.init(Q) leaves in Q's interior. */
int fvgpu_generate(const fv_params* params, double* rho, double* u, double* v, double* w, double* p);

/* ComputeDtFunctor::computeDt on the current state: *dt = CFL/max(inv[0..2]);
 * inv (may be NULL) receives {inv_dt_hyp, inv_dt_tc, inv_dt_visc}. */
int fvgpu_compute_dt(fv_sim* sim, double* dt, double inv[3]);
/* One UpdateFunctor::update with the given dt (Euler or RK2 per params). */
int fvgpu_step(fv_sim* sim, double dt);
/* One update from and to caller arrays of primitives (rho, u, v, w, p;
 * [Nz][Ny][Nx], no padding) that the GPU addresses directly: pinned host
 * memory, device memory, or ordinary host memory where the device reads
 * pageable memory.  Does primToCons of prim_in (the reference's set-up of U,
 * main.cpp:43-44), takes the CFL dt of that state when dt <= 0
 * (ComputeDtFunctor::computeDt) or dt otherwise, runs one update and writes
 * consToPrim of the result to prim_out (NULL entries are skipped); the
 * kernels read and write the caller's arrays themselves, with no staging
 * copies.  Returns when prim_out is written; *dt_used (may be NULL)
 * receives the dt taken.  The result also stays in the handle.  Arrays the
 * GPU cannot address give FV_ERR_PARAM. */
int fvgpu_step_host(fv_sim* sim, const double* const prim_in[5], double dt, double* const prim_out[5],
                    double* dt_used);
/* The main.cpp:51-74 loop: while (t + epsilon < tend && steps < max_steps)
 * { dt = computeDt(); update(dt); t += dt; }.  *t is read and written; *nsteps
 * (may be NULL) receives the number of steps taken.  max_steps <= 0 means no
 * limit.  dt never leaves the GPU between steps. */
int fvgpu_advance(fv_sim* sim, double tend, long max_steps, double* t, long* nsteps);
/* Enqueue nsteps steps of the same loop without a time bound (each dt from
 * the CFL reduction of the previous step, computed on the GPU) and return
 * without waiting.  A non-finite dt stops the remaining steps and is reported
 * by the next synchronising call (fvgpu_compute_dt / fvgpu_advance). */
int fvgpu_enqueue_steps(fv_sim* sim, long nsteps);
/* Sum over the interior of each conserved field (compensated summation). */
int fvgpu_conserved_totals(fv_sim* sim, double out[5]);

/* Launch on a caller-owned CUDA stream (cudaStream_t); NULL restores the
 * handle's own stream. */
int fvgpu_set_stream(fv_sim* sim, void* cuda_stream);
int fvgpu_synchronize(fv_sim* sim);
/* Number of kernels this handle has launched since creation. */
int fvgpu_launch_count(const fv_sim* sim, long* count);
/* Per-kernel CUDA-event timing.  While enabled every kernel launch is
 * bracketed by events on the launching stream.  fvgpu_kernel_times reports,
 * for kernel classes {0: stage kernels, 1: dt reduction, 2: conversions},
 * the launch count and the summed milliseconds since the last reset. */
int fvgpu_profile_enable(fv_sim* sim, int enable);
int fvgpu_kernel_times(fv_sim* sim, long counts[3], double ms[3]);

/* One update (Euler or RK2 per params, with the given dt) of a problem
 * whose conserved state lives in device arrays the caller owns, allocating
 * no memory at all.  No counterpart in the reference: it exists for host
 * codes that cannot call cudaMalloc in their time loop -- applications whose
 * device memory belongs to another allocator (a pool or arena that already
 * reserved the GPU) and latency-critical loops that cannot take the device
 * synchronisation of cudaMalloc/cudaFree.  The stage scratch (U* and the
 * dt/reduction control block) is one fixed 32 MiB array per device, held
 * until the process exits.  Under lazy module loading (the CUDA default
 * since 12.2) a device holds it once the call has been used there; with
 * CUDA_MODULE_LOADING=EAGER every process that loads this library holds it
 * on each device where it creates a context.
 *   fields  device pointers to rho, rho*u, rho*v, rho*w, E of the interior
 *           cells, rows of Nx cells along x with a stride of `pitch`
 *           doubles, rows following y (Nz == 1), z (Ny == 1) or, for a
 *           3-D grid, y then z (row k*Ny + j); in 2-D the momentum along the
 *           one-cell axis may be NULL when it is zero and viscosity is off.
 *           Updated in place.  B02 conductivity and reflecting one-cell
 *           axes of 3-D grids need fvgpu_create (FV_ERR_UNSUPPORTED).
 *   pitch   row stride in doubles (>= Nx).  5 x pitch x rows x 8 bytes
 *           + 256 must fit in 32 MiB (e.g. 512 x 1536 at pitch 512); larger
 *           problems get FV_ERR_PARAM and a message -- use fvgpu_create.
 *   dt      the step, > 0 and finite (FV_ERR_PARAM otherwise): unlike
 *           fvgpu_step there is no CFL fallback for dt <= 0.
 *   next_dt if non-NULL, receives the CFL dt of the updated state; the call
 *           then waits for the stream (so it is refused, FV_ERR_PARAM, while
 *           the stream is being captured) and reports FV_ERR_NONFINITE /
 *           FV_ERR_TIMEOUT for this call or any call since the last one that
 *           passed next_dt (the device-side error flag is sticky until such
 *           a call reads and clears it).  With next_dt NULL the call returns
 *           after enqueueing its work on `stream` (NULL: the legacy default
 *           stream) and reports launch errors only.
 *   errbuf  optional buffer for a message when the status is not FV_OK.
 * All calls share the scratch and leave its last contents there: calls whose
 * work overlaps on the GPU race.  The first call on each device looks up the
 * scratch address once (with that device current); make it before any
 * stream capture. */
int fvgpu_step_noalloc(const fv_params* params, double* const fields[5], long pitch, double dt,
                       double* next_dt, void* stream, char* errbuf, size_t errlen);

/* FP64 FMA throughput of the current device in lane operations per second
 * (a full-occupancy throughput loop of independent fma chains, timed after a
 * warm-up launch).  The bit-exact FP64 kernels are bound by this rate; the
 * bench reports their FP64 roofline against it.  No reference counterpart. */
int fvgpu_probe_fp64_rate(double* lane_ops_per_s);

/* Exercises the bounded device-side wait of the TMA staging path on its own:
 * one CTA waits on an mbarrier (at most max_polls polls); with arrive != 0 the
 * barrier completes first.  FV_OK when the wait completed, FV_ERR_TIMEOUT when
 * it gave up (the kernel then returns normally and the context stays usable). */
int fvgpu_probe_wait(int arrive, int max_polls);
/* The same for the grid barrier of the multi-step batch kernel: two resident
 * CTAs meet at it, the second only when arrive_all != 0; the first waits at
 * most max_polls polls.  FV_OK when the wait completed, FV_ERR_TIMEOUT when
 * it gave up (the kernel returns normally and the context stays usable).
 * No reference counterpart. */
int fvgpu_probe_grid_wait(int arrive_all, int max_polls);

/* ---- many independent problems (no reference counterpart) --------------- */
typedef struct fv_batch fv_batch;

/* n problems, each with its own parameters (grid size, gamma, BCs ...), all
 * advanced together: one persistent kernel launch per RK stage walks a tile
 * work-queue across every problem, each problem with its own dt. */
int fvgpu_batch_create(const fv_params* params, int n, fv_batch** out);
int fvgpu_batch_destroy(fv_batch* b);
const char* fvgpu_batch_last_error(const fv_batch* b);
int fvgpu_batch_set_prim(fv_batch* b, int inst, const double* rho, const double* u,
                         const double* v, const double* w, const double* p);
int fvgpu_batch_get_prim(fv_batch* b, int inst, double* rho, double* u, double* v,
                         double* w, double* p);
/* fvgpu_init_problem for problem inst of a batch (its params.problem). */
int fvgpu_batch_init_problem(fv_batch* b, int inst);
/* Advance every problem by nsteps steps, each with its own CFL dt (the
 * fixed-step form of the main.cpp loop).  Steps are replayed from a captured
 * CUDA graph. */
int fvgpu_batch_run(fv_batch* b, long nsteps);
/* Current time of each problem (host array of n). */
int fvgpu_batch_times(fv_batch* b, double* t);
int fvgpu_batch_set_stream(fv_batch* b, void* cuda_stream);
int fvgpu_batch_synchronize(fv_batch* b);
int fvgpu_batch_launch_count(const fv_batch* b, long* count);
/* Problems sharing plane and layout form a group advanced by one persistent
 * launch per stage; reports the groups and the work-item shape the autotuner
 * chose for each: cells along x by rows along the second axis (a strip
 * segment; 3-D groups: 16 x 16 columns), tuning first if needed; every
 * problem must have a state.  The autotuner times one whole step of each
 * candidate shape (the state is saved and restored around it); FV3D_TILE=WxH
 * forces a shape, FV3D_TILE_LOG=1 prints each candidate's time to stderr. */
int fvgpu_batch_tiling(fv_batch* b, int* ngroups, int* tx, int* ty, int max_groups);
/* The full schedule the autotuner chose per group (arrays of max_groups,
 * any may be NULL): strip width tx and rows per work item (as
 * fvgpu_batch_tiling), the rows of one marched block (cells per thread in
 * the update: tx x block_rows / 256; 3-D groups: 0) and whether the viscous
 * fluxes of the face-only branches are computed once per face in a separate
 * pass (1) or fused into each cell's update (0).  The FP32-mixed kernels
 * offer 8- and 16-row blocks and both viscous forms, tuned per (grid sizes,
 * precision, group) and remembered in the tile cache; FV3D_TILE=WxH/Bv
 * forces width W, rows H, block rows B and (suffix v) the per-face form.
 * No reference counterpart. */
int fvgpu_batch_schedule(fv_batch* b, int* ngroups, int* tx, int* rows, int* block_rows, int* split_viscous,
                         int max_groups);

#ifdef __cplusplus
}
#endif
#endif /* FV3D_GB300_H */
