/*
 * e2d.h -- C ABI of the GB300-native unsplit MUSCL-Hancock Godunov step.
 *
 * Drop-in for the hot path of euler2d_kokkos: the class template
 * euler2d::HydroRun<device_t> (src/HydroRun.h:44-134) with its
 * compute_dt / godunov_unsplit / make_boundaries methods, the HydroParams
 * parameter contract (src/HydroParams.h:107-265) and the ConfigMap ini reader
 * (config/ConfigMap.h:25-47).  The reference has no FFI: these entry points
 * are what a C, ctypes, cgo or JNI binding of that class would call.  Each
 * declaration names the reference interface it replaces.
 *
 * Conventions
 *  - Every function returns an e2d_status (0 = E2D_OK).  Failures never abort
 *    the process; e2d_last_error() gives the message of the last failure on a
 *    handle.
 *  - Device memory is owned by the handle.  Host buffers belong to the caller.
 *  - A handle is used from one host thread; its work runs on its own CUDA
 *    stream (e2d_get_stream).
 *  - State arrays hold (rho, E, rho*u, rho*v) for isize*jsize cells, ghosts
 *    included, in the reference's DataArray layout on its CUDA backend
 *    (LayoutLeft: element (i, j, v) at i + isize*(j + jsize*v)).  Host copies
 *    may also use the OpenMP backend's LayoutRight ((i*jsize + j)*4 + v).
 */
#ifndef E2D_H_
#define E2D_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define E2D_ABI_VERSION 2

typedef enum e2d_status {
  E2D_OK = 0,
  E2D_EINVAL = 1,   /* bad argument or parameter                        */
  E2D_ENOMEM = 2,   /* device or host allocation failed                 */
  E2D_ENUMERIC = 3, /* device saw NaN/Inf, rho <= 0, p <= 0 or dt <= 0  */
  E2D_ETIMEOUT = 4, /* a bounded device wait gave up                    */
  E2D_ECUDA = 5,    /* a CUDA runtime call failed                       */
  E2D_EIO = 6       /* ini file missing or unreadable                   */
} e2d_status;

/* Values of src/HydroParams.h:26-102 (ComponentIndex, RiemannSolverType,
 * BoundaryConditionType, ProblemType). */
enum { E2D_ID = 0, E2D_IP = 1, E2D_IE = 1, E2D_IU = 2, E2D_IV = 3 };
enum { E2D_RIEMANN_APPROX = 0, E2D_RIEMANN_HLL = 1, E2D_RIEMANN_HLLC = 2 };
enum { E2D_BC_REFLECT = 1, E2D_BC_ABSORB = 2, E2D_BC_PERIODIC = 3 };
enum {
  E2D_PROBLEM_IMPLODE = 0,
  E2D_PROBLEM_BLAST = 1,
  E2D_PROBLEM_FOUR_QUADRANT = 2,
  E2D_PROBLEM_DISCONTINUITY = 3,
  E2D_PROBLEM_SHOCKED_BUBBLE = 4
};
enum { E2D_LAYOUT_LEFT = 0, E2D_LAYOUT_RIGHT = 1 };
/* Arithmetic of the step: FP64 (bit-identical to the reference), FP32 with
 * a compensated hi/lo conservative update, or FP64 "fast" (opt-in: FMAs and
 * shared Newton-refined reciprocals in the step; within 1e-12 of the
 * reference on dt and 1e-10 relative L1 in the tests, not bit-identical;
 * e2d_step_n only -- e2d_godunov_unsplit, batches and the allocation-free
 * entry point refuse it with E2D_EINVAL). */
enum { E2D_PRECISION_FP64 = 0, E2D_PRECISION_FP32C = 1, E2D_PRECISION_FP64_FAST = 2 };

/* Flat mirror of HydroParams + HydroSettings (src/HydroParams.h:107-265).
 * Fill it with e2d_params_from_ini (the reference's ini semantics, reals
 * rounded to float as ConfigMap::getFloat does) or e2d_params_defaults, then
 * call e2d_params_init for the derived members. */
typedef struct e2d_params {
  /* [run] */
  int nStepmax;
  double tEnd;
  int nOutput;
  int enableOutput; /* 0 when nOutput == -1 */
  int ioVTK, ioHDF5;
  /* [mesh] */
  int nx, ny, ghostWidth;
  double xmin, xmax, ymin, ymax;
  int boundary_type_xmin, boundary_type_xmax, boundary_type_ymin, boundary_type_ymax;
  /* [hydro] */
  double gamma0, cfl, slope_type, smallr, smallc;
  int niter_riemann;
  int riemannSolverType;
  int problemType;
  /* [blast] */
  double blast_radius, blast_center_x, blast_center_y;
  double blast_density_in, blast_density_out, blast_pressure_in, blast_pressure_out;
  double blast_total_energy_inside;
  int blast_nbins;
  /* [shocked_bubble] */
  double bubble_radius, bubble_center_x, bubble_center_y, bubble_density, bubble_pressure;
  double preshock_density, preshock_pressure, postshock_density, postshock_pressure;
  double postshock_velocity, shock_loc;
  /* [four_quadrant] split point (the reference hard-codes 0.8, 0.8) and the
   * primitive state (rho, p, u, v) of quadrants 0 (x >= split_x, y >=
   * split_y), 1 (x < split_x, y >= split_y), 2 (both below), 3 (x >=
   * split_x, y < split_y); defaults: the reference's Lax-Liu case 3
   * (src/HydroRunFunctors.h:1607-1622), ini keys rho_q, p_q, u_q, v_q */
  double fq_split_x, fq_split_y;
  double fq_state[4][4];
  /* [implode] shape: 0 = the reference's x + y*y in (0.5, 1.5) band,
   * 1 = the classic diagonal split x + y > 0.5 */
  int implode_shape;
  /* [OTHER] implementationVersion: 0, 1 or 2 all run the fused step */
  int implementationVersion;
  /* GB300 build: arithmetic mode */
  int precision;
  /* derived by e2d_params_init (HydroParams::init, src/HydroParams.cpp:160-190) */
  int imin, imax, jmin, jmax, isize, jsize;
  double dx, dy, smallp, smallpp, gamma6;
} e2d_params;

typedef struct e2d_sim e2d_sim;

/* ABI version compiled into the library (E2D_ABI_VERSION). */
int e2d_abi_version(void);
/* Human-readable name of a status code. */
const char *e2d_status_string(int status);

/* Defaults of HydroParams::setup (src/HydroParams.cpp:42-156). */
int e2d_params_defaults(e2d_params *p);
/* ConfigMap(path) + HydroParams::setup (config/ConfigMap.cpp:21-40,
 * src/HydroParams.cpp:42-156): case-insensitive keys, reals via strtof. */
int e2d_params_from_ini(const char *path, e2d_params *p);
/* HydroParams::init (src/HydroParams.cpp:160-190); validates the values. */
int e2d_params_init(e2d_params *p);
/* ConfigMap::getString (config/inih/INIReader.cpp:36-42) on an ini file:
 * the value of section.name (case-insensitive) or dflt, copied with a
 * terminating NUL into buf (truncated to buflen - 1 bytes). */
int e2d_ini_get_string(const char *path, const char *section, const char *name, const char *dflt,
                       char *buf, size_t buflen);

/* HydroRun<device>::HydroRun (src/HydroRun.h:143-216) without the initial
 * condition: allocates U and U2 on the device (zeroed). */
int e2d_create(const e2d_params *p, e2d_sim **out);
/* ~HydroRun: frees every device buffer of the handle. */
int e2d_destroy(e2d_sim *sim);
/* Last failure message on this handle ("" if none). */
const char *e2d_last_error(const e2d_sim *sim);
/* The copy of the parameters the handle runs with. */
int e2d_get_params(const e2d_sim *sim, e2d_params *p);

/* The initial condition of HydroRun's constructor (src/HydroRun.h:185-214,
 * InitXxxFunctor in src/HydroRunFunctors.h:1347-1827) into U, then U2 = U. */
int e2d_init_problem(e2d_sim *sim);
/* Host -> device copy of a whole state (which = 0: U, 1: U2). */
int e2d_set_state(e2d_sim *sim, int which, const double *host, int layout);
/* Device -> host copy of a whole state (which = 0: U, 1: U2); synchronises. */
int e2d_get_state(e2d_sim *sim, int which, double *host, int layout);
/* HydroRun::saveVTK (src/HydroRun.h:506-609): device -> host copy of U (0)
 * or U2 (1) and an ASCII VTK ImageData (.vti) file of the interior cells,
 * variables rho, E, mx, my in the reference's text format. */
int e2d_save_vtk(e2d_sim *sim, int which, const char *filename);
/* The text writer of HydroRun::saveVTK (src/HydroRun.h:546-607) for a state
 * already on the host: p->nx x p->ny interior cells of `host` (LayoutLeft or
 * LayoutRight FP64, ghosts included) into `filename`.  No device work. */
int e2d_write_vtk(const e2d_params *p, const double *host, int layout, const char *filename);
/* Device address of U (which = 0) or U2 (1), LayoutLeft FP64, for zero-copy
 * use.  FP32C handles return a converted copy (hi + lo, ghosts filled) in a
 * staging array that the next call on the handle may overwrite. */
int e2d_device_state(e2d_sim *sim, int which, double **dptr);
/* Conservation audit: FP64 sums over the interior cells of rho, E, mx, my of
 * U (0) or U2 (1); deterministic summation order. */
int e2d_conservation(e2d_sim *sim, int which, double sums[4]);
/* L1 difference of variable var between state wa of a and state wb of b
 * (same grid): *l1_diff = sum |a - b|, *l1_ref = sum |b| over the interior,
 * accumulated in FP64 on the device of a. */
int e2d_l1_diff(e2d_sim *a, int wa, e2d_sim *b, int wb, int var, double *l1_diff, double *l1_ref);
/* The handle's CUDA stream (a cudaStream_t). */
int e2d_get_stream(e2d_sim *sim, void **stream);

/* Sedov post-processing, ComputeRadialProfileFunctor::apply
 * (src/ComputeRadialProfileFunctor.h:83-134, called from src/main.cpp:175-179):
 * the mean density of U (0) or U2 (1) in nbins rings about the box centre,
 * over every cell of the array including ghosts (nbins <= 0: the
 * [blast] nbins key).  distances[b] = (b + 0.5) * rmax / nbins with rmax the
 * half-diagonal of the box; counts may be NULL.  Differences from the
 * reference: cells whose ring index is >= nbins (the ghost corners) are not
 * counted, where the reference writes them past the end of its histogram
 * arrays; the per-ring sums are exact up to one final rounding (the
 * reference's atomic FP64 sums depend on the order of the additions); a
 * non-finite density returns E2D_ENUMERIC.  An empty ring gives NaN (0/0),
 * as in the reference. */
int e2d_radial_profile(e2d_sim *sim, int which, int nbins, double *distances, double *profile,
                       long long *counts);
/* cnpy::npy_save (src/cnpy/cnpy.h:130-187, header of :343-378) for a 1-D
 * double array: NPY format 1.0, descr '<f8' (host byte order), C order. */
int e2d_save_npy(const char *path, const double *data, long long n);

/* HydroRun::make_boundaries (src/HydroRun.h:388-399) on U (0) or U2 (1).
 * FP32C states keep no ghost cells (readers map them), so there it does
 * nothing. */
int e2d_make_boundaries(e2d_sim *sim, int which);
/* HydroRun::compute_dt (src/HydroRun.h:227-251): cfl / max wave speed of U
 * (useU == 0) or U2; blocks until the value is on the host. */
int e2d_compute_dt(e2d_sim *sim, int useU, double *dt);
/* HydroRun::godunov_unsplit (src/HydroRun.h:258-272): U -> U2 for even
 * nStep, U2 -> U for odd, with the caller's dt.  Asynchronous. */
int e2d_godunov_unsplit(e2d_sim *sim, int nStep, double dt);

/* One FP64 godunov_unsplit step (same kernels and bits as
 * e2d_godunov_unsplit) on device buffers the caller owns, allocating no
 * memory at all.  No counterpart in the reference: it exists for callers
 * that cannot let a library call cudaMalloc -- hosts that give out all
 * device memory from their own fixed pool, latency-critical loops that
 * cannot afford cudaMalloc's implicit device synchronisation, and code that
 * keeps no handle between calls.
 *   u_in, u_out: distinct device arrays of 4*isize*jsize doubles (LayoutLeft);
 *   like the reference, the ghost cells of u_in are filled in place and u_out
 *   receives the whole new state.  stream: a cudaStream_t, or NULL.  The call
 *   is asynchronous on that stream.
 * Scratch (primitives and loop state) lives in one file-scope device array
 * sized for E2D_NOALLOC_MAX_CELLS cells (isize*jsize, ghosts included):
 * larger grids are refused with E2D_EINVAL.  Each GPU that loads the library
 * holds that array (about 8.4 MB) until the process exits.  The first call
 * on a device looks up the array's device address (and sets the kernels'
 * shared-memory limit) with that device current; make that first call
 * before any stream capture.  All calls on a device share the one array, so
 * calls that overlap on the GPU (different streams, or host threads without
 * ordering) race with each other; serialise them.  The address and the limit
 * are kept for the life of the process: calls after cudaDeviceReset (or any
 * other teardown of the device's primary context) are not supported.  FP64
 * precision only. */
#define E2D_NOALLOC_MAX_CELLS (1 << 18)
int e2d_godunov_unsplit_noalloc(const e2d_params *p, double *u_in, double *u_out, double dt,
                                void *stream);

/* The time loop of src/main.cpp:100-145 for up to n steps on the device:
 * each step takes dt = cfl/max wave speed of the current state, clamps it to
 * t_end - t, runs godunov_unsplit and advances (t, nStep); steps with
 * t >= t_end do nothing.  *t and *nStep are read and updated.  dt_trace
 * (optional, n entries) receives the dt of each step taken.  FP64: one
 * prologue kernel (primitives and CFL maximum of the input state), then one
 * fused kernel per step whose epilogue folds the next step's CFL maximum;
 * launches are replayed from cached CUDA graphs.  Blocks until done.
 * E2D_ENUMERIC: a step saw a non-finite state or dt; E2D_ETIMEOUT: a bounded
 * wait for a TMA copy (FP64 tile staging, FP32C row staging of the TMA
 * variant) gave up (the state of this call is incomplete; the handle stays
 * usable). */
int e2d_step_n(e2d_sim *sim, int n, double t_end, double *t, int *nStep, double *dt_trace);

/* ---------------------------------------------------------------------------
 * Batched solves.  No counterpart in the reference, which runs one grid per
 * process: the serving mode here keeps many independent simulations of
 * uneven size resident in one device memory pool and advances all active
 * ones together, one persistent kernel launch per iteration for the FP32C
 * instances and one for the FP64 ones (the fused step over a tile
 * work-list; each instance with its own dt and t_end), replayed from CUDA
 * graphs.  Arithmetic: each instance's
 * params.precision (FP64 instances end bit for bit where the single FP64
 * path ends).  One Riemann solver per batch.  A handle is used from one host
 * thread.
 * ------------------------------------------------------------------------- */
typedef struct e2d_batch e2d_batch;
/* A batch with a device pool of pool_bytes and room for max_instances. */
int e2d_batch_create(int riemann, size_t pool_bytes, int max_instances, e2d_batch **out);
int e2d_batch_destroy(e2d_batch *b);
const char *e2d_batch_last_error(const e2d_batch *b);
/* Pool bytes an instance with these parameters needs to be admitted. */
size_t e2d_batch_instance_bytes(const e2d_params *p);
int e2d_batch_free_bytes(const e2d_batch *b, size_t *free_bytes, size_t *largest_block);
/* Admit one solve: its initial condition is u0 (host, LayoutLeft FP64, whole
 * array) or, if u0 is NULL, params->problemType's; it runs until t_end.
 * E2D_ENOMEM when the pool or the instance table has no room. */
int e2d_batch_admit(e2d_batch *b, const e2d_params *p, double t_end, const double *u0, int *id);
/* Advance every active instance by up to `iterations` steps; *n_active
 * receives the number of instances still short of their t_end. */
int e2d_batch_run(e2d_batch *b, int iterations, int *n_active);
/* Loop state of an instance as of the last run (t, steps, still active).
 * The outputs are filled in every case; the status is E2D_ENUMERIC or
 * E2D_ETIMEOUT for an instance the batch stopped (a non-finite state or dt;
 * a row-staging wait that gave up), which stays inactive. */
int e2d_batch_query(e2d_batch *b, int id, double *t, int *nstep, int *active);
/* Current state of an instance (hi + lo in FP64, ghosts filled), host copy. */
int e2d_batch_get_state(e2d_batch *b, int id, double *host, int layout);
/* Free an instance's pool bytes and slot. */
int e2d_batch_release(e2d_batch *b, int id);
/* Interior cell-updates done by run calls so far; instances in the pool. */
int e2d_batch_stats(e2d_batch *b, long long *cell_updates, int *n_instances);
/* The batch's CUDA stream (a cudaStream_t). */
int e2d_batch_stream(e2d_batch *b, void **stream);
/* Tuning: variant of the batch kernel (0..3: at least 1, 4, 3 or 2 resident
 * blocks of 128 threads per SM with rows loaded to registers; 4, 5: 3 or 4
 * blocks with rows staged through shared memory by cp.async; 6: 4 blocks,
 * rows staged by TMA copies waited on with mbarriers) and rows per strip (16..512,
 * rounded up to a multiple of 16) for the size classes max(nx, ny) <= 192,
 * <= 512, > 512.  Results do not depend on them.  e2d_batch_autotune times the staged variants (4, 5,
 * 6) and then 16, 32 and 64 rows per size class on the live batch (its iterations advance the
 * instances) and keeps the fastest. */
int e2d_batch_set_tuning(e2d_batch *b, int variant, const int strip_h[3]);
int e2d_batch_get_tuning(const e2d_batch *b, int *variant, int strip_h[3]);
int e2d_batch_autotune(e2d_batch *b, int iters_per_trial);

/* Building blocks of the FP64 step evaluated on the device, n independent
 * inputs each (host arrays; the per-function known-answer interface of the
 * reference's HydroBaseFunctor, src/HydroBaseFunctor.h):
 *   E2D_EVAL_PRIMITIVES   in 4/item (rho,E,mx,my)        out 5 (rho,p,u,v,c)
 *                         -- computePrimitives, :76-102
 *   E2D_EVAL_SLOPES       in 20/item (q,q+x,q-x,q+y,q-y) out 8 (dqx, dqy)
 *                         -- slope_unsplit_hydro_2d, :475-516
 *   E2D_EVAL_TRACE_*      in 12/item (q, dqx, dqy)       out 4 (face state)
 *                         -- trace_unsplit_2d_along_dir, :214-291
 *   E2D_EVAL_RIEMANN_*    in 8/item (qleft, qright)      out 4 (flux)
 *                         -- riemann_approx :558-693, riemann_hllc :704-809,
 *                            and the HLL flux (Toro eq. 10.21) added here.
 * dtdx / dtdy are used by the trace only. */
enum {
  E2D_EVAL_PRIMITIVES = 0,
  E2D_EVAL_SLOPES = 1,
  E2D_EVAL_TRACE_XMIN = 2,
  E2D_EVAL_TRACE_XMAX = 3,
  E2D_EVAL_TRACE_YMIN = 4,
  E2D_EVAL_TRACE_YMAX = 5,
  E2D_EVAL_RIEMANN_APPROX = 6,
  E2D_EVAL_RIEMANN_HLL = 7,
  E2D_EVAL_RIEMANN_HLLC = 8
};
int e2d_eval_device(const e2d_params *p, int what, int n, const double *in, double *out, double dtdx,
                    double dtdy);

/* Measured throughput of this GPU's FP64 operations in G operations/s:
 * rates[0..5] = fused multiply-add, add, multiply, divide, square root,
 * maximum (8 independent chains per thread, 8 blocks of 256 threads per SM,
 * CUDA events).  No counterpart in the reference: it is the denominator of
 * the FP64-pipe roofline that bounds the FP64 step on GB300. */
int e2d_fp64_rates(double rates[6]);

/* Per-kernel device time: with profiling on, e2d_step_n launches kernels
 * directly with CUDA events around each one.  names/ms/launches receive, per
 * kernel, its name, total milliseconds and launch count. */
int e2d_set_profiling(e2d_sim *sim, int on);
int e2d_kernel_times(e2d_sim *sim, int max_kernels, const char **names, double *ms, long *launches,
                     int *n_kernels);
int e2d_reset_kernel_times(e2d_sim *sim);

#ifdef __cplusplus
}
#endif
#endif /* E2D_H_ */
