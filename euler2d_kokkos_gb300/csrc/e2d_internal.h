// e2d_internal.h -- shared declarations of the GB300 euler2d library:
// the ini reader, the parameter helpers, the device-side parameter blocks,
// the device clock and the kernel launchers of each arithmetic mode.
#pragma once

#include <map>
#include <string>

#include <cuda.h>  // CUtensorMap (the map is encoded through the runtime's driver entry point)
#include <cuda_runtime.h>

#include "../../include/e2d.h"

namespace e2d {

// ---------------------------------------------------------------- host side
class IniMap {
 public:
  // 0 on success, -1 if the file cannot be opened, else the first bad line.
  int parse(const char *path);
  std::string get_string(const std::string &section, const std::string &name,
                         const std::string &dflt) const;
  long get_integer(const std::string &section, const std::string &name, long dflt) const;
  float get_float(const std::string &section, const std::string &name, float dflt) const;
  bool get_bool(const std::string &section, const std::string &name, bool dflt) const;

 private:
  std::map<std::string, std::string> values_;
};

void params_defaults(e2d_params *p);
int params_from_ini(const IniMap &m, e2d_params *p, std::string *msg);
int params_init(e2d_params *p, std::string *msg);

// ---------------------------------------------------------------- device side
// Grid geometry as every kernel sees it.
struct KGeom {
  int nx, ny, isize, jsize;
  long long plane;  // isize * jsize: stride between the 4 variable planes
  int bc_xmin, bc_xmax, bc_ymin, bc_ymax;
};

// Physics constants in the step's arithmetic type.  gm1, entho and smallc2
// are computed on the host with the same operations the reference performs
// inline (gamma0 - 1.0, 1.0 / (gamma0 - 1.0), smallc * smallc), so using them
// changes no bit of the result.
template <typename R>
struct KPhys {
  R gamma0, gamma6, cfl, slope_type, smallr, smallc, smallp, smallpp;
  R gm1, entho, smallc2;
  R dx, dy;
  // 1/dx, 1/dy when dx, dy are powers of two (then x / dx == x * (1/dx) bit
  // for bit: both round the same exact value), else 0
  R inv_dx_pow2, inv_dy_pow2;
  R inv_dx, inv_dy;  // 1/dx, 1/dy rounded (E2D_PRECISION_FP64_FAST only)
};

struct KParams64 {
  KGeom g;
  KPhys<double> ph;
  int tile;       // tile shape: -1 the default (32 x 32), else see launch_step_f64 and
                  // launch_flux_update_f64
  int fast;       // E2D_PRECISION_FP64_FAST: the fused step's fast forms (not bit-identical)
  int wait_test;  // nonzero: tile (1, 1) of the fused step never stages its primitives,
                  // so its bounded wait runs out (E2D_TEST_WAIT_TIMEOUT=1; tests the timeout path)
};

// FP32 step with FP64 copies of the constants the exact dt recompute uses.
// FP32C state arrays use a row pitch `wpitch` (isize rounded up to a
// multiple of 4 floats) so every row starts on a 16-byte boundary.
struct KParams32 {
  KGeom g;
  KPhys<float> ph;
  KPhys<double> ph64;
  int wpitch;
  long long wplane;  // wpitch * jsize
  int variant;       // step kernel register-budget variant (see launch_f32c_step)
  int strip_h;       // rows per warp strip of the step kernel
  int wait_test;     // nonzero: strip (1, 0) never stages its first row, so its bounded
                     // wait runs out (E2D_TEST_WAIT_TIMEOUT=1; tests the timeout path)
};
int default_strip_h(int nx, int ny);

// Device-resident loop state of the time loop of src/main.cpp:100-145.
struct DevClock {
  double t;                       // simulated time
  double t_end;                   // loop ends once t >= t_end
  double dt;                      // dt of the last step taken
  unsigned long long invdt_bits;  // running max of the CFL wave-speed term (bits of a double >= 0)
  int nstep;                      // steps taken since the start of the run
  int trace_base;                 // nstep of the first entry of the dt trace buffer
  int trace_cap;                  // entries available in the dt trace buffer
  unsigned int done_blocks;       // blocks of the current step kernel that finished
  unsigned int status;            // E2D_FLAG_* bits seen by the device
  unsigned int fill_count;        // blocks of the current primitives kernel that finished
  // FP32 path and the fused FP64 step: the step of parity n reads the CFL
  // maximum of its input from acc[n & 1] and folds that of its output into
  // acc[(n + 1) & 1]
  unsigned long long acc[2];
  double *trace;  // FP32 path: device dt trace (trace_cap entries) or null
};

enum : unsigned int {
  E2D_FLAG_NONFINITE = 1u,  // a state value is NaN or Inf
  E2D_FLAG_DENSITY = 2u,    // a density <= 0 was clamped to smallr
  E2D_FLAG_BAD_DT = 4u,     // the CFL wave-speed maximum is not a finite positive number
  E2D_FLAG_TIMEOUT = 8u,    // a bounded device wait (row or tile staging) gave up; that strip or tile
                            // is not updated
};

// Modes of the primitives kernel.
enum : int {
  FILL_WRITE_Q = 1,          // store primitives of every cell
  FILL_GHOSTS_IN = 2,        // store the ghost fill into the input state (make_boundaries)
  FILL_GHOSTS_OUT = 4,       // store the ghost fill into the output state (deep_copy)
  FILL_DT = 8,               // fold the CFL term of interior cells into clock->invdt_bits (or acc[slot])
  FILL_DEVICE_CLOCK = 16,    // do nothing once clock->t >= clock->t_end
  FILL_COPY_OUT = 32,        // copy the whole ghost-filled input state into the output (deep_copy)
};

// FP64 kernels (e2d_fp64.cu, bit-identical to the reference).
// acc_slot < 0: FILL_DT folds into clk->invdt_bits, else into clk->acc[acc_slot & 1].
cudaError_t launch_fill_f64(const KParams64 &kp, double *u_in, double *u_out, double *q,
                            DevClock *clk, int mode, cudaStream_t s, int acc_slot = -1);
// One fused step of the device time loop: reads u_in and q_in (primitives of
// u_in's interior, tm_q its TMA map when use_tma) and clk->acc[nstep & 1];
// writes u_out, the ghost cells of both states, q_out and clk->acc[(nstep+1) & 1].
cudaError_t launch_step_f64(const KParams64 &kp, int riemann, const CUtensorMap &tm_q, int use_tma,
                            const double *q_in, double *q_out, double *u_in, double *u_out, DevClock *clk,
                            double *dt_trace, cudaStream_t s);
// The reference's implementations 1 and 2 of the step (e2d_impl12.cu), after
// a fill with FILL_WRITE_Q | FILL_GHOSTS_IN | FILL_COPY_OUT (and FILL_DT |
// FILL_DEVICE_CLOCK in the device loop, use_clock = 1); implementation 1 needs
// impl12_scratch_doubles(kp, 1) doubles of scratch.
size_t impl12_scratch_doubles(const KParams64 &kp, int impl);
cudaError_t launch_impl12_f64(const KParams64 &kp, int impl, int riemann, const double *q, double *u_out,
                              double *scratch, DevClock *clk, int use_clock, double host_dt, double *dt_trace,
                              cudaStream_t s);
// TMA map of a primitives array for the fused step's tile shape; false if
// isize is odd or the driver cannot encode it (tiles are gathered then).
bool encode_q_map(CUtensorMap *map, const double *q, const KParams64 &kp);
// use_clock = 1: dt from clk (src/main.cpp:128-134 on the device) and the
// loop bookkeeping; 0: the caller's host_dt, clock untouched.
cudaError_t launch_flux_update_f64(const KParams64 &kp, int riemann, const double *q,
                                   const double *u_in, double *u_out, DevClock *clk,
                                   int use_clock, double host_dt, double *dt_trace,
                                   cudaStream_t s);
// Sets the kernels' shared-memory limits; call once per device before any
// launch or graph capture.
cudaError_t configure_f64_kernels();
cudaError_t launch_init_f64(const KParams64 &kp, const e2d_params &p, double *u, cudaStream_t s);
cudaError_t launch_eval_f64(const KParams64 &kp, int what, int n, const double *in, double *out,
                            double dtdx, double dtdy, cudaStream_t s);
void make_kparams(const e2d_params &p, KParams64 *kp);
void make_kparams32(const e2d_params &p, KParams32 *kp);

// FP32 path with compensated (hi, lo) state (e2d_fp32c.cu).  A state is 8
// float planes of isize*jsize: hi(rho, E, mx, my) then lo(rho, E, mx, my).
// Ghost cells of these arrays are not maintained: the step reads ghosts
// through the boundary map.
cudaError_t configure_f32c_kernels();
// FP32C step / batch kernel variants (register budget x row staging), see
// with_variant in e2d_fp32c.cu.
constexpr int kF32cVariants = 7;
cudaError_t launch_f32c_from_f64(const KParams32 &kp, const double *u, float *w, cudaStream_t s);
cudaError_t launch_f32c_to_f64(const KParams32 &kp, const float *w, double *u, cudaStream_t s);
// CFL maximum of a state (interior) into clk->acc[slot] (slot < 0: invdt_bits).
cudaError_t launch_f32c_dt(const KParams32 &kp, const float *w, DevClock *clk, int slot, cudaStream_t s);
cudaError_t launch_f32c_dt_to(const KParams32 &kp, const float *w, unsigned long long *target,
                              unsigned int *status, cudaStream_t s);
// TMA map of an FP32C state array (8 planes of wpitch x jsize floats) with a
// box of one row: 64 columns x 1 row x 8 planes, the row ring's slot.
// Returns false if the driver cannot encode it.
bool encode_f32c_map(CUtensorMap *map, const float *w, const KParams32 &kp);
// One FP32C step; tm_in: the map of w_in.
cudaError_t launch_f32c_step(const KParams32 &kp, int riemann, const float *w_in, float *w_out,
                             const CUtensorMap &tm_in, DevClock *clk, int use_clock, double host_dt,
                             cudaStream_t s);

// ---------------------------------------------------------------- batches
// One instance of a batch (device table entry): its grid, its two
// compensated states and its own time loop.  The loop state is advanced by
// the last strip of the instance to finish each iteration.
struct BatchInst {
  CUtensorMap tm[2];  // TMA maps of w[0], w[1] (64-byte aligned: first member)
  KParams32 kp;
  float *w[2];
  double t, t_end, dt;          // dt: of the pending step
  unsigned long long acc[2];    // CFL maxima by step parity
  int par;                      // w[par] holds the current state
  int active;                   // 1 while t < t_end
  int nstep;
  int nsx, nstrips;             // strips of the step kernel
  float dtdx, dtdy;             // of the pending step
  unsigned int done;            // strips finished in the current iteration
  unsigned int status;          // E2D_FLAG_* bits
};

// An FP64 instance of a batch: the reference's two states and the
// primitives of each in the pool, stepped by the fused step
// (k_batch_step_f64) after one prologue at admission (k_batch_prime_f64).
struct BatchInst64 {
  KParams64 kp;
  double *u[2];
  double *q[2];                  // q[par]: primitives of u[par] (interior cells)
  double t, t_end, dt;           // dt: of the last step taken
  unsigned long long acc[2];     // CFL maxima by step parity (the step of parity n reads acc[n & 1])
  int par;                       // u[par] holds the current state
  int active;                    // 1 while t < t_end
  int nstep;
  int nbx, nfill;                // prologue blocks per row, total
  int ntx, ntiles;               // 32 x 32 tiles per row, total
  unsigned int done;             // tiles finished in the current iteration
  unsigned int status;           // E2D_FLAG_* bits
};

// The prologue of a newly admitted FP64 instance (q[0], acc[0] from u[0]).
cudaError_t launch_batch_prime_f64(BatchInst64 *inst, int nfill, cudaStream_t s);
// One FP64 iteration of every listed FP64 instance in one persistent launch
// of at most grid_blocks blocks: list entry k is table slot list_slots[k];
// tile_begin[k] is its first global tile (n_inst + 1 entries, the last =
// total_tiles).
cudaError_t launch_batch_f64(int riemann, BatchInst64 *insts, const int *list_slots, const int *tile_begin,
                             int n_inst, int total_tiles, int grid_blocks, cudaStream_t s);
// Fill blocks and flux tiles of an FP64 instance.
void batch_f64_shape(const KParams64 &kp, int *nbx, int *nfill, int *ntx, int *ntiles);

// One iteration over every strip of every listed instance: list entry k is
// table slot list_slots[k]; strip_begin[k] is its first global strip
// (n_inst + 1 entries, the last = total_strips).
cudaError_t launch_batch_f32c(int riemann, int variant, BatchInst *insts, const int *list_slots,
                              const int *strip_begin, int n_inst, int total_strips, int grid_blocks,
                              cudaStream_t s);
// dt, dt/dx, dt/dy and `active` of an instance from acc[nstep & 1].
cudaError_t launch_batch_arm(BatchInst *inst, cudaStream_t s);
// Resident blocks per SM of the batch kernel variant (occupancy).
int batch_blocks_per_sm(int riemann, int variant);
int strips_of(const KParams32 &kp);

// FP64 reductions over the interior (e2d_reduce.cu): per-variable sums and
// the L1 difference of two states, deterministic (fixed summation tree).
// `partial` holds at least reduce_partial_count(p) doubles.
size_t reduce_partial_count(const KGeom &g);
cudaError_t launch_sums_f64(const KGeom &g, const double *u, double *partial, double *out4, cudaStream_t s);
cudaError_t launch_l1diff_f64(const KGeom &g, const double *a, const double *b, int var,
                              double *partial, double *out2, cudaStream_t s);

// Radial density profile about the box centre (e2d_reduce.cu), over every
// cell of the array including ghosts; rings >= nbins are not counted.
struct ProfileGeom {
  double xmin, ymin, dx, dy, cx, cy, rmax;
  int isize, jsize, ghost, nbins;
};
constexpr int kProfileSmemRings = 4096;  // per-block shared-memory partials up to this many rings
// scratch: 1 + 4*nbins 64-bit words; flags bit 0: a non-finite density.
cudaError_t launch_radial_profile(const ProfileGeom &g, const double *rho, unsigned long long *scratch,
                                  unsigned int *flags, cudaStream_t s);
// Mean density per ring from the scratch words copied to the host.
void finish_radial_profile(const ProfileGeom &g, const unsigned long long *host_scratch, double *profile,
                           long long *counts);

}  // namespace e2d
