// e2d_impl12.cu -- the reference's alternative implementations of the FP64
// step (HydroRun::godunov_unsplit_impl, src/HydroRun.h:332-360), kept as
// debug orchestrations that reproduce them; implementation 0 (the fused
// and two-launch steps of e2d_fp64.cu) remains the production path.
//
// Implementation 1 (src/HydroRun.h:332-354): limited slopes of every cell
// stored (ComputeSlopesFunctor, src/HydroRunFunctors.h:1061-1175), then per
// direction the face states and Riemann fluxes stored
// (ComputeTraceAndFluxes_Functor, :1180-1342) and the update of that
// direction (UpdateDirFunctor, :986-1055).  Its update order -- +Fx(i)
// -Fx(i+1), then +Fy(j) -Fy(j+1) -- is implementation 0's, so its results
// are implementation 0's bit for bit (in the reference as here).
//
// Implementation 2 (src/HydroRun.h:355-360): one pass that computes both
// fluxes of a cell's left and lower faces and scatters them into the
// output state with atomic adds (ComputeFluxesAndUpdateFunctor,
// :728-980).  The order of the additions into a cell depends on thread
// scheduling, so results vary at the rounding level from run to run, as
// the reference's own do.
//
// The FP64 building blocks are those of the production step (same bits).
#include "e2d_fp64_blocks.cuh"

namespace e2d {
namespace {

constexpr int BX = 32, BY = 8;

// dt/dx, dt/dy of this step: the caller's dt, or the device loop's from the
// clock (nothing to do once t >= t_end: *run = false).
__device__ __forceinline__ void step_ratios(const KPhys<double> &ph, const DevClock *clk, int use_clock,
                                            double host_dt, double &dtdx, double &dtdy, bool &run) {
  double dt = host_dt;
  run = true;
  if (use_clock) {
    run = clk->t < clk->t_end;
    dt = step_dt(ph, clk->invdt_bits, clk->t, clk->t_end);
  }
  dtdx = dt / ph.dx;
  dtdy = dt / ph.dy;
}

__device__ __forceinline__ int st_kind_of(const KPhys<double> &ph) {
  return (ph.slope_type == 2.0) ? 2 : (ph.slope_type == 1.0) ? 1 : 0;
}

// Primitives and both slopes of cell s (row stride isize).
__device__ __forceinline__ void cell_slopes(const KGeom &g, const KPhys<double> &ph, const double *__restrict__ q,
                                            size_t s, double qc[4], double dqx[4], double dqy[4]) {
  const int st = st_kind_of(ph);
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const double *P = q + v * g.plane;
    qc[v] = P[s];
    dqx[v] = slope(st, qc[v], P[s + 1], P[s - 1]);
    dqy[v] = slope(st, qc[v], P[s + g.isize], P[s - g.isize]);
  }
}

// Face states of one cell along one direction: its minus (XMIN / YMIN) and
// plus (XMAX / YMAX) faces.
__device__ __forceinline__ void cell_faces(const KPhys<double> &ph, const double qc[4], const double dqx[4],
                                           const double dqy[4], bool xdir, double dtdx, double dtdy,
                                           double fm[4], double fp[4]) {
  double s0[4];
  trace_sources(ph, qc, dqx, dqy, s0);
#pragma unroll
  for (int v = 0; v < 4; ++v)
    face_pair(ph, v, qc[v], xdir ? dqx[v] : dqy[v], s0[v], xdir ? dtdx : dtdy, fm[v], fp[v]);
}

// Scaled flux through the face between the left/lower state ql and the
// right/upper state qr (y: normal velocity first, src/HydroRunFunctors.h:628-632).
template <int RS>
__device__ __forceinline__ void face_flux(const KPhys<double> &ph, bool xdir, const double ql[4],
                                          const double qr[4], double dtd, double f[4]) {
  if (xdir) {
    riemann<RS>(ph, ql, qr, f);
#pragma unroll
    for (int v = 0; v < 4; ++v) f[v] = f[v] * dtd;
    return;
  }
  const double l[4] = {ql[E2D_ID], ql[E2D_IP], ql[E2D_IV], ql[E2D_IU]};
  const double r[4] = {qr[E2D_ID], qr[E2D_IP], qr[E2D_IV], qr[E2D_IU]};
  double g[4];
  riemann<RS>(ph, l, r, g);
  f[E2D_ID] = g[E2D_ID] * dtd;
  f[E2D_IP] = g[E2D_IP] * dtd;
  f[E2D_IU] = g[E2D_IV] * dtd;
  f[E2D_IV] = g[E2D_IU] * dtd;
}

// --------------------------------------------------------- implementation 1
// ComputeSlopesFunctor: cells (i, j) with ghostWidth-1 <= i, j <= size-ghostWidth.
__global__ void __launch_bounds__(BX *BY)
    k_impl1_slopes(const KParams64 kp, const double *__restrict__ q, double *__restrict__ sx,
                   double *__restrict__ sy) {
  const KGeom &g = kp.g;
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i < 1 || i > g.isize - 2 || j < 1 || j > g.jsize - 2) return;
  const size_t s = (size_t)i + (size_t)g.isize * j;
  double qc[4], dqx[4], dqy[4];
  cell_slopes(g, kp.ph, q, s, qc, dqx, dqy);
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    sx[s + v * g.plane] = dqx[v];
    sy[s + v * g.plane] = dqy[v];
  }
}

// ComputeTraceAndFluxes_Functor<dir>: the flux through the left (x) or lower
// (y) face of cells ghostWidth <= i, j <= size-ghostWidth, stored at the cell.
template <int RS>
__global__ void __launch_bounds__(BX *BY)
    k_impl1_fluxes(const KParams64 kp, const int xdir, const double *__restrict__ q, const double *__restrict__ sx,
                   const double *__restrict__ sy, double *__restrict__ f, const DevClock *clk, const int use_clock,
                   const double host_dt) {
  const KGeom &g = kp.g;
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i < 2 || i > g.isize - 2 || j < 2 || j > g.jsize - 2) return;
  double dtdx, dtdy;
  bool run;
  step_ratios(kp.ph, clk, use_clock, host_dt, dtdx, dtdy, run);
  if (!run) return;
  const size_t s = (size_t)i + (size_t)g.isize * j;
  const size_t n = xdir ? s - 1 : s - g.isize;  // the left / lower neighbour
  double qc[4], dqx[4], dqy[4], qn[4], nqx[4], nqy[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    qc[v] = q[s + v * g.plane];
    dqx[v] = sx[s + v * g.plane];
    dqy[v] = sy[s + v * g.plane];
    qn[v] = q[n + v * g.plane];
    nqx[v] = sx[n + v * g.plane];
    nqy[v] = sy[n + v * g.plane];
  }
  double cm[4], cp[4], nm[4], np[4], fl[4];
  cell_faces(kp.ph, qc, dqx, dqy, xdir, dtdx, dtdy, cm, cp);   // right state: the cell's minus face
  cell_faces(kp.ph, qn, nqx, nqy, xdir, dtdx, dtdy, nm, np);   // left state: the neighbour's plus face
  face_flux<RS>(kp.ph, xdir, np, cm, xdir ? dtdx : dtdy, fl);
#pragma unroll
  for (int v = 0; v < 4; ++v) f[s + v * g.plane] = fl[v];
}

// UpdateDirFunctor<dir>: interior cells, +F(cell) -F(next cell) per variable.
__global__ void __launch_bounds__(BX *BY)
    k_impl1_update(const KParams64 kp, const int xdir, const double *__restrict__ f, double *__restrict__ u,
                   const DevClock *clk, const int use_clock) {
  const KGeom &g = kp.g;
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i < 2 || i > g.isize - 3 || j < 2 || j > g.jsize - 3) return;
  if (use_clock && !(clk->t < clk->t_end)) return;
  const size_t s = (size_t)i + (size_t)g.isize * j;
  const size_t nx = xdir ? s + 1 : s + g.isize;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    double uu = u[s + v * g.plane];
    uu = uu + f[s + v * g.plane];
    uu = uu - f[nx + v * g.plane];
    u[s + v * g.plane] = uu;
  }
}

// --------------------------------------------------------- implementation 2
// ComputeFluxesAndUpdateFunctor: cells ghostWidth <= i, j <= size-ghostWidth
// compute the fluxes of their left and lower faces and scatter them into
// the output state (which holds a copy of the input) with atomic adds.
template <int RS>
__global__ void __launch_bounds__(BX *BY)
    k_impl2_scatter(const KParams64 kp, const double *__restrict__ q, double *__restrict__ u, const DevClock *clk,
                    const int use_clock, const double host_dt) {
  const KGeom &g = kp.g;
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i < 2 || i > g.isize - 2 || j < 2 || j > g.jsize - 2) return;
  double dtdx, dtdy;
  bool run;
  step_ratios(kp.ph, clk, use_clock, host_dt, dtdx, dtdy, run);
  if (!run) return;
  const size_t s = (size_t)i + (size_t)g.isize * j;
  double qc[4], dqx[4], dqy[4];
  cell_slopes(g, kp.ph, q, s, qc, dqx, dqy);
  for (int d = 0; d < 2; ++d) {
    const bool xdir = d == 0;
    const size_t n = xdir ? s - 1 : s - g.isize;
    double qn[4], nqx[4], nqy[4], cm[4], cp[4], nm[4], np[4], fl[4];
    cell_slopes(g, kp.ph, q, n, qn, nqx, nqy);
    cell_faces(kp.ph, qc, dqx, dqy, xdir, dtdx, dtdy, cm, cp);
    cell_faces(kp.ph, qn, nqx, nqy, xdir, dtdx, dtdy, nm, np);
    face_flux<RS>(kp.ph, xdir, np, cm, xdir ? dtdx : dtdy, fl);
    // src/HydroRunFunctors.h:881-895 (x) and :957-971 (y)
    const bool own = j < g.jsize - 2 && i < g.isize - 2;
    const bool nbr = xdir ? (j < g.jsize - 2 && i > 2) : (j > 2 && i < g.isize - 2);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      if (own) atomicAdd(u + s + v * g.plane, fl[v]);
      if (nbr) atomicAdd(u + n + v * g.plane, -fl[v]);
    }
  }
}

// The loop bookkeeping of src/main.cpp:139-143 after an implementation-1/2
// step of the device loop (one thread).
__global__ void k_impl_clock(const KParams64 kp, DevClock *clk, double *__restrict__ dt_trace) {
  if (!(clk->t < clk->t_end)) return;
  const double dt = step_dt(kp.ph, clk->invdt_bits, clk->t, clk->t_end);
  const int ns = clk->nstep;
  const int slot = ns - clk->trace_base;
  if (dt_trace && slot >= 0 && slot < clk->trace_cap) dt_trace[slot] = dt;
  if (!(dt > 0.0) || nonfinite(dt)) clk->status |= E2D_FLAG_BAD_DT;
  clk->dt = dt;
  clk->t = clk->t + dt;
  clk->nstep = ns + 1;
  clk->invdt_bits = 0ull;
}

template <int RS>
cudaError_t impl_kernels(const KParams64 &kp, int impl, const double *q, double *u_out, double *scratch,
                         DevClock *clk, int use_clock, double host_dt, double *dt_trace, cudaStream_t s) {
  const dim3 block(BX, BY), grid((kp.g.isize + BX - 1) / BX, (kp.g.jsize + BY - 1) / BY);
  if (impl == 2) {
    k_impl2_scatter<RS><<<grid, block, 0, s>>>(kp, q, u_out, clk, use_clock, host_dt);
  } else {
    double *sx = scratch, *sy = scratch + 4 * kp.g.plane, *f = scratch + 8 * kp.g.plane;
    k_impl1_slopes<<<grid, block, 0, s>>>(kp, q, sx, sy);
    for (int xdir = 1; xdir >= 0; --xdir) {
      k_impl1_fluxes<RS><<<grid, block, 0, s>>>(kp, xdir, q, sx, sy, f, clk, use_clock, host_dt);
      k_impl1_update<<<grid, block, 0, s>>>(kp, xdir, f, u_out, clk, use_clock);
    }
  }
  if (use_clock) k_impl_clock<<<1, 1, 0, s>>>(kp, clk, dt_trace);
  return cudaGetLastError();
}

}  // namespace

size_t impl12_scratch_doubles(const KParams64 &kp, int impl) {
  return impl == 1 ? (size_t)12 * kp.g.plane : 0;
}

cudaError_t launch_impl12_f64(const KParams64 &kp, int impl, int riemann, const double *q, double *u_out,
                              double *scratch, DevClock *clk, int use_clock, double host_dt, double *dt_trace,
                              cudaStream_t s) {
  switch (riemann) {
    case E2D_RIEMANN_HLLC: return impl_kernels<E2D_RIEMANN_HLLC>(kp, impl, q, u_out, scratch, clk, use_clock, host_dt, dt_trace, s);
    case E2D_RIEMANN_HLL: return impl_kernels<E2D_RIEMANN_HLL>(kp, impl, q, u_out, scratch, clk, use_clock, host_dt, dt_trace, s);
    default: return impl_kernels<E2D_RIEMANN_APPROX>(kp, impl, q, u_out, scratch, clk, use_clock, host_dt, dt_trace, s);
  }
}

}  // namespace e2d
