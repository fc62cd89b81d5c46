// e2d_fp64.cu -- FP64 kernels of the unsplit MUSCL-Hancock Godunov step,
// bit-identical to the reference (compiled with --fmad=false; every
// expression keeps the reference's operation order).
//
// The device time loop runs one fused launch per step (k_step_f64, after a
// prologue k_fill_f64 that folds the first step's CFL maximum and writes the
// primitives of the initial state); FP64 batch instances run the same fused
// step in one persistent launch per iteration (k_batch_step_f64).  The
// host-driven godunov_unsplit runs it as two launches:
//   k_fill_f64         ghost fill (make_boundaries, src/HydroRun.h:388-399)
//                      into both states, primitives of every cell
//                      (ConvertToPrimitivesFunctor, src/HydroRunFunctors.h:84-143)
//                      and the CFL maximum of the interior
//                      (ComputeDtFunctor, src/HydroRunFunctors.h:17-79);
//   k_flux_update_f64  per 32x32 tile: limited slopes once per cell, the
//                      half-step trace once per cell and face, one Riemann
//                      solve per face, the conservative update
//                      (ComputeAndStoreFluxesFunctor + UpdateFunctor,
//                      src/HydroRunFunctors.h:412-723) and the time-loop
//                      bookkeeping of src/main.cpp:128-143.
// The reference evaluates the slopes of a cell three times and the trace
// sources four times per cell; evaluating each once gives the same bits.
#include "e2d_fp64_blocks.cuh"
#include "e2d_tma.cuh"

#include <cudaTypedefs.h>

#include <cstdint>

namespace e2d {
namespace {

constexpr int FILL_BX = 64, FILL_BY = 4;

// Shared memory of a TX x TY tile of the flux kernel: primitives with a
// 2-cell halo, then XMIN/XMAX states of cells x in [-1, TX] and YMIN/YMAX
// states of cells y in [-1, TY].
template <int TX, int TY>
constexpr size_t flux_smem_bytes() {
  return sizeof(double) * (4 * (TY + 4) * (TX + 4) + 2 * (4 * TY * (TX + 2)) + 2 * (4 * (TY + 2) * TX));
}

// The fused step's shared memory: the same tile + alignment slack of the
// TMA destination.
template <int TX, int TY>
constexpr size_t step_smem_bytes() {
  return flux_smem_bytes<TX, TY>() + 128;
}

// Ghost fill + primitives + CFL term of array cell (i, j) (see the file
// comment); `term`/`flags` receive its CFL term and E2D_FLAG_* bits.
__device__ __forceinline__ void fill_cell(const KParams64 &kp, double *__restrict__ u_in,
                                          double *__restrict__ u_out, double *__restrict__ q,
                                          const int mode, const int i, const int j, double &term,
                                          unsigned int &flags) {
  const KGeom &g = kp.g;
  const KPhys<double> &ph = kp.ph;
  if (i >= g.isize || j >= g.jsize) return;
  bool fu, fv;
  const int si = src_lo_hi(i, g.nx, g.bc_xmin, g.bc_xmax, fu);
  const int sj = src_lo_hi(j, g.ny, g.bc_ymin, g.bc_ymax, fv);
  const bool ghost = (si != i) || (sj != j);
  const size_t s = (size_t)si + (size_t)g.isize * sj;
  const double rho = u_in[s];
  const double e = u_in[s + g.plane];
  double mx = u_in[s + 2 * g.plane];
  double my = u_in[s + 3 * g.plane];
  if (fu) mx = -mx;
  if (fv) my = -my;
  const size_t d = (size_t)i + (size_t)g.isize * j;
  if (mode & FILL_COPY_OUT) {
    u_out[d] = rho;
    u_out[d + g.plane] = e;
    u_out[d + 2 * g.plane] = mx;
    u_out[d + 3 * g.plane] = my;
  }
  if (ghost) {
    if (mode & FILL_GHOSTS_IN) {
      u_in[d] = rho;
      u_in[d + g.plane] = e;
      u_in[d + 2 * g.plane] = mx;
      u_in[d + 3 * g.plane] = my;
    }
    if (mode & FILL_GHOSTS_OUT) {
      u_out[d] = rho;
      u_out[d + g.plane] = e;
      u_out[d + 2 * g.plane] = mx;
      u_out[d + 3 * g.plane] = my;
    }
  }
  if (mode & (FILL_WRITE_Q | FILL_DT)) {
    double dd, p, ux, uy;
    primitives(ph, rho, e, mx, my, dd, p, ux, uy);
    if (mode & FILL_WRITE_Q) {
      q[d] = dd;
      q[d + g.plane] = p;
      q[d + 2 * g.plane] = ux;
      q[d + 3 * g.plane] = uy;
    }
    if ((mode & FILL_DT) && !ghost) {
      term = cfl_term(ph, dd, p, ux, uy);
      flags |= state_flags(rho, e, mx, my);
    }
  }
}

// Block maximum of the CFL term into *acc (fmax drops NaN like the
// reference's reducer; positive doubles order like their bit patterns) and
// the OR of the flags into *status.  Every thread of the block calls it.
__device__ __forceinline__ void fill_reduce(double term, unsigned int flags, unsigned long long *acc,
                                            unsigned int *status) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) term = fmax(term, __shfl_xor_sync(0xffffffffu, term, off));
  flags = __reduce_or_sync(0xffffffffu, flags);
  __shared__ double wmax[FILL_BX * FILL_BY / 32];
  __shared__ unsigned int wflags[FILL_BX * FILL_BY / 32];
  const int tid = threadIdx.y * FILL_BX + threadIdx.x;
  if ((tid & 31) == 0) {
    wmax[tid >> 5] = term;
    wflags[tid >> 5] = flags;
  }
  __syncthreads();
  if (tid == 0) {
    double m = wmax[0];
    unsigned int f = wflags[0];
    for (int w = 1; w < FILL_BX * FILL_BY / 32; ++w) {
      m = fmax(m, wmax[w]);
      f |= wflags[w];
    }
    if (m > 0.0) atomicMax(acc, (unsigned long long)__double_as_longlong(m));
    if (f) atomicOr(status, f);
  }
}

__global__ void __launch_bounds__(FILL_BX *FILL_BY)
    k_fill_f64(const KParams64 kp, double *__restrict__ u_in, double *__restrict__ u_out,
               double *__restrict__ q, DevClock *clk, const int mode, const int acc_slot) {
  if ((mode & FILL_DEVICE_CLOCK) && !(clk->t < clk->t_end)) return;
  double term = 0.0;
  unsigned int flags = 0;
  fill_cell(kp, u_in, u_out, q, mode, blockIdx.x * FILL_BX + threadIdx.x, blockIdx.y * FILL_BY + threadIdx.y,
            term, flags);
  if (mode & FILL_DT)
    fill_reduce(term, flags, acc_slot < 0 ? &clk->invdt_bits : &clk->acc[acc_slot & 1], &clk->status);
}

// ------------------------------------------------------------ kernel 2
// Tile shapes (kp.tile): 0 -> 32 x 32 cells, 512 threads, 1 block per SM
// (180.7 KB shared; 1.125 slope/trace evaluations and 2.06 Riemann solves
// per cell); 1 -> 32 x 16, 256 threads, 2 blocks per SM (94.7 KB; 1.19 and
// 2.09).  Measured on the 4096^2 blast: 15.12 and 15.38 ms per step; smaller
// tiles (16 x 16, 32 x 8: 16.1, 16.7 ms) lose more to halo work than they
// gain in residency.  Results do not depend on the shape.

// Shared memory of a tile: primitives with a 2-cell halo, then the face
// states (the scaled fluxes replace the XMIN / YMIN states in stage 3).
template <int TX, int TY>
struct TileSmem {
  static constexpr int QW = TX + 4;  // primitives tile width (2-cell halo)
  static constexpr int QH = TY + 4;
  static constexpr int XW = TX + 2;  // x-face states: cells x in [-1, TX]
  static constexpr int YH = TY + 2;  // y-face states: cells y in [-1, TY]
  double *sQ, *sXm, *sXp, *sYm, *sYp;
  __device__ explicit TileSmem(double *smem) {
    sQ = smem;                   // [4][QH][QW]  primitives with halo
    sXm = sQ + 4 * QH * QW;      // [4][TY][XW]  XMIN states, then x-fluxes
    sXp = sXm + 4 * TY * XW;     // [4][TY][XW]  XMAX states
    sYm = sXp + 4 * TY * XW;     // [4][YH][TX]  YMIN states, then y-fluxes
    sYp = sYm + 4 * YH * TX;     // [4][YH][TX]  YMAX states
  }
};

// Stage 1 of the two-launch step: primitives of the tile and its 2-cell
// halo from the primitives array (ghost cells included, written by the fill
// kernel); cells beyond the array get a harmless 1.0.
template <int TX, int TY, int NT>
__device__ __forceinline__ void load_qtile(const KGeom &g, const double *__restrict__ q, int i0, int j0,
                                           double *sQ) {
  constexpr int QW = TX + 4, QH = TY + 4;
  for (int k = threadIdx.x; k < QH * QW; k += NT) {
    const int y = k / QW, x = k - y * QW;
    const int gi = i0 + x, gj = j0 + y;
    if (gi < g.isize && gj < g.jsize) {
      const size_t s = (size_t)gi + (size_t)g.isize * gj;
#pragma unroll
      for (int v = 0; v < 4; ++v) sQ[v * QH * QW + k] = q[s + v * g.plane];
    } else {
#pragma unroll
      for (int v = 0; v < 4; ++v) sQ[v * QH * QW + k] = 1.0;
    }
  }
}

// Stage 1 of the fused step for tiles whose halo reaches ghost cells: the
// primitives of a ghost cell are those of its source cell with the normal
// velocity negated where the boundary reflects -- bit for bit the
// primitives of the reference's ghost-filled state (u = mx / d changes only
// its sign with mx; e, p and c depend on u^2).  Only interior cells of q are
// read.
template <int TX, int TY, int NT>
__device__ __forceinline__ void gather_qtile(const KGeom &g, const double *__restrict__ q, int i0, int j0,
                                             double *sQ) {
  constexpr int QW = TX + 4, QH = TY + 4;
  for (int k = threadIdx.x; k < QH * QW; k += NT) {
    const int y = k / QW, x = k - y * QW;
    const int gi = i0 + x, gj = j0 + y;
    if (gi < g.isize && gj < g.jsize) {
      bool fu, fv;
      const int si = src_lo_hi(gi, g.nx, g.bc_xmin, g.bc_xmax, fu);
      const int sj = src_lo_hi(gj, g.ny, g.bc_ymin, g.bc_ymax, fv);
      const size_t s = (size_t)si + (size_t)g.isize * sj;
      const double ux = q[s + 2 * g.plane], uy = q[s + 3 * g.plane];
      sQ[k] = q[s];
      sQ[QH * QW + k] = q[s + g.plane];
      sQ[2 * QH * QW + k] = fu ? -ux : ux;
      sQ[3 * QH * QW + k] = fv ? -uy : uy;
    } else {
#pragma unroll
      for (int v = 0; v < 4; ++v) sQ[v * QH * QW + k] = 1.0;
    }
  }
}

// Stages 2 and 3 of a tile whose primitives are in shared memory (the
// caller has synchronised after writing them): slopes, trace sources and
// face states of the tile cells and of the 1-cell ring (corners excluded)
// -- src/HydroBaseFunctor.h:214-291 --, then one Riemann solve per face.
// On return (after a block barrier) sXm holds the x-fluxes scaled by dt/dx
// and sYm the y-fluxes scaled by dt/dy.
template <int RS, int TX, int TY, int NT, bool FAST = false>
__device__ __forceinline__ void tile_fluxes(const KPhys<double> &ph, const double dtdx, const double dtdy,
                                            double *smem) {
  using T = TileSmem<TX, TY>;
  constexpr int QW = T::QW, QH = T::QH, XW = T::XW, YH = T::YH;
  const T sm(smem);
  const double *sQ = sm.sQ;
  double *sXm = sm.sXm, *sXp = sm.sXp, *sYm = sm.sYm, *sYp = sm.sYp;
  const int tid = threadIdx.x;

  // stage 2: slopes, trace sources and face states.  Items enumerate the
  // tile and its 1-cell ring without the ring's four corners (which carry no
  // face), so the last partial round of 32 x 32 tiles is 4 whole warps -- one
  // per scheduler -- instead of 4 warps and 4 threads.  The FP64 pipe takes
  // as long for a warp instruction with a few active lanes as for a full
  // one, so a partial round costs what its busiest scheduler's warps cost.
  const int st_kind = (ph.slope_type == 2.0) ? 2 : (ph.slope_type == 1.0) ? 1 : 0;
  constexpr int NS2 = YH * XW - 4;
  for (int k = tid; k < NS2; k += NT) {
    int yy, xx;  // cell (xx-1, yy-1) of the tile
    if (k < TX) {
      yy = 0;
      xx = k + 1;
    } else if (k < TX + TY * XW) {
      const int r = k - TX;
      yy = 1 + r / XW;
      xx = r - (yy - 1) * XW;
    } else {
      yy = YH - 1;
      xx = k - (TX + TY * XW) + 1;
    }
    const bool xin = (xx >= 1) && (xx <= TX);
    const bool yin = (yy >= 1) && (yy <= TY);
    const int c = (yy + 1) * QW + (xx + 1);
    double qc[4], dqx[4], dqy[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const double *P = sQ + v * QH * QW;
      qc[v] = P[c];
      dqx[v] = slope(st_kind, qc[v], P[c + 1], P[c - 1]);
      dqy[v] = slope(st_kind, qc[v], P[c + QW], P[c - QW]);
    }
    double s0[4];
    if (FAST)
      trace_sources_fast(ph, qc, dqx, dqy, s0);
    else
      trace_sources(ph, qc, dqx, dqy, s0);
    if (yin) {
      const int o = (yy - 1) * XW + xx;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        double fm, fp;
        if (FAST)
          face_pair_fast(ph, v, qc[v], dqx[v], s0[v], 0.5 * dtdx, fm, fp);
        else
          face_pair(ph, v, qc[v], dqx[v], s0[v], dtdx, fm, fp);
        if (xx >= 1) sXm[v * TY * XW + o] = fm;
        if (xx <= TX) sXp[v * TY * XW + o] = fp;
      }
    }
    if (xin) {
      const int o = yy * TX + (xx - 1);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        double fm, fp;
        if (FAST)
          face_pair_fast(ph, v, qc[v], dqy[v], s0[v], 0.5 * dtdy, fm, fp);
        else
          face_pair(ph, v, qc[v], dqy[v], s0[v], dtdy, fm, fp);
        if (yy >= 1) sYm[v * YH * TX + o] = fm;
        if (yy <= TY) sYp[v * YH * TX + o] = fp;
      }
    }
  }
  __syncthreads();

  // stage 3: one Riemann solve per face; the scaled flux replaces the
  // right-hand state, which no other face reads
  constexpr int NXF = (TX + 1) * TY;
  constexpr int NYF = TX * (TY + 1);
  for (int k = tid; k < NXF + NYF; k += NT) {
    double ql[4], qr[4], f[4];
    if (k < NXF) {
      const int y = k / (TX + 1), fx = k - y * (TX + 1);
      const int ol = y * XW + fx, orr = ol + 1;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        ql[v] = sXp[v * TY * XW + ol];
        qr[v] = sXm[v * TY * XW + orr];
      }
      riemann_sel<RS, FAST>(ph, ql, qr, f);
#pragma unroll
      for (int v = 0; v < 4; ++v) sXm[v * TY * XW + orr] = f[v] * dtdx;
    } else {
      const int kk = k - NXF;
      const int fy = kk / TX, x = kk - fy * TX;
      const int ol = fy * TX + x, orr = ol + TX;
      // normal velocity first: swap IU/IV (src/HydroRunFunctors.h:628-632)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int vs = (v == E2D_IU) ? E2D_IV : (v == E2D_IV) ? E2D_IU : v;
        ql[vs] = sYp[v * YH * TX + ol];
        qr[vs] = sYm[v * YH * TX + orr];
      }
      riemann_sel<RS, FAST>(ph, ql, qr, f);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int vs = (v == E2D_IU) ? E2D_IV : (v == E2D_IV) ? E2D_IU : v;
        sYm[v * YH * TX + orr] = f[vs] * dtdy;
      }
    }
  }
  __syncthreads();
}

// The conservative update of cell (x, y) of a tile in the reference's order
// (src/HydroRunFunctors.h:691-713): +Fx(i) -Fx(i+1) +Fy(j) -Fy(j+1).
template <int TX, int TY>
__device__ __forceinline__ double update_var(const TileSmem<TX, TY> &sm, int v, int x, int y, double uu) {
  using T = TileSmem<TX, TY>;
  uu = uu + sm.sXm[v * TY * T::XW + y * T::XW + x + 1];
  uu = uu - sm.sXm[v * TY * T::XW + y * T::XW + x + 2];
  uu = uu + sm.sYm[v * T::YH * TX + (y + 1) * TX + x];
  uu = uu - sm.sYm[v * T::YH * TX + (y + 2) * TX + x];
  return uu;
}

// Stages 1-4 of the two-launch step for tile (bx, by) of a grid,
// block-wide; the caller provides dt/dx, dt/dy and TX x TY shared memory.
template <int RS, int TX, int TY, int NT>
__device__ __forceinline__ void flux_tile(const KParams64 &kp, const double *__restrict__ q,
                                          const double *__restrict__ u_in, double *__restrict__ u_out,
                                          const int bx, const int by, const double dtdx, const double dtdy,
                                          double *smem) {
  const KGeom &g = kp.g;
  const int i0 = bx * TX;  // array column of the tile's first halo cell
  const int j0 = by * TY;
  load_qtile<TX, TY, NT>(g, q, i0, j0, smem);
  __syncthreads();
  tile_fluxes<RS, TX, TY, NT>(kp.ph, dtdx, dtdy, smem);
  const TileSmem<TX, TY> sm(smem);
  // stage 4: conservative update
  for (int k = threadIdx.x; k < TX * TY; k += NT) {
    const int y = k / TX, x = k - y * TX;
    const int gi = i0 + 2 + x, gj = j0 + 2 + y;
    if (gi < g.nx + 2 && gj < g.ny + 2) {
      const size_t s = (size_t)gi + (size_t)g.isize * gj;
#pragma unroll
      for (int v = 0; v < 4; ++v) u_out[s + v * g.plane] = update_var<TX, TY>(sm, v, x, y, u_in[s + v * g.plane]);
    }
  }
}

template <int RS, int TX, int TY, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    k_flux_update_f64(const KParams64 kp, const double *__restrict__ q,
                      const double *__restrict__ u_in, double *__restrict__ u_out, DevClock *clk,
                      const int use_clock, const double host_dt, double *__restrict__ dt_trace) {
  extern __shared__ double smem[];
  const KPhys<double> &ph = kp.ph;
  const int tid = threadIdx.x;
  // dt of this step (the caller's, or src/main.cpp:128-134 on the device)
  // and dt/dx, dt/dy, computed once per block and broadcast: per-thread FP64
  // divisions here would cost ~2 divisions per cell on the FP64 pipe
  __shared__ double s_dt[3];
  __shared__ int s_run;
  if (tid == 0) {
    double dt = host_dt;
    int run = 1;
    if (use_clock) {
      run = clk->t < clk->t_end;
      dt = step_dt(ph, clk->invdt_bits, clk->t, clk->t_end);
    }
    s_dt[0] = dt;
    s_dt[1] = dt / ph.dx;
    s_dt[2] = dt / ph.dy;
    s_run = run;
  }
  __syncthreads();
  if (!s_run) return;
  const double dt = s_dt[0];
  flux_tile<RS, TX, TY, NT>(kp, q, u_in, u_out, blockIdx.x, blockIdx.y, s_dt[1], s_dt[2], smem);

  if (!use_clock) return;
  // the last block to finish advances the loop state (src/main.cpp:139-143)
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned int nblocks = gridDim.x * gridDim.y;
    const unsigned int ticket = atomicAdd(&clk->done_blocks, 1u);
    if (ticket == nblocks - 1) {
      __threadfence();
      const int ns = clk->nstep;
      const int slot = ns - clk->trace_base;
      if (dt_trace && slot >= 0 && slot < clk->trace_cap) dt_trace[slot] = dt;
      if (!(dt > 0.0) || nonfinite(dt)) clk->status |= E2D_FLAG_BAD_DT;
      clk->dt = dt;
      clk->t = clk->t + dt;  // only this block writes t during the step
      clk->nstep = ns + 1;
      clk->invdt_bits = 0ull;
      clk->done_blocks = 0u;
      __threadfence();
    }
  }
}

// ------------------------------------------------------------ the fused step
// Block maximum of the CFL term into *acc and the OR of the flags into
// *status, one atomic of each per block (fmax drops NaN like the reference's
// reducer; positive doubles order like their bit patterns).
template <int NT>
__device__ __forceinline__ void block_fold(double term, unsigned int flags, unsigned long long *acc,
                                           unsigned int *status) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) term = fmax(term, __shfl_xor_sync(0xffffffffu, term, off));
  flags = __reduce_or_sync(0xffffffffu, flags);
  __shared__ double wmax[NT / 32];
  __shared__ unsigned int wflags[NT / 32];
  const int tid = threadIdx.x;
  if ((tid & 31) == 0) {
    wmax[tid >> 5] = term;
    wflags[tid >> 5] = flags;
  }
  __syncthreads();
  if (tid == 0) {
    double m = wmax[0];
    unsigned int f = wflags[0];
#pragma unroll
    for (int w = 1; w < NT / 32; ++w) {
      m = fmax(m, wmax[w]);
      f |= wflags[w];
    }
    if (m > 0.0) atomicMax(acc, (unsigned long long)__double_as_longlong(m));
    if (f) atomicOr(status, f);
  }
}

// The fused step's epilogue for the cells of a tile whose fluxes are in
// shared memory: the conservative update into u_out, the primitives of the
// new cells into q_out and the running maximum of their CFL terms and flags.
template <int TX, int TY, int NT, bool FAST>
__device__ __forceinline__ void step_epilogue(const KParams64 &kp, const double *__restrict__ u_in,
                                              double *__restrict__ u_out, double *__restrict__ q_out, int i0,
                                              int j0, double *smem, double &term, unsigned int &flags) {
  const KGeom &g = kp.g;
  const KPhys<double> &ph = kp.ph;
  const TileSmem<TX, TY> sm(smem);
  for (int k = threadIdx.x; k < TX * TY; k += NT) {
    const int y = k / TX, x = k - y * TX;
    const int gi = i0 + 2 + x, gj = j0 + 2 + y;
    if (gi < g.nx + 2 && gj < g.ny + 2) {
      const size_t s = (size_t)gi + (size_t)g.isize * gj;
      double un[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        un[v] = update_var<TX, TY>(sm, v, x, y, u_in[s + v * g.plane]);
        u_out[s + v * g.plane] = un[v];
      }
      double dd, p, ux, uy, rd = 0.0;
      if (FAST)
        primitives_fast(ph, un[E2D_ID], un[E2D_IP], un[E2D_IU], un[E2D_IV], dd, p, ux, uy, rd);
      else
        primitives(ph, un[E2D_ID], un[E2D_IP], un[E2D_IU], un[E2D_IV], dd, p, ux, uy);
      q_out[s] = dd;
      q_out[s + g.plane] = p;
      q_out[s + 2 * g.plane] = ux;
      q_out[s + 3 * g.plane] = uy;
      term = fmax(term, FAST ? cfl_term_fast(ph, rd, p, ux, uy) : cfl_term(ph, dd, p, ux, uy));
      flags |= state_flags(un[E2D_ID], un[E2D_IP], un[E2D_IU], un[E2D_IV]);
    }
  }
}

// The ghost cells next to a tile -- those whose nearest interior cell is in
// it -- receive the ghost fill of u_in in both states, read from interior
// cells of u_in only (no block writes those during a step).
template <int TX, int TY, int NT>
__device__ __forceinline__ void ghost_fill_tile(const KGeom &g, double *__restrict__ u_in, double *__restrict__ u_out,
                                                int i0, int j0, bool lo_x, bool hi_x, bool lo_y, bool hi_y) {
  if (!(lo_x || hi_x || lo_y || hi_y)) return;
  const int xa = lo_x ? 0 : i0 + 2, xb = hi_x ? g.isize : i0 + 2 + TX;
  const int ya = lo_y ? 0 : j0 + 2, yb = hi_y ? g.jsize : j0 + 2 + TY;
  const int w = xb - xa, n = w * (yb - ya);
  for (int k = threadIdx.x; k < n; k += NT) {
    const int j = ya + k / w, i = xa + k % w;
    if (i >= 2 && i < g.nx + 2 && j >= 2 && j < g.ny + 2) continue;
    bool fu, fv;
    const int si = src_lo_hi(i, g.nx, g.bc_xmin, g.bc_xmax, fu);
    const int sj = src_lo_hi(j, g.ny, g.bc_ymin, g.bc_ymax, fv);
    const size_t s = (size_t)si + (size_t)g.isize * sj, d = (size_t)i + (size_t)g.isize * j;
    double v4[4] = {u_in[s], u_in[s + g.plane], u_in[s + 2 * g.plane], u_in[s + 3 * g.plane]};
    if (fu) v4[E2D_IU] = -v4[E2D_IU];
    if (fv) v4[E2D_IV] = -v4[E2D_IV];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      u_in[d + v * g.plane] = v4[v];
      u_out[d + v * g.plane] = v4[v];
    }
  }
}

template <int TX, int TY>
__host__ __device__ constexpr unsigned int qtile_bytes() {
  return (unsigned int)(sizeof(double) * 4 * (TX + 4) * (TY + 4));
}

// One whole time step of the device loop (src/main.cpp:128-143 around
// godunov_unsplit_impl, src/HydroRun.h:279-364), one TX x TY tile per block:
//  - dt from the CFL maximum of the input state, clock->acc[nstep & 1],
//    which the previous step (or the prologue fill) folded;
//  - stage 1: primitives of the tile and its 2-cell halo, from q_in (the
//    primitives of u_in's interior cells): one TMA copy of the box for tiles
//    whose halo is interior, else a gather through the boundary map;
//  - stages 2-3: slopes, trace, face states, one Riemann solve per face;
//  - epilogue: the conservative update into u_out, the primitives of the
//    new cells into q_out and their CFL term, folded into
//    clock->acc[(nstep + 1) & 1] with one atomic per block;
//  - boundary tiles write the ghost fill of u_in into the ghost cells of
//    both states (make_boundaries + deep_copy of the reference), reading
//    only interior cells of u_in, which no block writes;
//  - the last block to finish advances the loop state.
// Bit-identical to the two-launch step; FP64 work per cell is the same.
template <int RS, int TX, int TY, int NT, int MINB, bool FAST>
__global__ void __launch_bounds__(NT, MINB)
    k_step_f64(const KParams64 kp, const __grid_constant__ CUtensorMap tm_q, const int use_tma,
               const double *__restrict__ q_in, double *__restrict__ q_out, double *__restrict__ u_in,
               double *__restrict__ u_out, DevClock *clk, double *__restrict__ dt_trace) {
  extern __shared__ unsigned char smem_raw[];
  // a TMA destination must be 128-byte aligned
  double *smem = reinterpret_cast<double *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  __shared__ double s_dt[3];
  __shared__ int s_run, s_par;
  __shared__ __align__(8) unsigned long long s_bar;
  const KGeom &g = kp.g;
  const KPhys<double> &ph = kp.ph;
  const int tid = threadIdx.x;
  const int bx = blockIdx.x, by = blockIdx.y;
  const int i0 = bx * TX, j0 = by * TY;  // array cell of the halo box's corner
  constexpr int QW = TX + 4, QH = TY + 4;
  const bool tma_tile = use_tma && i0 >= 2 && j0 >= 2 && i0 + QW <= g.nx + 2 && j0 + QH <= g.ny + 2;
  if (tid == 0) {
    const int run = clk->t < clk->t_end;
    const int par = clk->nstep & 1;
    const double dt = step_dt(ph, clk->acc[par], clk->t, clk->t_end);
    s_dt[0] = dt;
    s_dt[1] = dt / ph.dx;
    s_dt[2] = dt / ph.dy;
    s_run = run;
    s_par = par;
    if (run && tma_tile) {
      mbar_init(&s_bar, 1u);
      mbar_init_fence();
      // wait_test: tile (1, 1) never copies, so its bounded wait runs out
      if (!(kp.wait_test && bx == 1 && by == 1)) {
        mbar_arrive_expect(&s_bar, qtile_bytes<TX, TY>());
        tma_load_3d(smem, &tm_q, i0, j0, 0, &s_bar);
      }
    }
  }
  __syncthreads();
  if (!s_run) return;  // past t_end: no copy was issued
  const int par = s_par;
  bool ok = true;
  if (tma_tile) {
    ok = __syncthreads_and(mbar_wait(&s_bar, 0u));
    if (!ok) {
      // flag the step, then wait (bounded) for the copy that may still land
      // in this block's shared memory before leaving the tile
      if (tid == 0) atomicOr(&clk->status, E2D_FLAG_TIMEOUT);
      mbar_wait(&s_bar, 0u);
      __syncthreads();
    }
  } else {
    gather_qtile<TX, TY, NT>(g, q_in, i0, j0, smem);
    __syncthreads();
  }

  double term = 0.0;
  unsigned int flags = 0;
  if (ok) {
    tile_fluxes<RS, TX, TY, NT, FAST>(ph, s_dt[1], s_dt[2], smem);
    step_epilogue<TX, TY, NT, FAST>(kp, u_in, u_out, q_out, i0, j0, smem, term, flags);
  }
  ghost_fill_tile<TX, TY, NT>(g, u_in, u_out, i0, j0, bx == 0, bx == (int)gridDim.x - 1, by == 0,
                              by == (int)gridDim.y - 1);

  block_fold<NT>(term, flags, &clk->acc[par ^ 1], &clk->status);

  // the last block to finish advances the loop state (src/main.cpp:139-143)
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned int ticket = atomicAdd(&clk->done_blocks, 1u);
    if (ticket == gridDim.x * gridDim.y - 1) {
      __threadfence();
      const double dt = s_dt[0];
      const int ns = clk->nstep;
      const int slot = ns - clk->trace_base;
      if (dt_trace && slot >= 0 && slot < clk->trace_cap) dt_trace[slot] = dt;
      if (!(dt > 0.0) || nonfinite(dt)) clk->status |= E2D_FLAG_BAD_DT;
      clk->dt = dt;
      clk->t = clk->t + dt;  // only this block writes t during the step
      clk->nstep = ns + 1;
      clk->acc[par] = 0ull;  // read by this step; folded into by the next
      clk->done_blocks = 0u;
      __threadfence();
    }
  }
}

// ------------------------------------------------------------ batches
// Instance k of a work list with begin[k] <= w < begin[k + 1].
__device__ __forceinline__ int list_entry(const int *__restrict__ begin, int n, int w) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (begin[mid] <= w)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// An admitted FP64 instance's first primitives and CFL maximum (the device
// loop's prologue): q[0] from u[0], the maximum into acc[0].
__global__ void __launch_bounds__(FILL_BX *FILL_BY) k_batch_prime_f64(BatchInst64 *__restrict__ I) {
  const int by = blockIdx.x / I->nbx, bx = blockIdx.x - by * I->nbx;
  double term = 0.0;
  unsigned int flags = 0;
  fill_cell(I->kp, I->u[0], nullptr, I->q[0], FILL_WRITE_Q | FILL_DT, bx * FILL_BX + threadIdx.x,
            by * FILL_BY + threadIdx.y, term, flags);
  fill_reduce(term, flags, &I->acc[0], &I->status);
}

// One iteration of every listed FP64 instance in one persistent launch: each
// block takes 32 x 32 tiles from the work list (instance k's tiles are
// tile_begin[k] .. tile_begin[k+1]-1) and runs the fused step on each with
// its instance's dt, primitives and ghost cells (tiles gathered, no TMA);
// the instance's last tile advances its loop state.
template <int RS>
__global__ void __launch_bounds__(512, 1)
    k_batch_step_f64(BatchInst64 *__restrict__ insts, const int *__restrict__ list_slots,
                     const int *__restrict__ tile_begin, const int n_inst, const int total_tiles) {
  extern __shared__ unsigned char smem_raw[];
  double *smem = reinterpret_cast<double *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  __shared__ double s_dt[3];
  const int tid = threadIdx.x;
  for (int w = blockIdx.x; w < total_tiles; w += gridDim.x) {
    const int k = list_entry(tile_begin, n_inst, w);
    BatchInst64 &I = insts[list_slots[k]];
    if (!I.active) continue;  // block-uniform
    const KParams64 &kp = I.kp;
    const int par = I.par;
    if (tid == 0) {
      const double dt = step_dt(kp.ph, I.acc[par], I.t, I.t_end);
      s_dt[0] = dt;
      s_dt[1] = dt / kp.ph.dx;
      s_dt[2] = dt / kp.ph.dy;
    }
    const int b = w - tile_begin[k];
    const int by = b / I.ntx, bx = b - by * I.ntx;
    const int nty = I.ntiles / I.ntx;
    const int i0 = bx * 32, j0 = by * 32;
    gather_qtile<32, 32, 512>(kp.g, I.q[par], i0, j0, smem);
    __syncthreads();
    double term = 0.0;
    unsigned int flags = 0;
    tile_fluxes<RS, 32, 32, 512>(kp.ph, s_dt[1], s_dt[2], smem);
    step_epilogue<32, 32, 512, false>(kp, I.u[par], I.u[par ^ 1], I.q[par ^ 1], i0, j0, smem, term, flags);
    ghost_fill_tile<32, 32, 512>(kp.g, I.u[par], I.u[par ^ 1], i0, j0, bx == 0, bx == I.ntx - 1, by == 0,
                                 by == nty - 1);
    block_fold<512>(term, flags, &I.acc[par ^ 1], &I.status);
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      const unsigned int ticket = atomicAdd(&I.done, 1u);
      if (ticket == (unsigned)I.ntiles - 1u) {
        __threadfence();
        const double dt = s_dt[0];
        if (!(dt > 0.0) || nonfinite(dt)) I.status |= E2D_FLAG_BAD_DT;
        I.dt = dt;
        I.t = I.t + dt;
        I.nstep = I.nstep + 1;
        I.par = par ^ 1;
        I.acc[par] = 0ull;  // read by this step; folded into by the next
        I.done = 0u;
        I.active = (I.t < I.t_end) && !(I.status & (E2D_FLAG_NONFINITE | E2D_FLAG_BAD_DT));
        __threadfence();
      }
    }
    __syncthreads();  // s_dt and the shared tile are rewritten by the next tile
  }
}

// ------------------------------------------------------------ building blocks
// One building block of the step per thread, with the exact device code the
// step kernels use (see e2d_eval_device in include/e2d.h for the layouts).
__global__ void k_eval_f64(const KParams64 kp, const int what, const int n,
                           const double *__restrict__ in, double *__restrict__ out, const double dtdx,
                           const double dtdy) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const KPhys<double> &ph = kp.ph;
  const int st_kind = (ph.slope_type == 2.0) ? 2 : (ph.slope_type == 1.0) ? 1 : 0;
  if (what == E2D_EVAL_PRIMITIVES) {
    const double *u = in + 4 * k;
    double d, p, ux, uy;
    primitives(ph, u[E2D_ID], u[E2D_IP], u[E2D_IU], u[E2D_IV], d, p, ux, uy);
    double *o = out + 5 * k;
    o[E2D_ID] = d;
    o[E2D_IP] = p;
    o[E2D_IU] = ux;
    o[E2D_IV] = uy;
    o[4] = sqrt(ph.gamma0 * p / d);
  } else if (what == E2D_EVAL_SLOPES) {
    const double *s = in + 20 * k;  // q, q(+x), q(-x), q(+y), q(-y)
    double *o = out + 8 * k;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      o[v] = slope(st_kind, s[v], s[4 + v], s[8 + v]);
      o[4 + v] = slope(st_kind, s[v], s[12 + v], s[16 + v]);
    }
  } else if (what >= E2D_EVAL_TRACE_XMIN && what <= E2D_EVAL_TRACE_YMAX) {
    const double *s = in + 12 * k;  // q, dqx, dqy
    double s0[4];
    trace_sources(ph, s, s + 4, s + 8, s0);
    const int face = what - E2D_EVAL_TRACE_XMIN;
    const bool xdir = face < 2;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      double fm, fp;
      face_pair(ph, v, s[v], xdir ? s[4 + v] : s[8 + v], s0[v], xdir ? dtdx : dtdy, fm, fp);
      out[4 * k + v] = (face == 0 || face == 2) ? fm : fp;
    }
  } else {
    const double *s = in + 8 * k;  // qleft, qright
    double *o = out + 4 * k;
    if (what == E2D_EVAL_RIEMANN_HLLC)
      riemann_hllc(ph, s, s + 4, o);
    else if (what == E2D_EVAL_RIEMANN_HLL)
      riemann_hll(ph, s, s + 4, o);
    else
      riemann_approx(ph, s, s + 4, o);
  }
}

// ------------------------------------------------------------ initial conditions
// src/HydroRunFunctors.h:1347-1827: cell centres x = xmin + dx/2 + (i-g)*dx.
__global__ void k_init_f64(const KParams64 kp, const e2d_params p, double *__restrict__ u,
                           const double blast_e_inside) {
  const KGeom &g = kp.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.isize || j >= g.jsize) return;
  const double gamma0 = p.gamma0;
  const double x = p.xmin + p.dx / 2 + (i - 2) * p.dx;
  const double y = p.ymin + p.dy / 2 + (j - 2) * p.dy;
  double d = 0, e = 0, mx = 0, my = 0;
  switch (p.problemType) {
    case E2D_PROBLEM_IMPLODE: {  // :1375-1401
      bool in;
      if (p.implode_shape == 0) {
        const double tmp = x + y * y;
        in = tmp > 0.5 && tmp < 1.5;
      } else {
        in = x + y > 0.5;
      }
      d = in ? 1.0 : 0.125;
      e = in ? 1.0 / (gamma0 - 1.0) : 0.14 / (gamma0 - 1.0);
      break;
    }
    case E2D_PROBLEM_BLAST: {  // :1451-1520
      const double r2 = p.blast_radius * p.blast_radius;
      const double d2 = (x - p.blast_center_x) * (x - p.blast_center_x) +
                        (y - p.blast_center_y) * (y - p.blast_center_y);
      const bool in = d2 < r2;
      d = in ? p.blast_density_in : p.blast_density_out;
      e = (in ? p.blast_pressure_in : p.blast_pressure_out) / (gamma0 - 1.0);
      if (in && blast_e_inside > 0.0) e = blast_e_inside;
      break;
    }
    case E2D_PROBLEM_FOUR_QUADRANT: {  // :1578-1665 (default states: Lax-Liu case 3)
      const int r = (x < p.fq_split_x) ? ((y < p.fq_split_y) ? 2 : 1) : ((y < p.fq_split_y) ? 3 : 0);
      const double rho = p.fq_state[r][0], pr = p.fq_state[r][1], uu = p.fq_state[r][2], vv = p.fq_state[r][3];
      d = rho;
      mx = uu * rho;
      my = vv * rho;
      e = pr / (gamma0 - 1.0) + rho * (uu * uu + vv * vv) * 0.5;
      break;
    }
    case E2D_PROBLEM_DISCONTINUITY: {  // :1697-1731
      if (x + y < 1) {
        d = 1.0 + x * x;
      } else {
        d = 0.25;
      }
      e = 1.0 / (gamma0 - 1.0);
      break;
    }
    default: {  // E2D_PROBLEM_SHOCKED_BUBBLE, :1761-1822
      if (x < p.shock_loc) {
        d = p.postshock_density;
        mx = p.postshock_density * p.postshock_velocity;
        my = 0.0;
        const double rho_eint = p.postshock_pressure / (gamma0 - 1);
        e = rho_eint + 0.5 * (mx * mx + my * my) / d;
      } else {
        const double rad = sqrt((x - p.bubble_center_x) * (x - p.bubble_center_x) +
                                (y - p.bubble_center_y) * (y - p.bubble_center_y));
        const bool in = rad < p.bubble_radius;
        d = in ? p.bubble_density : p.preshock_density;
        const double rho_eint = (in ? p.bubble_pressure : p.preshock_pressure) / (gamma0 - 1);
        e = rho_eint + 0.5 * (mx * mx + my * my) / d;
      }
      break;
    }
  }
  const size_t o = (size_t)i + (size_t)g.isize * j;
  u[o] = d;
  u[o + g.plane] = e;
  u[o + 2 * g.plane] = mx;
  u[o + 3 * g.plane] = my;
}

}  // namespace


cudaError_t launch_fill_f64(const KParams64 &kp, double *u_in, double *u_out, double *q,
                            DevClock *clk, int mode, cudaStream_t s, int acc_slot) {
  dim3 block(FILL_BX, FILL_BY);
  dim3 grid((kp.g.isize + FILL_BX - 1) / FILL_BX, (kp.g.jsize + FILL_BY - 1) / FILL_BY);
  k_fill_f64<<<grid, block, 0, s>>>(kp, u_in, u_out, q, clk, mode, acc_slot);
  return cudaGetLastError();
}

template <int RS, int TX, int TY, int NT, int MINB>
static cudaError_t launch_flux_shape(const KParams64 &kp, const double *q, const double *u_in,
                                     double *u_out, DevClock *clk, int use_clock, double host_dt,
                                     double *dt_trace, cudaStream_t s) {
  dim3 grid((kp.g.nx + TX - 1) / TX, (kp.g.ny + TY - 1) / TY);
  k_flux_update_f64<RS, TX, TY, NT, MINB><<<grid, NT, flux_smem_bytes<TX, TY>(), s>>>(
      kp, q, u_in, u_out, clk, use_clock, host_dt, dt_trace);
  return cudaGetLastError();
}

template <int RS>
static cudaError_t launch_flux_t(const KParams64 &kp, const double *q, const double *u_in,
                                 double *u_out, DevClock *clk, int use_clock, double host_dt,
                                 double *dt_trace, cudaStream_t s) {
  if (kp.tile == 1)
    return launch_flux_shape<RS, 32, 16, 256, 2>(kp, q, u_in, u_out, clk, use_clock, host_dt, dt_trace, s);
  return launch_flux_shape<RS, 32, 32, 512, 1>(kp, q, u_in, u_out, clk, use_clock, host_dt, dt_trace, s);
}

template <int RS, int TX, int TY, int NT, int MINB>
static cudaError_t set_flux_smem() {
  return cudaFuncSetAttribute(k_flux_update_f64<RS, TX, TY, NT, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)flux_smem_bytes<TX, TY>());
}

template <int RS, int TX, int TY, int NT, int MINB, bool FAST = false>
static cudaError_t set_step_smem() {
  return cudaFuncSetAttribute(k_step_f64<RS, TX, TY, NT, MINB, FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)step_smem_bytes<TX, TY>());
}

template <int RS>
static cudaError_t configure_rs() {
  cudaError_t e = set_flux_smem<RS, 32, 32, 512, 1>();
  if (e == cudaSuccess) e = set_flux_smem<RS, 32, 16, 256, 2>();
  if (e == cudaSuccess) e = set_step_smem<RS, 32, 32, 512, 1>();
  if (e == cudaSuccess) e = set_step_smem<RS, 32, 16, 256, 2>();
  if (e == cudaSuccess) e = set_step_smem<RS, 32, 31, 512, 1>();
  if (e == cudaSuccess) e = set_step_smem<RS, 32, 15, 256, 2>();
  if (e == cudaSuccess) e = set_step_smem<RS, 32, 32, 512, 1, true>();
  if (e == cudaSuccess) e = set_step_smem<RS, 32, 16, 256, 2, true>();
  return e;
}

template <int RS>
static cudaError_t set_batch_flux_smem() {
  return cudaFuncSetAttribute(k_batch_step_f64<RS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)step_smem_bytes<32, 32>());
}

cudaError_t configure_f64_kernels() {
  cudaError_t e = configure_rs<E2D_RIEMANN_HLLC>();
  if (e == cudaSuccess) e = configure_rs<E2D_RIEMANN_HLL>();
  if (e == cudaSuccess) e = configure_rs<E2D_RIEMANN_APPROX>();
  if (e == cudaSuccess) e = set_batch_flux_smem<E2D_RIEMANN_HLLC>();
  if (e == cudaSuccess) e = set_batch_flux_smem<E2D_RIEMANN_HLL>();
  if (e == cudaSuccess) e = set_batch_flux_smem<E2D_RIEMANN_APPROX>();
  return e;
}

void batch_f64_shape(const KParams64 &kp, int *nbx, int *nfill, int *ntx, int *ntiles) {
  *nbx = (kp.g.isize + FILL_BX - 1) / FILL_BX;
  *nfill = *nbx * ((kp.g.jsize + FILL_BY - 1) / FILL_BY);
  *ntx = (kp.g.nx + 31) / 32;
  *ntiles = *ntx * ((kp.g.ny + 31) / 32);
}

cudaError_t launch_batch_prime_f64(BatchInst64 *inst, int nfill, cudaStream_t s) {
  k_batch_prime_f64<<<nfill, dim3(FILL_BX, FILL_BY), 0, s>>>(inst);
  return cudaGetLastError();
}

cudaError_t launch_batch_f64(int riemann, BatchInst64 *insts, const int *list_slots, const int *tile_begin,
                             int n_inst, int total_tiles, int grid_blocks, cudaStream_t s) {
  if (n_inst <= 0 || total_tiles <= 0) return cudaSuccess;
  const size_t sm = step_smem_bytes<32, 32>();
  const int grid = grid_blocks < total_tiles ? grid_blocks : total_tiles;
  switch (riemann) {
    case E2D_RIEMANN_HLLC:
      k_batch_step_f64<E2D_RIEMANN_HLLC><<<grid, 512, sm, s>>>(insts, list_slots, tile_begin, n_inst, total_tiles);
      break;
    case E2D_RIEMANN_HLL:
      k_batch_step_f64<E2D_RIEMANN_HLL><<<grid, 512, sm, s>>>(insts, list_slots, tile_begin, n_inst, total_tiles);
      break;
    default:
      k_batch_step_f64<E2D_RIEMANN_APPROX><<<grid, 512, sm, s>>>(insts, list_slots, tile_begin, n_inst, total_tiles);
      break;
  }
  return cudaGetLastError();
}

cudaError_t launch_flux_update_f64(const KParams64 &kp, int riemann, const double *q,
                                   const double *u_in, double *u_out, DevClock *clk,
                                   int use_clock, double host_dt, double *dt_trace,
                                   cudaStream_t s) {
  switch (riemann) {
    case E2D_RIEMANN_HLLC:
      return launch_flux_t<E2D_RIEMANN_HLLC>(kp, q, u_in, u_out, clk, use_clock, host_dt, dt_trace, s);
    case E2D_RIEMANN_HLL:
      return launch_flux_t<E2D_RIEMANN_HLL>(kp, q, u_in, u_out, clk, use_clock, host_dt, dt_trace, s);
    default:
      return launch_flux_t<E2D_RIEMANN_APPROX>(kp, q, u_in, u_out, clk, use_clock, host_dt, dt_trace, s);
  }
}

// Fused-step tile shapes (kp.tile): 32 x 32 cells, 512 threads, one block
// per SM (the default); 1 -> 32 x 16, 256 threads, two blocks per SM (0.6 %
// slower per 4096^2 HLLC step: 5 % more instructions per cell for the halo,
// the FP64 pipe 86 % instead of 82 % busy); 2 -> 32 x 31 (2047 Riemann
// solves: four full rounds of 512 threads); 3 -> 32 x 15 (two blocks per SM,
// 1007 solves: four rounds of 256).  The fast forms exist for 32 x 32 and
// 32 x 16.  Results do not depend on the shape.
template <int RS, int TX, int TY, int NT, int MINB, bool FAST = false>
static cudaError_t launch_step_shape(const KParams64 &kp, const CUtensorMap &tm_q, int use_tma, const double *q_in,
                                     double *q_out, double *u_in, double *u_out, DevClock *clk, double *dt_trace,
                                     cudaStream_t s) {
  dim3 grid((kp.g.nx + TX - 1) / TX, (kp.g.ny + TY - 1) / TY);
  k_step_f64<RS, TX, TY, NT, MINB, FAST><<<grid, NT, step_smem_bytes<TX, TY>(), s>>>(kp, tm_q, use_tma, q_in, q_out,
                                                                                      u_in, u_out, clk, dt_trace);
  return cudaGetLastError();
}

template <int RS>
static cudaError_t launch_step_t(const KParams64 &kp, const CUtensorMap &tm_q, int use_tma, const double *q_in,
                                 double *q_out, double *u_in, double *u_out, DevClock *clk, double *dt_trace,
                                 cudaStream_t s) {
  if (kp.fast) {  // the fast forms: 32 x 32 (default) and 32 x 16 tiles
    if (kp.tile == 1)
      return launch_step_shape<RS, 32, 16, 256, 2, true>(kp, tm_q, use_tma, q_in, q_out, u_in, u_out, clk, dt_trace,
                                                         s);
    return launch_step_shape<RS, 32, 32, 512, 1, true>(kp, tm_q, use_tma, q_in, q_out, u_in, u_out, clk, dt_trace, s);
  }
  switch (kp.tile) {
    case 1: return launch_step_shape<RS, 32, 16, 256, 2>(kp, tm_q, use_tma, q_in, q_out, u_in, u_out, clk, dt_trace, s);
    case 2: return launch_step_shape<RS, 32, 31, 512, 1>(kp, tm_q, use_tma, q_in, q_out, u_in, u_out, clk, dt_trace, s);
    case 3: return launch_step_shape<RS, 32, 15, 256, 2>(kp, tm_q, use_tma, q_in, q_out, u_in, u_out, clk, dt_trace, s);
    default: return launch_step_shape<RS, 32, 32, 512, 1>(kp, tm_q, use_tma, q_in, q_out, u_in, u_out, clk, dt_trace, s);
  }
}

cudaError_t launch_step_f64(const KParams64 &kp, int riemann, const CUtensorMap &tm_q, int use_tma,
                            const double *q_in, double *q_out, double *u_in, double *u_out, DevClock *clk,
                            double *dt_trace, cudaStream_t s) {
  switch (riemann) {
    case E2D_RIEMANN_HLLC:
      return launch_step_t<E2D_RIEMANN_HLLC>(kp, tm_q, use_tma, q_in, q_out, u_in, u_out, clk, dt_trace, s);
    case E2D_RIEMANN_HLL:
      return launch_step_t<E2D_RIEMANN_HLL>(kp, tm_q, use_tma, q_in, q_out, u_in, u_out, clk, dt_trace, s);
    default:
      return launch_step_t<E2D_RIEMANN_APPROX>(kp, tm_q, use_tma, q_in, q_out, u_in, u_out, clk, dt_trace, s);
  }
}

// The box of the fused step's primitives tile for the tile shape of kp:
// dimensions (isize, jsize, 4 planes), box (TX + 4) x (TY + 4) x 4.  Row and
// plane strides must be multiples of 16 bytes, so isize must be even; false
// (tiles are then gathered) otherwise or if the driver cannot encode it.
bool encode_q_map(CUtensorMap *map, const double *q, const KParams64 &kp) {
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult qr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr) != cudaSuccess ||
        qr != cudaDriverEntryPointSuccess)
      return nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode || (kp.g.isize & 1) || (reinterpret_cast<uintptr_t>(q) & 15u)) return false;
  const int ty = kp.tile == 1 ? 16 : kp.tile == 2 && !kp.fast ? 31 : kp.tile == 3 && !kp.fast ? 15 : 32;
  const cuuint64_t dims[3] = {(cuuint64_t)kp.g.isize, (cuuint64_t)kp.g.jsize, 4};
  const cuuint64_t strides[2] = {(cuuint64_t)kp.g.isize * sizeof(double), (cuuint64_t)kp.g.plane * sizeof(double)};
  const cuuint32_t box[3] = {32 + 4, (cuuint32_t)ty + 4, 4};
  const cuuint32_t estr[3] = {1, 1, 1};
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double *>(q), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t launch_eval_f64(const KParams64 &kp, int what, int n, const double *in, double *out,
                            double dtdx, double dtdy, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_eval_f64<<<(n + 127) / 128, 128, 0, s>>>(kp, what, n, in, out, dtdx, dtdy);
  return cudaGetLastError();
}

cudaError_t launch_init_f64(const KParams64 &kp, const e2d_params &p, double *u, cudaStream_t s) {
  // Sedov variant (src/HydroRunFunctors.h:1425-1447, :1496-1547): the
  // inside energy is total_energy_inside / (inside cell count * dx * dy).
  double e_inside = 0.0;
  if (p.problemType == E2D_PROBLEM_BLAST && p.blast_total_energy_inside > 0) {
    long long count = 0;
    const double r2 = p.blast_radius * p.blast_radius;
    for (int j = 0; j < kp.g.jsize; ++j)
      for (int i = 0; i < kp.g.isize; ++i) {
        const double x = p.xmin + p.dx / 2 + (i - 2) * p.dx;
        const double y = p.ymin + p.dy / 2 + (j - 2) * p.dy;
        const double d2 = (x - p.blast_center_x) * (x - p.blast_center_x) +
                          (y - p.blast_center_y) * (y - p.blast_center_y);
        if (d2 < r2) count++;
      }
    if (count > 0) e_inside = p.blast_total_energy_inside / ((double)count * (p.dx * p.dy));
  }
  dim3 block(64, 4);
  dim3 grid((kp.g.isize + 63) / 64, (kp.g.jsize + 3) / 4);
  k_init_f64<<<grid, block, 0, s>>>(kp, p, u, e_inside);
  return cudaGetLastError();
}

}  // namespace e2d
