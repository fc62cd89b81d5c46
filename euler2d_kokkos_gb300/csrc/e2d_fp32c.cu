// e2d_fp32c.cu -- FP32 step with a compensated (hi, lo) conservative update.
//
// The state keeps each conserved variable as an unevaluated sum hi + lo of
// two floats (~48 significant bits), so the small flux increments of a step
// are not rounded away; slopes, traces and Riemann fluxes are computed in FP32
// from hi.  The update adds the flux balance with TwoSum (Knuth, "The Art of
// Computer Programming" vol. 2, 4.2.2) and renormalises with Fast2Sum
// (Dekker, 1971).  The CFL maximum stays FP64: each block selects its
// largest FP32 wave-speed term and recomputes that cell's term in FP64 from
// hi + lo; blocks combine with an FP64 max.
//
// One launch per time step (k_step_f32c): per 32x16 tile it reads hi of the
// tile and its 2-cell halo (ghost cells through the boundary map, so no fill
// pass), computes primitives, slopes, face states and fluxes in shared
// memory, writes the updated (hi, lo) and folds the next step's CFL maximum
// into the device clock.  Algorithmic traffic: 32 B read + 32 B written per
// cell.
#include "e2d_common.cuh"
#include "e2d_internal.h"

namespace e2d {
namespace {

constexpr int TX = 32;
constexpr int TY = 16;
constexpr int QW = TX + 4;
constexpr int QH = TY + 4;
constexpr int XW = TX + 2;
constexpr int YH = TY + 2;
constexpr int NT = 256;
constexpr size_t kSmemFloats = 4 * QH * QW + 2 * (4 * TY * XW) + 2 * (4 * YH * TX);

// ------------------------------------------------------------ FP32 numerics
// Same equations as the FP64 path (src/HydroBaseFunctor.h), FP32 arithmetic.
__device__ __forceinline__ void prims32(const KPhys<float> &ph, float rho, float e, float mx, float my,
                                        float &d, float &p, float &ux, float &uy) {
  d = fmaxf(rho, ph.smallr);
  const float inv = 1.0f / d;
  ux = mx * inv;
  uy = my * inv;
  const float eken = 0.5f * (ux * ux + uy * uy);
  const float ei = e * inv - eken;
  p = fmaxf(ph.gm1 * d * ei, d * ph.smallp);
}

__device__ __forceinline__ float slope32(int st_kind, float st, float q, float qp, float qm) {
  if (st_kind == 0) return 0.0f;
  const float dlft = st * (q - qm);
  const float drgt = st * (qp - q);
  const float dcen = 0.5f * (qp - qm);
  const float slop = fminf(fabsf(dlft), fabsf(drgt));
  const float dlim = (dlft * drgt <= 0.0f) ? 0.0f : slop;
  const float m = fminf(dlim, fabsf(dcen));
  return dcen >= 0.0f ? m : -m;
}

__device__ __forceinline__ void sources32(const KPhys<float> &ph, const float q[4], const float dqx[4],
                                          const float dqy[4], float s0[4]) {
  const float r = q[E2D_ID], p = q[E2D_IP], u = q[E2D_IU], v = q[E2D_IV];
  const float ir = 1.0f / r;
  const float div = dqx[E2D_IU] + dqy[E2D_IV];
  s0[E2D_ID] = -u * dqx[E2D_ID] - v * dqy[E2D_ID] - div * r;
  s0[E2D_IP] = -u * dqx[E2D_IP] - v * dqy[E2D_IP] - div * ph.gamma0 * p;
  s0[E2D_IU] = -u * dqx[E2D_IU] - v * dqy[E2D_IU] - dqx[E2D_IP] * ir;
  s0[E2D_IV] = -u * dqx[E2D_IV] - v * dqy[E2D_IV] - dqy[E2D_IP] * ir;
}

__device__ __forceinline__ void riemann_hllc32(const KPhys<float> &ph, const float *ql, const float *qr,
                                               float *flux) {
  const float rl = fmaxf(ql[E2D_ID], ph.smallr);
  const float pl = fmaxf(ql[E2D_IP], rl * ph.smallp);
  const float ul = ql[E2D_IU], vl = ql[E2D_IV];
  const float rr = fmaxf(qr[E2D_ID], ph.smallr);
  const float pr = fmaxf(qr[E2D_IP], rr * ph.smallp);
  const float ur = qr[E2D_IU], vr = qr[E2D_IV];
  const float etotl = pl * ph.entho + 0.5f * rl * (ul * ul + vl * vl);
  const float etotr = pr * ph.entho + 0.5f * rr * (ur * ur + vr * vr);
  const float cfastl = sqrtf(fmaxf(ph.gamma0 * pl / rl, ph.smallc2));
  const float cfastr = sqrtf(fmaxf(ph.gamma0 * pr / rr, ph.smallc2));
  const float cmax = fmaxf(cfastl, cfastr);
  const float SL = fminf(ul, ur) - cmax;
  const float SR = fmaxf(ul, ur) + cmax;
  const float rcl = rl * (ul - SL);
  const float rcr = rr * (SR - ur);
  const float iden = 1.0f / (rcr + rcl);
  const float ustar = (rcr * ur + rcl * ul + (pl - pr)) * iden;
  const float ptotstar = (rcr * pl + rcl * pr + rcl * rcr * (ul - ur)) * iden;
  const bool lft = ustar > 0.0f;
  const float S = lft ? SL : SR;
  const float rs = lft ? rl : rr, us = lft ? ul : ur, ps = lft ? pl : pr, es = lft ? etotl : etotr;
  const float sdu = S - us;
  const float isds = 1.0f / (S - ustar);
  const float rstar = rs * sdu * isds;
  const float etotstar = (sdu * es - ps * us + ptotstar * ustar) * isds;
  float ro, uo, ptoto, etoto;
  if (SL > 0.0f) {
    ro = rl, uo = ul, ptoto = pl, etoto = etotl;
  } else if (lft || SR > 0.0f) {
    ro = rstar, uo = ustar, ptoto = ptotstar, etoto = etotstar;
  } else {
    ro = rr, uo = ur, ptoto = pr, etoto = etotr;
  }
  flux[E2D_ID] = ro * uo;
  flux[E2D_IU] = flux[E2D_ID] * uo + ptoto;
  flux[E2D_IP] = (etoto + ptoto) * uo;
  flux[E2D_IV] = flux[E2D_ID] * (flux[E2D_ID] > 0.0f ? vl : vr);
}

__device__ __forceinline__ void riemann_hll32(const KPhys<float> &ph, const float *ql, const float *qr,
                                              float *flux) {
  const float rl = fmaxf(ql[E2D_ID], ph.smallr);
  const float pl = fmaxf(ql[E2D_IP], rl * ph.smallp);
  const float ul = ql[E2D_IU], vl = ql[E2D_IV];
  const float rr = fmaxf(qr[E2D_ID], ph.smallr);
  const float pr = fmaxf(qr[E2D_IP], rr * ph.smallp);
  const float ur = qr[E2D_IU], vr = qr[E2D_IV];
  const float etotl = pl * ph.entho + 0.5f * rl * (ul * ul + vl * vl);
  const float etotr = pr * ph.entho + 0.5f * rr * (ur * ur + vr * vr);
  const float cmax = fmaxf(sqrtf(fmaxf(ph.gamma0 * pl / rl, ph.smallc2)),
                           sqrtf(fmaxf(ph.gamma0 * pr / rr, ph.smallc2)));
  const float SL = fminf(ul, ur) - cmax;
  const float SR = fmaxf(ul, ur) + cmax;
  const float UL[4] = {rl, etotl, rl * ul, rl * vl};
  const float UR[4] = {rr, etotr, rr * ur, rr * vr};
  const float FL[4] = {UL[E2D_IU], (etotl + pl) * ul, UL[E2D_IU] * ul + pl, UL[E2D_IU] * vl};
  const float FR[4] = {UR[E2D_IU], (etotr + pr) * ur, UR[E2D_IU] * ur + pr, UR[E2D_IU] * vr};
  if (SL > 0.0f) {
#pragma unroll
    for (int v = 0; v < 4; ++v) flux[v] = FL[v];
  } else if (SR <= 0.0f) {
#pragma unroll
    for (int v = 0; v < 4; ++v) flux[v] = FR[v];
  } else {
    const float iden = 1.0f / (SR - SL);
    const float sls = SL * SR;
#pragma unroll
    for (int v = 0; v < 4; ++v) flux[v] = (SR * FL[v] - SL * FR[v] + sls * (UR[v] - UL[v])) * iden;
  }
}

__device__ __noinline__ void riemann_approx32(const KPhys<float> &ph, const float *ql, const float *qr,
                                              float *flux) {
  const float gamma0 = ph.gamma0, gamma6 = ph.gamma6;
  const float rl = fmaxf(ql[E2D_ID], ph.smallr), ul = ql[E2D_IU];
  const float pl = fmaxf(ql[E2D_IP], rl * ph.smallp);
  const float rr = fmaxf(qr[E2D_ID], ph.smallr), ur = qr[E2D_IU];
  const float pr = fmaxf(qr[E2D_IP], rr * ph.smallp);
  const float cl = gamma0 * pl * rl, cr = gamma0 * pr * rr;
  float wl = sqrtf(cl), wr = sqrtf(cr);
  float pold = fmaxf(((wr * pl + wl * pr) + wl * wr * (ul - ur)) / (wl + wr), 0.0f);
  float conv = 1.0f;
  for (int iter = 0; iter < 10 && conv > 1e-6f; ++iter) {
    const float wwl = sqrtf(cl * (1.0f + gamma6 * (pold - pl) / pl));
    const float wwr = sqrtf(cr * (1.0f + gamma6 * (pold - pr) / pr));
    const float qxl = 2.0f * wwl * wwl * wwl / (wwl * wwl + cl);
    const float qxr = 2.0f * wwr * wwr * wwr / (wwr * wwr + cr);
    const float usl = ul - (pold - pl) / wwl;
    const float usr = ur + (pold - pr) / wwr;
    const float delp = fmaxf(qxr * qxl / (qxr + qxl) * (usl - usr), -pold);
    pold = pold + delp;
    conv = fabsf(delp / (pold + ph.smallpp));
  }
  const float pstar = pold;
  wl = sqrtf(cl * (1.0f + gamma6 * (pstar - pl) / pl));
  wr = sqrtf(cr * (1.0f + gamma6 * (pstar - pr) / pr));
  const float ustar = 0.5f * (ul + (pl - pstar) / wl + ur - (pr - pstar) / wr);
  const float sgnm = copysignf(1.0f, ustar);
  const bool lft = sgnm > 0.0f;
  const float ro = lft ? rl : rr, uo = lft ? ul : ur, po = lft ? pl : pr, wo = lft ? wl : wr;
  const float co = fmaxf(ph.smallc, sqrtf(fabsf(gamma0 * po / ro)));
  const float rstar = fmaxf(ro / (1.0f + ro * (po - pstar) / (wo * wo)), ph.smallr);
  const float cstar = fmaxf(ph.smallc, sqrtf(fabsf(gamma0 * pstar / rstar)));
  float spout = co - sgnm * uo, spin = cstar - sgnm * ustar;
  const float ushock = wo / ro - sgnm * uo;
  if (pstar >= po) spin = spout = ushock;
  const float scr = fmaxf(spout - spin, ph.smallc + fabsf(spout + spin));
  float frac = 0.5f * (1.0f + (spout + spin) / scr);
  frac = (frac != frac) ? 0.0f : fminf(fmaxf(frac, 0.0f), 1.0f);
  float gd = frac * rstar + (1.0f - frac) * ro;
  float gu = frac * ustar + (1.0f - frac) * uo;
  float gp = frac * pstar + (1.0f - frac) * po;
  if (spout < 0.0f) gd = ro, gu = uo, gp = po;
  if (spin > 0.0f) gd = rstar, gu = ustar, gp = pstar;
  const float gv = lft ? ql[E2D_IV] : qr[E2D_IV];
  flux[E2D_ID] = gd * gu;
  flux[E2D_IU] = flux[E2D_ID] * gu + gp;
  flux[E2D_IV] = flux[E2D_ID] * gv;
  const float etot = gp * ph.entho + 0.5f * gd * (gu * gu + gv * gv);
  flux[E2D_IP] = gu * (etot + gp);
}

template <int RS>
__device__ __forceinline__ void riemann32(const KPhys<float> &ph, const float *ql, const float *qr, float *f) {
  if (RS == E2D_RIEMANN_HLLC)
    riemann_hllc32(ph, ql, qr, f);
  else if (RS == E2D_RIEMANN_HLL)
    riemann_hll32(ph, ql, qr, f);
  else
    riemann_approx32(ph, ql, qr, f);
}

// CFL term of src/HydroRunFunctors.h:56-72 in FP64 from a compensated cell.
__device__ __forceinline__ double cfl_term64(const KPhys<double> &ph, double rho, double e, double mx,
                                             double my) {
  const double d = fmax(rho, ph.smallr);
  const double ux = mx / d, uy = my / d;
  const double eken = 0.5 * (ux * ux + uy * uy);
  const double ei = e / d - eken;
  const double p = fmax(ph.gm1 * d * ei, d * ph.smallp);
  const double c = sqrt(ph.gamma0 * p / d);
  return (c + fabs(ux)) / ph.dx + (c + fabs(uy)) / ph.dy;
}

__device__ __forceinline__ float cfl_term32(const KPhys<float> &ph, float rho, float e, float mx, float my) {
  float d, p, ux, uy;
  prims32(ph, rho, e, mx, my, d, p, ux, uy);
  const float c = sqrtf(ph.gamma0 * p / d);
  return (c + fabsf(ux)) / ph.dx + (c + fabsf(uy)) / ph.dy;
}

// Block arg-max of an FP32 term; the winner's term is recomputed in FP64 from
// its (hi, lo) state in w and folded into *target.  Every thread passes its
// best (term, cell) pair; cell < 0 means none.
__device__ __forceinline__ void block_cfl_fold(const KParams32 &kp, float term, int cell, const float *w,
                                               unsigned long long *target, unsigned int *status) {
  __shared__ float s_term[NT / 32];
  __shared__ int s_cell[NT / 32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float ot = __shfl_xor_sync(0xffffffffu, term, off);
    const int oc = __shfl_xor_sync(0xffffffffu, cell, off);
    if (ot > term || (ot == term && oc > cell)) term = ot, cell = oc;
  }
  const int tid = threadIdx.x;
  if ((tid & 31) == 0) {
    s_term[tid >> 5] = term;
    s_cell[tid >> 5] = cell;
  }
  __syncthreads();
  if (tid == 0) {
    float bt = s_term[0];
    int bc = s_cell[0];
    for (int k = 1; k < NT / 32; ++k)
      if (s_term[k] > bt || (s_term[k] == bt && s_cell[k] > bc)) bt = s_term[k], bc = s_cell[k];
    if (bc >= 0) {
      const long long P = kp.g.plane;
      double u[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) u[v] = (double)w[bc + v * P] + (double)w[bc + (4 + v) * P];
      const double t64 = cfl_term64(kp.ph64, u[E2D_ID], u[E2D_IP], u[E2D_IU], u[E2D_IV]);
      if (t64 > 0.0 && !nonfinite64(t64))
        atomicMax(target, (unsigned long long)__double_as_longlong(t64));
      else
        atomicOr(status, nonfinite64(t64) ? (unsigned)E2D_FLAG_NONFINITE : (unsigned)E2D_FLAG_BAD_DT);
    }
  }
}

// ------------------------------------------------------------ conversions
__global__ void k_f32c_from_f64(const KGeom g, const double *__restrict__ u, float *__restrict__ w) {
  const long long n = g.plane;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const double x = u[k + v * n];
      const float hi = (float)x;
      w[k + v * n] = hi;
      w[k + (4 + v) * n] = (float)(x - (double)hi);
    }
  }
}

// hi + lo in FP64 for every cell; ghost cells through the boundary map (the
// state after make_boundaries).
__global__ void k_f32c_to_f64(const KGeom g, const float *__restrict__ w, double *__restrict__ u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.isize || j >= g.jsize) return;
  bool fu, fv;
  const int si = ghost_source(i, g.nx, g.bc_xmin, g.bc_xmax, fu);
  const int sj = ghost_source(j, g.ny, g.bc_ymin, g.bc_ymax, fv);
  const long long s = si + (long long)g.isize * sj, d = i + (long long)g.isize * j, n = g.plane;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    double x = (double)w[s + v * n] + (double)w[s + (4 + v) * n];
    if ((v == E2D_IU && fu) || (v == E2D_IV && fv)) x = -x;
    u[d + v * n] = x;
  }
}

// CFL maximum of a compensated state.
__global__ void __launch_bounds__(NT) k_f32c_dt(const KParams32 kp, const float *__restrict__ w,
                                                DevClock *clk, const int slot) {
  const KGeom &g = kp.g;
  float best = -1.0f;
  int bcell = -1;
  const long long ncell = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)NT + threadIdx.x; k < ncell; k += (long long)gridDim.x * NT) {
    const int j = (int)(k / g.nx), i = (int)(k - (long long)j * g.nx);
    const int c = (i + 2) + g.isize * (j + 2);
    const float t = cfl_term32(kp.ph, w[c], w[c + g.plane], w[c + 2 * g.plane], w[c + 3 * g.plane]);
    if (t > best) best = t, bcell = c;
  }
  block_cfl_fold(kp, best, bcell, w, slot < 0 ? &clk->invdt_bits : &clk->acc[slot], &clk->status);
}

// ------------------------------------------------------------ the step
template <int RS>
__global__ void __launch_bounds__(NT, 4)
    k_step_f32c(const KParams32 kp, const float *__restrict__ w_in, float *__restrict__ w_out,
                DevClock *clk, const int use_clock, const double host_dt, double *__restrict__ dt_trace) {
  extern __shared__ float sm[];
  float *sQ = sm;                    // [4][QH][QW]
  float *sXm = sQ + 4 * QH * QW;     // [4][TY][XW] XMIN states, then x-fluxes
  float *sXp = sXm + 4 * TY * XW;    // [4][TY][XW] XMAX states
  float *sYm = sXp + 4 * TY * XW;    // [4][YH][TX] YMIN states, then y-fluxes
  float *sYp = sYm + 4 * YH * TX;    // [4][YH][TX] YMAX states

  const KGeom &g = kp.g;
  const KPhys<float> &ph = kp.ph;
  const int tid = threadIdx.x;
  const long long P = g.plane;

  // dt of this step (FP64, src/main.cpp:128-134), computed by one thread: the
  // FP64 pipe runs at 1/70 of the FP32 rate, so per-thread divisions here
  // would dominate the kernel
  __shared__ double s_dt[3];
  __shared__ int s_run, s_slot;
  if (tid == 0) {
    double dt = host_dt, t = 0.0;
    int run = 1, slot = 0;
    if (use_clock) {
      t = clk->t;
      const double t_end = clk->t_end;
      run = t < t_end;
      slot = clk->nstep & 1;
      const double inv_dt = __longlong_as_double((long long)clk->acc[slot]);
      dt = kp.ph64.cfl / inv_dt;
      if (t + dt > t_end) dt = t_end - t;
    }
    s_dt[0] = dt;
    s_dt[1] = dt / kp.ph64.dx;
    s_dt[2] = dt / kp.ph64.dy;
    s_run = run;
    s_slot = slot;
  }
  __syncthreads();
  if (!s_run) return;
  const double dt = s_dt[0];
  const int slot = s_slot;
  const float dtdx = (float)s_dt[1];
  const float dtdy = (float)s_dt[2];
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;

  // stage 1: primitives of the tile and its halo; ghosts via the boundary map
  for (int k = tid; k < QH * QW; k += NT) {
    const int y = k / QW, x = k - y * QW;
    int gi = i0 + x, gj = j0 + y;
    if (gi >= g.isize) gi = g.isize - 1;
    if (gj >= g.jsize) gj = g.jsize - 1;
    bool fu, fv;
    const int si = ghost_source(gi, g.nx, g.bc_xmin, g.bc_xmax, fu);
    const int sj = ghost_source(gj, g.ny, g.bc_ymin, g.bc_ymax, fv);
    const long long s = si + (long long)g.isize * sj;
    const float rho = w_in[s], e = w_in[s + P];
    float mx = w_in[s + 2 * P], my = w_in[s + 3 * P];
    if (fu) mx = -mx;
    if (fv) my = -my;
    float d, p, ux, uy;
    prims32(ph, rho, e, mx, my, d, p, ux, uy);
    sQ[k] = d;
    sQ[QH * QW + k] = p;
    sQ[2 * QH * QW + k] = ux;
    sQ[3 * QH * QW + k] = uy;
  }
  __syncthreads();

  // stage 2: slopes, sources and face states
  const int st_kind = (ph.slope_type == 2.0f) ? 2 : (ph.slope_type == 1.0f) ? 1 : 0;
  const float st = ph.slope_type;
  for (int k = tid; k < YH * XW; k += NT) {
    const int yy = k / XW, xx = k - yy * XW;
    const bool xin = (xx >= 1) && (xx <= TX);
    const bool yin = (yy >= 1) && (yy <= TY);
    if (!xin && !yin) continue;
    const int c = (yy + 1) * QW + (xx + 1);
    float qc[4], dqx[4], dqy[4], s0[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const float *Pq = sQ + v * QH * QW;
      qc[v] = Pq[c];
      dqx[v] = slope32(st_kind, st, qc[v], Pq[c + 1], Pq[c - 1]);
      dqy[v] = slope32(st_kind, st, qc[v], Pq[c + QW], Pq[c - QW]);
    }
    sources32(ph, qc, dqx, dqy, s0);
    if (yin) {
      const int o = (yy - 1) * XW + xx;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float h = 0.5f * dqx[v], sx = 0.5f * s0[v] * dtdx;
        float fm = qc[v] - h + sx, fp = qc[v] + h + sx;
        if (v == E2D_ID) fm = fmaxf(fm, ph.smallr), fp = fmaxf(fp, ph.smallr);
        if (xx >= 1) sXm[v * TY * XW + o] = fm;
        if (xx <= TX) sXp[v * TY * XW + o] = fp;
      }
    }
    if (xin) {
      const int o = yy * TX + (xx - 1);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float h = 0.5f * dqy[v], sy = 0.5f * s0[v] * dtdy;
        float fm = qc[v] - h + sy, fp = qc[v] + h + sy;
        if (v == E2D_ID) fm = fmaxf(fm, ph.smallr), fp = fmaxf(fp, ph.smallr);
        if (yy >= 1) sYm[v * YH * TX + o] = fm;
        if (yy <= TY) sYp[v * YH * TX + o] = fp;
      }
    }
  }
  __syncthreads();

  // stage 3: Riemann solves; scaled fluxes replace the right-hand states
  constexpr int NXF = (TX + 1) * TY;
  constexpr int NYF = TX * (TY + 1);
  for (int k = tid; k < NXF + NYF; k += NT) {
    float ql[4], qr[4], f[4];
    if (k < NXF) {
      const int y = k / (TX + 1), fx = k - y * (TX + 1);
      const int ol = y * XW + fx, orr = ol + 1;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        ql[v] = sXp[v * TY * XW + ol];
        qr[v] = sXm[v * TY * XW + orr];
      }
      riemann32<RS>(ph, ql, qr, f);
#pragma unroll
      for (int v = 0; v < 4; ++v) sXm[v * TY * XW + orr] = f[v] * dtdx;
    } else {
      const int kk = k - NXF;
      const int fy = kk / TX, x = kk - fy * TX;
      const int ol = fy * TX + x, orr = ol + TX;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int vs = (v == E2D_IU) ? E2D_IV : (v == E2D_IV) ? E2D_IU : v;
        ql[vs] = sYp[v * YH * TX + ol];
        qr[vs] = sYm[v * YH * TX + orr];
      }
      riemann32<RS>(ph, ql, qr, f);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int vs = (v == E2D_IU) ? E2D_IV : (v == E2D_IV) ? E2D_IU : v;
        sYm[v * YH * TX + orr] = f[vs] * dtdy;
      }
    }
  }
  __syncthreads();

  // stage 4: compensated update and the next step's CFL term
  float best = -1.0f;
  int bcell = -1;
  for (int k = tid; k < TX * TY; k += NT) {
    const int y = k / TX, x = k - y * TX;
    const int gi = i0 + 2 + x, gj = j0 + 2 + y;
    if (gi < g.nx + 2 && gj < g.ny + 2) {
      const long long s = gi + (long long)g.isize * gj;
      float nh[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float du = (sXm[v * TY * XW + y * XW + x + 1] - sXm[v * TY * XW + y * XW + x + 2]) +
                         (sYm[v * YH * TX + (y + 1) * TX + x] - sYm[v * YH * TX + (y + 2) * TX + x]);
        const float hi = w_in[s + v * P];
        float lo = w_in[s + (4 + v) * P];
        // TwoSum(hi, du)
        const float sum = hi + du;
        const float bb = sum - hi;
        const float err = (hi - (sum - bb)) + (du - bb);
        lo = lo + err;
        // Fast2Sum(sum, lo), |sum| >= |lo|
        const float h2 = sum + lo;
        const float l2 = lo - (h2 - sum);
        w_out[s + v * P] = h2;
        w_out[s + (4 + v) * P] = l2;
        nh[v] = h2;
      }
      if (use_clock) {
        const float tt = cfl_term32(ph, nh[E2D_ID], nh[E2D_IP], nh[E2D_IU], nh[E2D_IV]);
        if (tt > best) best = tt, bcell = (int)s;
      }
    }
  }
  if (!use_clock) return;
  __syncthreads();  // this block's writes of w_out are visible to thread 0
  block_cfl_fold(kp, best, bcell, w_out, &clk->acc[slot ^ 1], &clk->status);

  // the last block to finish advances the loop state (src/main.cpp:139-143)
  if (tid == 0) {
    __threadfence();
    const unsigned int nblocks = gridDim.x * gridDim.y;
    const unsigned int ticket = atomicAdd(&clk->done_blocks, 1u);
    if (ticket == nblocks - 1) {
      __threadfence();
      const int ns = clk->nstep;
      const int tslot = ns - clk->trace_base;
      if (dt_trace && tslot >= 0 && tslot < clk->trace_cap) dt_trace[tslot] = dt;
      if (!(dt > 0.0) || nonfinite64(dt)) clk->status |= E2D_FLAG_BAD_DT;
      clk->dt = dt;
      clk->t = clk->t + dt;  // only this block writes t during the step
      clk->nstep = ns + 1;
      clk->acc[slot] = 0ull;
      clk->done_blocks = 0u;
      __threadfence();
    }
  }
}

}  // namespace

void make_kparams32(const e2d_params &p, KParams32 *kp) {
  KParams64 k64;
  make_kparams(p, &k64);
  kp->g = k64.g;
  kp->ph64 = k64.ph;
  const KPhys<double> &d = k64.ph;
  kp->ph = KPhys<float>{(float)d.gamma0, (float)d.gamma6, (float)d.cfl, (float)d.slope_type,
                        (float)d.smallr, (float)d.smallc, (float)d.smallp, (float)d.smallpp,
                        (float)d.gm1, (float)d.entho, (float)d.smallc2, (float)d.dx, (float)d.dy};
}

cudaError_t configure_f32c_kernels() {
  const int smem = (int)(kSmemFloats * sizeof(float));
  cudaError_t e = cudaFuncSetAttribute(k_step_f32c<E2D_RIEMANN_HLLC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_step_f32c<E2D_RIEMANN_HLL>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_step_f32c<E2D_RIEMANN_APPROX>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

cudaError_t launch_f32c_from_f64(const KParams32 &kp, const double *u, float *w, cudaStream_t s) {
  const long long n = kp.g.plane;
  const int blocks = (int)((n + 255) / 256 < 65535 * 8 ? (n + 255) / 256 : 65535 * 8);
  k_f32c_from_f64<<<blocks, 256, 0, s>>>(kp.g, u, w);
  return cudaGetLastError();
}

cudaError_t launch_f32c_to_f64(const KParams32 &kp, const float *w, double *u, cudaStream_t s) {
  dim3 block(64, 4);
  dim3 grid((kp.g.isize + 63) / 64, (kp.g.jsize + 3) / 4);
  k_f32c_to_f64<<<grid, block, 0, s>>>(kp.g, w, u);
  return cudaGetLastError();
}

cudaError_t launch_f32c_dt(const KParams32 &kp, const float *w, DevClock *clk, int slot, cudaStream_t s) {
  const long long ncell = (long long)kp.g.nx * kp.g.ny;
  long long blocks = (ncell + NT - 1) / NT;
  if (blocks > 152 * 32) blocks = 152 * 32;
  k_f32c_dt<<<(int)blocks, NT, 0, s>>>(kp, w, clk, slot);
  return cudaGetLastError();
}

cudaError_t launch_f32c_step(const KParams32 &kp, int riemann, const float *w_in, float *w_out,
                             DevClock *clk, int use_clock, double host_dt, double *dt_trace,
                             cudaStream_t s) {
  dim3 grid((kp.g.nx + TX - 1) / TX, (kp.g.ny + TY - 1) / TY);
  const size_t smem = kSmemFloats * sizeof(float);
  switch (riemann) {
    case E2D_RIEMANN_HLLC:
      k_step_f32c<E2D_RIEMANN_HLLC><<<grid, NT, smem, s>>>(kp, w_in, w_out, clk, use_clock, host_dt, dt_trace);
      break;
    case E2D_RIEMANN_HLL:
      k_step_f32c<E2D_RIEMANN_HLL><<<grid, NT, smem, s>>>(kp, w_in, w_out, clk, use_clock, host_dt, dt_trace);
      break;
    default:
      k_step_f32c<E2D_RIEMANN_APPROX><<<grid, NT, smem, s>>>(kp, w_in, w_out, clk, use_clock, host_dt, dt_trace);
      break;
  }
  return cudaGetLastError();
}

}  // namespace e2d
