// e2d_fp64_blocks.cuh -- the building blocks of the FP64 step, bit-identical
// to the reference's FP64 arithmetic (compile with --fmad=false; every
// expression keeps the reference's operation order): primitives, limited
// slopes, the half-step trace, the three Riemann solvers and the CFL term.
// Shared by the fused / two-launch step kernels (e2d_fp64.cu) and the
// implementation-1/2 orchestrations (e2d_impl12.cu).
#pragma once

#include "e2d_common.cuh"
#include "e2d_f64_exact.cuh"
#include "e2d_internal.h"

namespace e2d {
namespace {

using f64x::gt0;
using f64x::half;
using f64x::max_nn;
using f64x::max_pos;
using f64x::max_any;
using f64x::min_any;

__device__ __forceinline__ int src_lo_hi(int i, int n, int bc_lo, int bc_hi, bool &flip) {
  return ghost_source(i, n, bc_lo, bc_hi, flip);
}
__device__ __forceinline__ bool nonfinite(double x) { return nonfinite64(x); }

// ------------------------------------------------------------ numerics
// src/HydroBaseFunctor.h:76-102 (computePrimitives) without the sound speed.
__device__ __forceinline__ void primitives(const KPhys<double> &ph, double rho, double e, double mx,
                                           double my, double &d, double &p, double &ux, double &uy) {
  d = max_pos(rho, ph.smallr);
  ux = mx / d;
  uy = my / d;
  const double eken = half(ux * ux + uy * uy);
  const double ei = e / d - eken;
  p = max_pos(ph.gm1 * d * ei, d * ph.smallp);
}

// src/HydroBaseFunctor.h:475-516 for one variable and direction: slope_type
// 0 gives a zero slope, 1 and 2 the limited slope.
__device__ __forceinline__ double slope(int st_kind, double q, double qp, double qm) {
  if (st_kind == 0) return 0.0;
  return f64x::slope_limited(st_kind == 2, q, qp, qm);
}

// Sources of trace_unsplit_2d_along_dir (src/HydroBaseFunctor.h:246-249).
__device__ __forceinline__ void trace_sources(const KPhys<double> &ph, const double q[4],
                                              const double dqx[4], const double dqy[4], double s0[4]) {
  const double r = q[E2D_ID], p = q[E2D_IP], u = q[E2D_IU], v = q[E2D_IV];
  const double drx = dqx[E2D_ID], dpx = dqx[E2D_IP], dux = dqx[E2D_IU], dvx = dqx[E2D_IV];
  const double dry = dqy[E2D_ID], dpy = dqy[E2D_IP], duy = dqy[E2D_IU], dvy = dqy[E2D_IV];
  s0[E2D_ID] = -u * drx - v * dry - (dux + dvy) * r;
  s0[E2D_IP] = -u * dpx - v * dpy - (dux + dvy) * ph.gamma0 * p;
  s0[E2D_IU] = -u * dux - v * duy - (dpx) / r;
  s0[E2D_IV] = -u * dvx - v * dvy - (dpy) / r;
}

// The two face states of one direction (src/HydroBaseFunctor.h:251-289):
// minus face q - dq/2 + s0*dtd/2, plus face q + dq/2 + s0*dtd/2, density
// clamped at smallr.
__device__ __forceinline__ void face_pair(const KPhys<double> &ph, int v, double q, double dq,
                                          double s0, double dtd, double &fm, double &fp) {
  const double h = half(dq);
  const double sx = half(s0 * dtd);
  fm = q - h + sx;
  fp = q + h + sx;
  if (v == E2D_ID) {
    fm = max_pos(fm, ph.smallr);
    fp = max_pos(fp, ph.smallr);
  }
}

// src/HydroBaseFunctor.h:523-547.
__device__ __forceinline__ void cmpflx(const KPhys<double> &ph, const double g[4], double f[4]) {
  f[E2D_ID] = g[E2D_ID] * g[E2D_IU];
  f[E2D_IU] = f[E2D_ID] * g[E2D_IU] + g[E2D_IP];
  f[E2D_IV] = f[E2D_ID] * g[E2D_IV];
  const double ekin = 0.5 * g[E2D_ID] * (g[E2D_IU] * g[E2D_IU] + g[E2D_IV] * g[E2D_IV]);
  const double etot = g[E2D_IP] * ph.entho + ekin;
  f[E2D_IP] = g[E2D_IU] * (etot + g[E2D_IP]);
}

// src/HydroBaseFunctor.h:558-693 (riemann_approx).
__device__ __noinline__ void riemann_approx(const KPhys<double> &ph, const double *ql,
                                            const double *qr, double *flux) {
  const double gamma0 = ph.gamma0, gamma6 = ph.gamma6;
  const double rl = fmax(ql[E2D_ID], ph.smallr), ul = ql[E2D_IU];
  const double pl = fmax(ql[E2D_IP], rl * ph.smallp);
  const double rr = fmax(qr[E2D_ID], ph.smallr), ur = qr[E2D_IU];
  const double pr = fmax(qr[E2D_IP], rr * ph.smallp);
  const double cl = gamma0 * pl * rl;
  const double cr = gamma0 * pr * rr;
  double wl = sqrt(cl);
  double wr = sqrt(cr);
  double pstar = fmax(((wr * pl + wl * pr) + wl * wr * (ul - ur)) / (wl + wr), 0.0);
  double pold = pstar;
  double conv = 1.0;
  for (int iter = 0; (iter < 10) && (conv > 1e-6); ++iter) {
    const double wwl = sqrt(cl * (1.0 + gamma6 * (pold - pl) / pl));
    const double wwr = sqrt(cr * (1.0 + gamma6 * (pold - pr) / pr));
    const double qxl = 2.0 * wwl * wwl * wwl / (wwl * wwl + cl);
    const double qxr = 2.0 * wwr * wwr * wwr / (wwr * wwr + cr);
    const double usl = ul - (pold - pl) / wwl;
    const double usr = ur + (pold - pr) / wwr;
    const double delp = fmax(qxr * qxl / (qxr + qxl) * (usl - usr), -pold);
    pold = pold + delp;
    conv = fabs(delp / (pold + ph.smallpp));
  }
  pstar = pold;
  wl = sqrt(cl * (1.0 + gamma6 * (pstar - pl) / pl));
  wr = sqrt(cr * (1.0 + gamma6 * (pstar - pr) / pr));
  const double ustar = 0.5 * (ul + (pl - pstar) / wl + ur - (pr - pstar) / wr);
  const double sgnm = copysign(1.0, ustar);
  const bool lft = sgnm > 0.0;
  const double ro = lft ? rl : rr, uo = lft ? ul : ur, po = lft ? pl : pr, wo = lft ? wl : wr;
  const double co = fmax(ph.smallc, sqrt(fabs(gamma0 * po / ro)));
  const double rstar = fmax((ro / (1.0 + ro * (po - pstar) / (wo * wo))), ph.smallr);
  const double cstar = fmax(ph.smallc, sqrt(fabs(gamma0 * pstar / rstar)));
  double spout = co - sgnm * uo;
  double spin = cstar - sgnm * ustar;
  const double ushock = wo / ro - sgnm * uo;
  if (pstar >= po) {
    spin = ushock;
    spout = ushock;
  }
  const double scr = fmax(spout - spin, ph.smallc + fabs(spout + spin));
  double frac = 0.5 * (1.0 + (spout + spin) / scr);
  if (frac != frac)
    frac = 0.0;
  else
    frac = frac >= 1.0 ? 1.0 : frac <= 0.0 ? 0.0 : frac;
  double g[4];
  g[E2D_ID] = frac * rstar + (1.0 - frac) * ro;
  g[E2D_IU] = frac * ustar + (1.0 - frac) * uo;
  g[E2D_IP] = frac * pstar + (1.0 - frac) * po;
  if (spout < 0.0) {
    g[E2D_ID] = ro;
    g[E2D_IU] = uo;
    g[E2D_IP] = po;
  }
  if (spin > 0.0) {
    g[E2D_ID] = rstar;
    g[E2D_IU] = ustar;
    g[E2D_IP] = pstar;
  }
  g[E2D_IV] = lft ? ql[E2D_IV] : qr[E2D_IV];
  cmpflx(ph, g, flux);
}

// src/HydroBaseFunctor.h:704-809 (riemann_hllc).  The reference builds the
// star states of both sides and keeps one; here only the star state of the
// side the contact selects (ustar > 0: left) is built, which yields the same
// value.  Cut-offs,
// maxima, the 0.5 factors and the sign tests use the exact integer forms of
// e2d_f64_exact.cuh.
__device__ __forceinline__ void riemann_hllc(const KPhys<double> &ph, const double *ql,
                                             const double *qr, double *flux) {
  const double rl = max_pos(ql[E2D_ID], ph.smallr);
  const double pl = max_pos(ql[E2D_IP], rl * ph.smallp);
  const double ul = ql[E2D_IU];
  const double hrl = half(rl);
  double ecinl = hrl * ul * ul;
  ecinl = ecinl + hrl * ql[E2D_IV] * ql[E2D_IV];
  const double etotl = pl * ph.entho + ecinl;
  const double rr = max_pos(qr[E2D_ID], ph.smallr);
  const double pr = max_pos(qr[E2D_IP], rr * ph.smallp);
  const double ur = qr[E2D_IU];
  const double hrr = half(rr);
  double ecinr = hrr * ur * ur;
  ecinr = ecinr + hrr * qr[E2D_IV] * qr[E2D_IV];
  const double etotr = pr * ph.entho + ecinr;
  const double cfastl = sqrt(max_pos(ph.gamma0 * pl / rl, ph.smallc2));
  const double cfastr = sqrt(max_pos(ph.gamma0 * pr / rr, ph.smallc2));
  const double cmax = max_nn(cfastl, cfastr);
  const double SL = min_any(ul, ur) - cmax;
  const double SR = max_any(ul, ur) + cmax;
  const double rcl = rl * (ul - SL);
  const double rcr = rr * (SR - ur);
  const double ustar = (rcr * ur + rcl * ul + (pl - pr)) / (rcr + rcl);
  const double ptotstar = (rcr * pl + rcl * pr + rcl * rcr * (ul - ur)) / (rcr + rcl);
  const bool lft = gt0(ustar);
  const double S = lft ? SL : SR;
  const double rs = lft ? rl : rr, us = lft ? ul : ur, ps = lft ? pl : pr;
  const double es = lft ? etotl : etotr;
  const double sdu = S - us;
  const double sds = S - ustar;
  const double rstar = rs * sdu / sds;
  const double etotstar = (sdu * es - ps * us + ptotstar * ustar) / sds;
  double ro, uo, ptoto, etoto;
  if (gt0(SL)) {
    ro = rl, uo = ul, ptoto = pl, etoto = etotl;
  } else if (lft || gt0(SR)) {
    ro = rstar, uo = ustar, ptoto = ptotstar, etoto = etotstar;
  } else {
    ro = rr, uo = ur, ptoto = pr, etoto = etotr;
  }
  flux[E2D_ID] = ro * uo;
  flux[E2D_IU] = flux[E2D_ID] * uo + ptoto;
  flux[E2D_IP] = (etoto + ptoto) * uo;
  flux[E2D_IV] = gt0(flux[E2D_ID]) ? flux[E2D_ID] * ql[E2D_IV] : flux[E2D_ID] * qr[E2D_IV];
}

// HLL flux (Harten, Lax, van Leer; Toro, "Riemann Solvers and Numerical
// Methods for Fluid Dynamics", 3rd ed., eq. 10.21).  The reference declares
// RIEMANN_HLL but has no solver; this uses riemann_hllc's cut-offs and Davis
// wave speeds; the star flux multiplies by one reciprocal of SR - SL.
// Operation order matches the oracle's riemann_hll.
__device__ __forceinline__ void riemann_hll(const KPhys<double> &ph, const double *ql,
                                            const double *qr, double *flux) {
  const double rl = max_pos(ql[E2D_ID], ph.smallr);
  const double pl = max_pos(ql[E2D_IP], rl * ph.smallp);
  const double ul = ql[E2D_IU], vl = ql[E2D_IV];
  const double rr = max_pos(qr[E2D_ID], ph.smallr);
  const double pr = max_pos(qr[E2D_IP], rr * ph.smallp);
  const double ur = qr[E2D_IU], vr = qr[E2D_IV];
  const double hrl = half(rl), hrr = half(rr);
  double ecinl = hrl * ul * ul;
  ecinl = ecinl + hrl * vl * vl;
  const double etotl = pl * ph.entho + ecinl;
  double ecinr = hrr * ur * ur;
  ecinr = ecinr + hrr * vr * vr;
  const double etotr = pr * ph.entho + ecinr;
  const double cfastl = sqrt(max_pos(ph.gamma0 * pl / rl, ph.smallc2));
  const double cfastr = sqrt(max_pos(ph.gamma0 * pr / rr, ph.smallc2));
  const double cmax = max_nn(cfastl, cfastr);
  const double SL = min_any(ul, ur) - cmax;
  const double SR = max_any(ul, ur) + cmax;
  const double UL[4] = {rl, etotl, rl * ul, rl * vl};
  const double UR[4] = {rr, etotr, rr * ur, rr * vr};
  double FL[4], FR[4];
  FL[E2D_ID] = UL[E2D_IU];
  FL[E2D_IP] = (etotl + pl) * ul;
  FL[E2D_IU] = UL[E2D_IU] * ul + pl;
  FL[E2D_IV] = UL[E2D_IU] * vl;
  FR[E2D_ID] = UR[E2D_IU];
  FR[E2D_IP] = (etotr + pr) * ur;
  FR[E2D_IU] = UR[E2D_IU] * ur + pr;
  FR[E2D_IV] = UR[E2D_IU] * vr;
  if (gt0(SL)) {
#pragma unroll
    for (int v = 0; v < 4; ++v) flux[v] = FL[v];
  } else if (f64x::le0(SR)) {
#pragma unroll
    for (int v = 0; v < 4; ++v) flux[v] = FR[v];
  } else {
    // one division: the four star fluxes share the factor 1 / (SR - SL)
    const double sls = SL * SR;
    const double rden = 1.0 / (SR - SL);
#pragma unroll
    for (int v = 0; v < 4; ++v) flux[v] = (SR * FL[v] - SL * FR[v] + sls * (UR[v] - UL[v])) * rden;
  }
}

template <int RS>
__device__ __forceinline__ void riemann(const KPhys<double> &ph, const double *ql, const double *qr,
                                        double *flux) {
  if (RS == E2D_RIEMANN_HLLC)
    riemann_hllc(ph, ql, qr, flux);
  else if (RS == E2D_RIEMANN_HLL)
    riemann_hll(ph, ql, qr, flux);
  else
    riemann_approx(ph, ql, qr, flux);
}

// CFL wave-speed term of a cell from its primitives (src/HydroRunFunctors.h:56-72):
// (c + |u|) / dx + (c + |v|) / dy, c = sqrt(gamma p / d); a division by a
// power-of-two dx, dy is the exact product by its reciprocal.
__device__ __forceinline__ double cfl_term(const KPhys<double> &ph, double dd, double p, double ux, double uy) {
  const double c = sqrt(ph.gamma0 * p / dd);
  const double vx = c + fabs(ux);
  const double vy = c + fabs(uy);
  const double tx = ph.inv_dx_pow2 != 0.0 ? vx * ph.inv_dx_pow2 : vx / ph.dx;
  const double ty = ph.inv_dy_pow2 != 0.0 ? vy * ph.inv_dy_pow2 : vy / ph.dy;
  return tx + ty;
}

// E2D_FLAG_* bits of a cell's conserved values.
__device__ __forceinline__ unsigned int state_flags(double rho, double e, double mx, double my) {
  unsigned int f = 0;
  if (nonfinite(rho) || nonfinite(e) || nonfinite(mx) || nonfinite(my)) f |= E2D_FLAG_NONFINITE;
  if (!(rho > 0.0)) f |= E2D_FLAG_DENSITY;
  return f;
}


// ------------------------------------------------------------ fast forms
// The opt-in E2D_PRECISION_FP64_FAST step: the same formulas with a*b + c
// contracted into one FMA where it falls naturally and every division
// replaced by a product with a reciprocal computed once per denominator.
// Results differ from the reference's by rounding (not bit-identical); the
// tests hold them to 1e-12 on dt and 1e-10 relative L1.

// 1/b: the hardware estimate (rcp.approx.ftz.f64) refined by two
// Newton-Raphson iterations for f(y) = 1/y - b, y <- y + y (1 - b y), each
// of which roughly doubles the number of correct bits.  For normal b
// (denominators here are densities >= smallr and sums of positive terms).
__device__ __forceinline__ double rcp_nr(double b) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(b));
  double e = fma(-b, y, 1.0);
  y = fma(y, e, y);
  e = fma(-b, y, 1.0);
  return fma(y, e, y);
}

// primitives() with one reciprocal of the density (returned in rd).
__device__ __forceinline__ void primitives_fast(const KPhys<double> &ph, double rho, double e, double mx,
                                                double my, double &d, double &p, double &ux, double &uy,
                                                double &rd) {
  d = max_pos(rho, ph.smallr);
  rd = rcp_nr(d);
  ux = mx * rd;
  uy = my * rd;
  const double ei = fma(e, rd, -0.5 * fma(ux, ux, uy * uy));
  p = max_pos(ph.gm1 * d * ei, d * ph.smallp);
}

__device__ __forceinline__ void trace_sources_fast(const KPhys<double> &ph, const double q[4], const double dqx[4],
                                                   const double dqy[4], double s0[4]) {
  const double r = q[E2D_ID], p = q[E2D_IP], u = q[E2D_IU], v = q[E2D_IV];
  const double div = dqx[E2D_IU] + dqy[E2D_IV];
  const double ir = rcp_nr(r);
  s0[E2D_ID] = fma(-u, dqx[E2D_ID], fma(-v, dqy[E2D_ID], -div * r));
  s0[E2D_IP] = fma(-u, dqx[E2D_IP], fma(-v, dqy[E2D_IP], -div * ph.gamma0 * p));
  s0[E2D_IU] = fma(-u, dqx[E2D_IU], fma(-v, dqy[E2D_IU], -dqx[E2D_IP] * ir));
  s0[E2D_IV] = fma(-u, dqx[E2D_IV], fma(-v, dqy[E2D_IV], -dqy[E2D_IP] * ir));
}

// face_pair() with hdtd = dt/dx / 2 (or dt/dy / 2).
__device__ __forceinline__ void face_pair_fast(const KPhys<double> &ph, int v, double q, double dq, double s0,
                                               double hdtd, double &fm, double &fp) {
  const double qs = fma(s0, hdtd, q);
  fm = fma(dq, -0.5, qs);
  fp = fma(dq, 0.5, qs);
  if (v == E2D_ID) {
    fm = max_pos(fm, ph.smallr);
    fp = max_pos(fp, ph.smallr);
  }
}

// riemann_hllc() with shared reciprocals: 1 / rl, 1 / rr, 1 / (rcr + rcl)
// for u* and p*, 1 / (S - u*) for the star density and energy.
__device__ __forceinline__ void riemann_hllc_fast(const KPhys<double> &ph, const double *ql, const double *qr,
                                                  double *flux) {
  const double rl = max_pos(ql[E2D_ID], ph.smallr);
  const double pl = max_pos(ql[E2D_IP], rl * ph.smallp);
  const double ul = ql[E2D_IU];
  const double etotl = fma(pl, ph.entho, 0.5 * rl * fma(ul, ul, ql[E2D_IV] * ql[E2D_IV]));
  const double rr = max_pos(qr[E2D_ID], ph.smallr);
  const double pr = max_pos(qr[E2D_IP], rr * ph.smallp);
  const double ur = qr[E2D_IU];
  const double etotr = fma(pr, ph.entho, 0.5 * rr * fma(ur, ur, qr[E2D_IV] * qr[E2D_IV]));
  const double cfastl = sqrt(max_pos(ph.gamma0 * pl * rcp_nr(rl), ph.smallc2));
  const double cfastr = sqrt(max_pos(ph.gamma0 * pr * rcp_nr(rr), ph.smallc2));
  const double cmax = max_nn(cfastl, cfastr);
  const double SL = min_any(ul, ur) - cmax;
  const double SR = max_any(ul, ur) + cmax;
  const double rcl = rl * (ul - SL);
  const double rcr = rr * (SR - ur);
  const double isum = rcp_nr(rcr + rcl);
  const double ustar = fma(rcr, ur, fma(rcl, ul, pl - pr)) * isum;
  const double ptotstar = fma(rcr, pl, fma(rcl, pr, rcl * rcr * (ul - ur))) * isum;
  const bool lft = gt0(ustar);
  const double S = lft ? SL : SR;
  const double rs = lft ? rl : rr, us = lft ? ul : ur, ps = lft ? pl : pr;
  const double es = lft ? etotl : etotr;
  const double sdu = S - us;
  const double isds = rcp_nr(S - ustar);
  const double rstar = rs * sdu * isds;
  const double etotstar = fma(sdu, es, fma(-ps, us, ptotstar * ustar)) * isds;
  double ro, uo, ptoto, etoto;
  if (gt0(SL)) {
    ro = rl, uo = ul, ptoto = pl, etoto = etotl;
  } else if (lft || gt0(SR)) {
    ro = rstar, uo = ustar, ptoto = ptotstar, etoto = etotstar;
  } else {
    ro = rr, uo = ur, ptoto = pr, etoto = etotr;
  }
  flux[E2D_ID] = ro * uo;
  flux[E2D_IU] = fma(flux[E2D_ID], uo, ptoto);
  flux[E2D_IP] = (etoto + ptoto) * uo;
  flux[E2D_IV] = gt0(flux[E2D_ID]) ? flux[E2D_ID] * ql[E2D_IV] : flux[E2D_ID] * qr[E2D_IV];
}

// riemann_hll() with FMAs and reciprocals of rl, rr.
__device__ __forceinline__ void riemann_hll_fast(const KPhys<double> &ph, const double *ql, const double *qr,
                                                 double *flux) {
  const double rl = max_pos(ql[E2D_ID], ph.smallr);
  const double pl = max_pos(ql[E2D_IP], rl * ph.smallp);
  const double ul = ql[E2D_IU], vl = ql[E2D_IV];
  const double rr = max_pos(qr[E2D_ID], ph.smallr);
  const double pr = max_pos(qr[E2D_IP], rr * ph.smallp);
  const double ur = qr[E2D_IU], vr = qr[E2D_IV];
  const double etotl = fma(pl, ph.entho, 0.5 * rl * fma(ul, ul, vl * vl));
  const double etotr = fma(pr, ph.entho, 0.5 * rr * fma(ur, ur, vr * vr));
  const double cfastl = sqrt(max_pos(ph.gamma0 * pl * rcp_nr(rl), ph.smallc2));
  const double cfastr = sqrt(max_pos(ph.gamma0 * pr * rcp_nr(rr), ph.smallc2));
  const double cmax = max_nn(cfastl, cfastr);
  const double SL = min_any(ul, ur) - cmax;
  const double SR = max_any(ul, ur) + cmax;
  const double UL[4] = {rl, etotl, rl * ul, rl * vl};
  const double UR[4] = {rr, etotr, rr * ur, rr * vr};
  const double FL[4] = {UL[E2D_IU], (etotl + pl) * ul, fma(UL[E2D_IU], ul, pl), UL[E2D_IU] * vl};
  const double FR[4] = {UR[E2D_IU], (etotr + pr) * ur, fma(UR[E2D_IU], ur, pr), UR[E2D_IU] * vr};
  if (gt0(SL)) {
#pragma unroll
    for (int v = 0; v < 4; ++v) flux[v] = FL[v];
  } else if (f64x::le0(SR)) {
#pragma unroll
    for (int v = 0; v < 4; ++v) flux[v] = FR[v];
  } else {
    const double sls = SL * SR;
    const double rden = rcp_nr(SR - SL);
#pragma unroll
    for (int v = 0; v < 4; ++v) flux[v] = fma(sls, UR[v] - UL[v], fma(SR, FL[v], -SL * FR[v])) * rden;
  }
}

template <int RS, bool FAST>
__device__ __forceinline__ void riemann_sel(const KPhys<double> &ph, const double *ql, const double *qr,
                                            double *flux) {
  if (FAST && RS == E2D_RIEMANN_HLLC)
    riemann_hllc_fast(ph, ql, qr, flux);
  else if (FAST && RS == E2D_RIEMANN_HLL)
    riemann_hll_fast(ph, ql, qr, flux);
  else
    riemann<RS>(ph, ql, qr, flux);
}

// cfl_term() from the reciprocal of the density.
__device__ __forceinline__ double cfl_term_fast(const KPhys<double> &ph, double rd, double p, double ux,
                                                double uy) {
  const double c = sqrt(ph.gamma0 * p * rd);
  return fma(c + fabs(ux), ph.inv_dx, (c + fabs(uy)) * ph.inv_dy);
}

// dt of a step from the CFL maximum (src/main.cpp:128-134).
__device__ __forceinline__ double step_dt(const KPhys<double> &ph, unsigned long long invdt_bits, double t,
                                          double t_end) {
  const double inv_dt = __longlong_as_double((long long)invdt_bits);
  double dt = ph.cfl / inv_dt;
  if (t + dt > t_end) dt = t_end - t;
  return dt;
}

}  // namespace
}  // namespace e2d
