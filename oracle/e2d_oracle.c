/*
 * e2d_oracle.c -- CPU restatement of euler2d_kokkos' unsplit MUSCL-Hancock
 * Godunov step (implementation 0), double precision, plain C + OpenMP.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the GPU path and the
 * benchmark's CPU baseline.  The product never links it.  Parity of this
 * restatement with the reference itself is pinned by tests/golden/ (fixtures
 * produced by oracle/_ref, the reference's own sources compiled here).
 *
 * Every floating-point expression keeps the reference's operation order so
 * that, built with -ffp-contract=off, results are bit-identical to the
 * reference on any IEEE-754 host.  Citations are to files of the reference
 * project (src/..., config/...).
 */
#include "e2d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(p, i, j, v) ((size_t)(i) + (size_t)(p)->isize * ((size_t)(j) + (size_t)(p)->jsize * (size_t)(v)))

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* src/HydroParams.cpp:160-190 (HydroParams::init). */
void orc_params_init(orc_params *p) {
  p->ghost = 2;
  p->isize = p->nx + 2 * p->ghost;
  p->jsize = p->ny + 2 * p->ghost;
  p->dx = (p->xmax - p->xmin) / p->nx;
  p->dy = (p->ymax - p->ymin) / p->ny;
  p->smallp = p->smallc * p->smallc / p->gamma0;
  p->smallpp = p->smallr * p->smallp;
  p->gamma6 = (p->gamma0 + 1.0) / (2.0 * p->gamma0);
}

/* src/HydroBaseFunctor.h:76-102 (computePrimitives). */
void orc_primitives(const orc_params *p, const double u[4], double q[4], double *c) {
  const double gamma0 = p->gamma0;
  double d = fmax(u[ORC_ID], p->smallr);
  double ux = u[ORC_IU] / d;
  double uy = u[ORC_IV] / d;
  double eken = 0.5 * (ux * ux + uy * uy);
  double e = u[ORC_IP] / d - eken;
  double pr = fmax((gamma0 - 1.0) * d * e, d * p->smallp);
  *c = sqrt(gamma0 * pr / d);
  q[ORC_ID] = d;
  q[ORC_IP] = pr;
  q[ORC_IU] = ux;
  q[ORC_IV] = uy;
}

/* src/HydroBaseFunctor.h:421-455 (slope_unsplit_hydro_2d_scalar), one direction. */
static double slope_1d(double st, double q, double qp, double qm) {
  double dlft = st * (q - qm);
  double drgt = st * (qp - q);
  double dcen = 0.5 * (qp - qm);
  double dsgn = (dcen >= 0.0) ? 1.0 : -1.0;
  double slop = fmin(fabs(dlft), fabs(drgt));
  double dlim = slop;
  if ((dlft * drgt) <= 0.0) dlim = 0.0;
  return dsgn * fmin(dlim, fabs(dcen));
}

/* src/HydroBaseFunctor.h:475-516 (slope_unsplit_hydro_2d). */
void orc_slopes(const orc_params *p, const double q[4], const double qpx[4], const double qmx[4],
                const double qpy[4], const double qmy[4], double dqx[4], double dqy[4]) {
  const double st = p->slope_type;
  for (int v = 0; v < 4; ++v) {
    dqx[v] = 0.0;
    dqy[v] = 0.0;
  }
  if (st == 0.0) return;
  if (st == 1.0 || st == 2.0) {
    for (int v = 0; v < 4; ++v) {
      dqx[v] = slope_1d(st, q[v], qpx[v], qmx[v]);
      dqy[v] = slope_1d(st, q[v], qpy[v], qmy[v]);
    }
  }
}

/* src/HydroBaseFunctor.h:214-291 (trace_unsplit_2d_along_dir). */
void orc_trace(const orc_params *p, const double q[4], const double dqx[4], const double dqy[4],
               double dtdx, double dtdy, int face, double qf[4]) {
  const double gamma0 = p->gamma0;
  double r = q[ORC_ID], pr = q[ORC_IP], u = q[ORC_IU], v = q[ORC_IV];
  double drx = dqx[ORC_ID], dpx = dqx[ORC_IP], dux = dqx[ORC_IU], dvx = dqx[ORC_IV];
  double dry = dqy[ORC_ID], dpy = dqy[ORC_IP], duy = dqy[ORC_IU], dvy = dqy[ORC_IV];
  double sr0 = -u * drx - v * dry - (dux + dvy) * r;
  double sp0 = -u * dpx - v * dpy - (dux + dvy) * gamma0 * pr;
  double su0 = -u * dux - v * duy - (dpx) / r;
  double sv0 = -u * dvx - v * dvy - (dpy) / r;
  if (face == ORC_FACE_XMIN) {
    qf[ORC_ID] = r - 0.5 * drx + sr0 * dtdx * 0.5;
    qf[ORC_IP] = pr - 0.5 * dpx + sp0 * dtdx * 0.5;
    qf[ORC_IU] = u - 0.5 * dux + su0 * dtdx * 0.5;
    qf[ORC_IV] = v - 0.5 * dvx + sv0 * dtdx * 0.5;
  } else if (face == ORC_FACE_XMAX) {
    qf[ORC_ID] = r + 0.5 * drx + sr0 * dtdx * 0.5;
    qf[ORC_IP] = pr + 0.5 * dpx + sp0 * dtdx * 0.5;
    qf[ORC_IU] = u + 0.5 * dux + su0 * dtdx * 0.5;
    qf[ORC_IV] = v + 0.5 * dvx + sv0 * dtdx * 0.5;
  } else if (face == ORC_FACE_YMIN) {
    qf[ORC_ID] = r - 0.5 * dry + sr0 * dtdy * 0.5;
    qf[ORC_IP] = pr - 0.5 * dpy + sp0 * dtdy * 0.5;
    qf[ORC_IU] = u - 0.5 * duy + su0 * dtdy * 0.5;
    qf[ORC_IV] = v - 0.5 * dvy + sv0 * dtdy * 0.5;
  } else {
    qf[ORC_ID] = r + 0.5 * dry + sr0 * dtdy * 0.5;
    qf[ORC_IP] = pr + 0.5 * dpy + sp0 * dtdy * 0.5;
    qf[ORC_IU] = u + 0.5 * duy + su0 * dtdy * 0.5;
    qf[ORC_IV] = v + 0.5 * dvy + sv0 * dtdy * 0.5;
  }
  qf[ORC_ID] = fmax(p->smallr, qf[ORC_ID]);
}

/* src/HydroBaseFunctor.h:523-547 (cmpflx). */
static void cmpflx(const orc_params *p, const double g[4], double f[4]) {
  f[ORC_ID] = g[ORC_ID] * g[ORC_IU];
  f[ORC_IU] = f[ORC_ID] * g[ORC_IU] + g[ORC_IP];
  f[ORC_IV] = f[ORC_ID] * g[ORC_IV];
  double entho = 1.0 / (p->gamma0 - 1.0);
  double ekin = 0.5 * g[ORC_ID] * (g[ORC_IU] * g[ORC_IU] + g[ORC_IV] * g[ORC_IV]);
  double etot = g[ORC_IP] * entho + ekin;
  f[ORC_IP] = g[ORC_IU] * (etot + g[ORC_IP]);
}

/* src/HydroBaseFunctor.h:558-693 (riemann_approx): RAMSES two-shock solver,
 * Newton iterations capped at 10 with a 1e-6 convergence test (hard-coded
 * there, :592). */
static void riemann_approx(const orc_params *p, const double ql[4], const double qr[4],
                           double flux[4]) {
  const double gamma0 = p->gamma0, gamma6 = p->gamma6, smallr = p->smallr, smallc = p->smallc;
  const double smallp = p->smallp, smallpp = p->smallpp;
  double rl = fmax(ql[ORC_ID], smallr), ul = ql[ORC_IU], pl = fmax(ql[ORC_IP], rl * smallp);
  double rr = fmax(qr[ORC_ID], smallr), ur = qr[ORC_IU], pr = fmax(qr[ORC_IP], rr * smallp);
  double cl = gamma0 * pl * rl;
  double cr = gamma0 * pr * rr;
  double wl = sqrt(cl);
  double wr = sqrt(cr);
  double pstar = fmax(((wr * pl + wl * pr) + wl * wr * (ul - ur)) / (wl + wr), 0.0);
  double pold = pstar;
  double conv = 1.0;
  for (int iter = 0; (iter < 10) && (conv > 1e-6); ++iter) {
    double wwl = sqrt(cl * (1.0 + gamma6 * (pold - pl) / pl));
    double wwr = sqrt(cr * (1.0 + gamma6 * (pold - pr) / pr));
    double qxl = 2.0 * wwl * wwl * wwl / (wwl * wwl + cl);
    double qxr = 2.0 * wwr * wwr * wwr / (wwr * wwr + cr);
    double usl = ul - (pold - pl) / wwl;
    double usr = ur + (pold - pr) / wwr;
    double delp = fmax(qxr * qxl / (qxr + qxl) * (usl - usr), -pold);
    pold = pold + delp;
    conv = fabs(delp / (pold + smallpp));
  }
  pstar = pold;
  wl = sqrt(cl * (1.0 + gamma6 * (pstar - pl) / pl));
  wr = sqrt(cr * (1.0 + gamma6 * (pstar - pr) / pr));
  double ustar = 0.5 * (ul + (pl - pstar) / wl + ur - (pr - pstar) / wr);
  double sgnm = copysign(1.0, ustar);
  double ro, uo, po, wo;
  if (sgnm > 0.0) {
    ro = rl; uo = ul; po = pl; wo = wl;
  } else {
    ro = rr; uo = ur; po = pr; wo = wr;
  }
  double co = fmax(smallc, sqrt(fabs(gamma0 * po / ro)));
  double rstar = fmax((ro / (1.0 + ro * (po - pstar) / (wo * wo))), smallr);
  double cstar = fmax(smallc, sqrt(fabs(gamma0 * pstar / rstar)));
  double spout = co - sgnm * uo;
  double spin = cstar - sgnm * ustar;
  double ushock = wo / ro - sgnm * uo;
  if (pstar >= po) {
    spin = ushock;
    spout = ushock;
  }
  double scr = fmax(spout - spin, smallc + fabs(spout + spin));
  double frac = 0.5 * (1.0 + (spout + spin) / scr);
  if (frac != frac)
    frac = 0.0;
  else
    frac = frac >= 1.0 ? 1.0 : frac <= 0.0 ? 0.0 : frac;
  double g[4];
  g[ORC_ID] = frac * rstar + (1.0 - frac) * ro;
  g[ORC_IU] = frac * ustar + (1.0 - frac) * uo;
  g[ORC_IP] = frac * pstar + (1.0 - frac) * po;
  if (spout < 0.0) {
    g[ORC_ID] = ro; g[ORC_IU] = uo; g[ORC_IP] = po;
  }
  if (spin > 0.0) {
    g[ORC_ID] = rstar; g[ORC_IU] = ustar; g[ORC_IP] = pstar;
  }
  g[ORC_IV] = (sgnm > 0.0) ? ql[ORC_IV] : qr[ORC_IV];
  cmpflx(p, g, flux);
}

/* src/HydroBaseFunctor.h:704-809 (riemann_hllc). */
static void riemann_hllc(const orc_params *p, const double ql[4], const double qr[4],
                         double flux[4]) {
  const double gamma0 = p->gamma0, smallr = p->smallr, smallp = p->smallp, smallc = p->smallc;
  const double entho = 1.0 / (gamma0 - 1.0);
  double rl = fmax(ql[ORC_ID], smallr);
  double pl = fmax(ql[ORC_IP], rl * smallp);
  double ul = ql[ORC_IU];
  double ecinl = 0.5 * rl * ul * ul;
  ecinl += 0.5 * rl * ql[ORC_IV] * ql[ORC_IV];
  double etotl = pl * entho + ecinl;
  double ptotl = pl;
  double rr = fmax(qr[ORC_ID], smallr);
  double pr = fmax(qr[ORC_IP], rr * smallp);
  double ur = qr[ORC_IU];
  double ecinr = 0.5 * rr * ur * ur;
  ecinr += 0.5 * rr * qr[ORC_IV] * qr[ORC_IV];
  double etotr = pr * entho + ecinr;
  double ptotr = pr;
  double cfastl = sqrt(fmax(gamma0 * pl / rl, smallc * smallc));
  double cfastr = sqrt(fmax(gamma0 * pr / rr, smallc * smallc));
  double SL = fmin(ul, ur) - fmax(cfastl, cfastr);
  double SR = fmax(ul, ur) + fmax(cfastl, cfastr);
  double rcl = rl * (ul - SL);
  double rcr = rr * (SR - ur);
  double ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  double ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);
  double rstarl = rl * (SL - ul) / (SL - ustar);
  double etotstarl = ((SL - ul) * etotl - ptotl * ul + ptotstar * ustar) / (SL - ustar);
  double rstarr = rr * (SR - ur) / (SR - ustar);
  double etotstarr = ((SR - ur) * etotr - ptotr * ur + ptotstar * ustar) / (SR - ustar);
  double ro, uo, ptoto, etoto;
  if (SL > 0.0) {
    ro = rl; uo = ul; ptoto = ptotl; etoto = etotl;
  } else if (ustar > 0.0) {
    ro = rstarl; uo = ustar; ptoto = ptotstar; etoto = etotstarl;
  } else if (SR > 0.0) {
    ro = rstarr; uo = ustar; ptoto = ptotstar; etoto = etotstarr;
  } else {
    ro = rr; uo = ur; ptoto = ptotr; etoto = etotr;
  }
  flux[ORC_ID] = ro * uo;
  flux[ORC_IU] = ro * uo * uo + ptoto;
  flux[ORC_IP] = (etoto + ptoto) * uo;
  flux[ORC_IV] = (flux[ORC_ID] > 0.0) ? flux[ORC_ID] * ql[ORC_IV] : flux[ORC_ID] * qr[ORC_IV];
}

/* HLL flux.  The reference has no HLL solver (its RIEMANN_HLL enum value,
 * src/HydroParams.h:47-52, selects nothing).  This follows the published HLL
 * flux of Harten, Lax and van Leer as written in Toro, "Riemann Solvers and
 * Numerical Methods for Fluid Dynamics" (3rd ed., eq. 10.21), with the same
 * cut-offs and Davis wave-speed estimates as riemann_hllc above, so that the
 * three solvers share their inputs. */
static void riemann_hll(const orc_params *p, const double ql[4], const double qr[4],
                        double flux[4]) {
  const double gamma0 = p->gamma0, smallr = p->smallr, smallp = p->smallp, smallc = p->smallc;
  const double entho = 1.0 / (gamma0 - 1.0);
  double rl = fmax(ql[ORC_ID], smallr);
  double pl = fmax(ql[ORC_IP], rl * smallp);
  double ul = ql[ORC_IU], vl = ql[ORC_IV];
  double rr = fmax(qr[ORC_ID], smallr);
  double pr = fmax(qr[ORC_IP], rr * smallp);
  double ur = qr[ORC_IU], vr = qr[ORC_IV];
  double ecinl = 0.5 * rl * ul * ul;
  ecinl += 0.5 * rl * vl * vl;
  double etotl = pl * entho + ecinl;
  double ecinr = 0.5 * rr * ur * ur;
  ecinr += 0.5 * rr * vr * vr;
  double etotr = pr * entho + ecinr;
  double cfastl = sqrt(fmax(gamma0 * pl / rl, smallc * smallc));
  double cfastr = sqrt(fmax(gamma0 * pr / rr, smallc * smallc));
  double SL = fmin(ul, ur) - fmax(cfastl, cfastr);
  double SR = fmax(ul, ur) + fmax(cfastl, cfastr);
  /* conserved states and physical fluxes, reference variable order */
  double UL[4] = {rl, etotl, rl * ul, rl * vl};
  double UR[4] = {rr, etotr, rr * ur, rr * vr};
  double FL[4], FR[4];
  FL[ORC_ID] = UL[ORC_IU];
  FL[ORC_IP] = (etotl + pl) * ul;
  FL[ORC_IU] = UL[ORC_IU] * ul + pl;
  FL[ORC_IV] = UL[ORC_IU] * vl;
  FR[ORC_ID] = UR[ORC_IU];
  FR[ORC_IP] = (etotr + pr) * ur;
  FR[ORC_IU] = UR[ORC_IU] * ur + pr;
  FR[ORC_IV] = UR[ORC_IU] * vr;
  if (SL > 0.0) {
    for (int v = 0; v < 4; ++v) flux[v] = FL[v];
  } else if (SR <= 0.0) {
    for (int v = 0; v < 4; ++v) flux[v] = FR[v];
  } else {
    double sls = SL * SR;
    double rden = 1.0 / (SR - SL); /* one division shared by the four fluxes */
    for (int v = 0; v < 4; ++v)
      flux[v] = (SR * FL[v] - SL * FR[v] + sls * (UR[v] - UL[v])) * rden;
  }
}

void orc_riemann(const orc_params *p, int solver, const double ql[4], const double qr[4],
                 double flux[4]) {
  if (solver == ORC_RIEMANN_APPROX)
    riemann_approx(p, ql, qr, flux);
  else if (solver == ORC_RIEMANN_HLL)
    riemann_hll(p, ql, qr, flux);
  else
    riemann_hllc(p, ql, qr, flux);
}

/* src/HydroRunFunctors.h:1832-2030 (MakeBoundariesFunctor) in the order of
 * src/HydroRun.h:394-397: XMIN, XMAX over every j (ghost rows included), then
 * YMIN, YMAX over every i, which fixes the corner ghosts. */
void orc_make_boundaries(const orc_params *p, double *u) {
  const int g = p->ghost, nx = p->nx, ny = p->ny;
  for (int j = 0; j < p->jsize; ++j)
    for (int i = 0; i < g; ++i)
      for (int v = 0; v < 4; ++v) {
        double sign = 1.0;
        int i0;
        if (p->bc_xmin == ORC_BC_REFLECT) {
          i0 = 2 * g - 1 - i;
          if (v == ORC_IU) sign = -1.0;
        } else if (p->bc_xmin == ORC_BC_ABSORB) {
          i0 = g;
        } else {
          i0 = nx + i;
        }
        u[IDX(p, i, j, v)] = u[IDX(p, i0, j, v)] * sign;
      }
  for (int j = 0; j < p->jsize; ++j)
    for (int i = nx + g; i <= nx + 2 * g - 1; ++i)
      for (int v = 0; v < 4; ++v) {
        double sign = 1.0;
        int i0;
        if (p->bc_xmax == ORC_BC_REFLECT) {
          i0 = 2 * nx + 2 * g - 1 - i;
          if (v == ORC_IU) sign = -1.0;
        } else if (p->bc_xmax == ORC_BC_ABSORB) {
          i0 = nx + g - 1;
        } else {
          i0 = i - nx;
        }
        u[IDX(p, i, j, v)] = u[IDX(p, i0, j, v)] * sign;
      }
  for (int i = 0; i < p->isize; ++i)
    for (int j = 0; j < g; ++j)
      for (int v = 0; v < 4; ++v) {
        double sign = 1.0;
        int j0;
        if (p->bc_ymin == ORC_BC_REFLECT) {
          j0 = 2 * g - 1 - j;
          if (v == ORC_IV) sign = -1.0;
        } else if (p->bc_ymin == ORC_BC_ABSORB) {
          j0 = g;
        } else {
          j0 = ny + j;
        }
        u[IDX(p, i, j, v)] = u[IDX(p, i, j0, v)] * sign;
      }
  for (int i = 0; i < p->isize; ++i)
    for (int j = ny + g; j <= ny + 2 * g - 1; ++j)
      for (int v = 0; v < 4; ++v) {
        double sign = 1.0;
        int j0;
        if (p->bc_ymax == ORC_BC_REFLECT) {
          j0 = 2 * ny + 2 * g - 1 - j;
          if (v == ORC_IV) sign = -1.0;
        } else if (p->bc_ymax == ORC_BC_ABSORB) {
          j0 = ny + g - 1;
        } else {
          j0 = j - ny;
        }
        u[IDX(p, i, j, v)] = u[IDX(p, i, j0, v)] * sign;
      }
}

/* src/HydroRun.h:227-251 (compute_dt) with src/HydroRunFunctors.h:44-75
 * (ComputeDtFunctor): max over the interior of (c+|u|)/dx + (c+|v|)/dy. */
double orc_compute_dt(const orc_params *p, const double *u) {
  const int g = p->ghost;
  double inv_dt = 0.0;
  /* The Kokkos::Max reducer starts from the lowest double; every interior
   * term is positive, so starting at 0 gives the same maximum. */
#pragma omp parallel for reduction(max : inv_dt) schedule(static)
  for (int j = g; j < p->jsize - g; ++j)
    for (int i = g; i < p->isize - g; ++i) {
      double uc[4], q[4], c;
      for (int v = 0; v < 4; ++v) uc[v] = u[IDX(p, i, j, v)];
      orc_primitives(p, uc, q, &c);
      double vx = c + fabs(q[ORC_IU]);
      double vy = c + fabs(q[ORC_IV]);
      double t = vx / p->dx + vy / p->dy;
      inv_dt = fmax(inv_dt, t);
    }
  return p->cfl / inv_dt;
}

static void load_q(const orc_params *p, const double *Q, int i, int j, double q[4]) {
  for (int v = 0; v < 4; ++v) q[v] = Q[IDX(p, i, j, v)];
}

/* src/HydroRun.h:279-330 (godunov_unsplit_impl, implementationVersion 0):
 * boundaries on u_in, full copy into u_out, primitives over the whole array,
 * ComputeAndStoreFluxesFunctor (src/HydroRunFunctors.h:451-644) and
 * UpdateFunctor (src/HydroRunFunctors.h:686-718). */
void orc_godunov_step(const orc_params *p, double *u_in, double *u_out, double dt, double *work) {
  const size_t n = (size_t)p->isize * p->jsize;
  double *Q = work, *Fx = work + 4 * n, *Fy = work + 8 * n;
  const int g = p->ghost, isize = p->isize, jsize = p->jsize;
  const double dtdx = dt / p->dx, dtdy = dt / p->dy;

  orc_make_boundaries(p, u_in);
  memcpy(u_out, u_in, sizeof(double) * 4 * n);

#pragma omp parallel for schedule(static)
  for (int j = 0; j < jsize; ++j)
    for (int i = 0; i < isize; ++i) {
      double uc[4], q[4], c;
      for (int v = 0; v < 4; ++v) uc[v] = u_in[IDX(p, i, j, v)];
      orc_primitives(p, uc, q, &c);
      for (int v = 0; v < 4; ++v) Q[IDX(p, i, j, v)] = q[v];
    }

#pragma omp parallel for schedule(static)
  for (int j = g; j <= jsize - g; ++j)
    for (int i = g; i <= isize - g; ++i) {
      double qc[4], qpx[4], qmx[4], qpy[4], qmy[4], dqx[4], dqy[4];
      double qn[4], dqxn[4], dqyn[4], ql[4], qr[4], f[4], a[4], b[4], c4[4], d4[4];
      /* slopes at (i,j) */
      load_q(p, Q, i, j, qc);
      load_q(p, Q, i + 1, j, qpx);
      load_q(p, Q, i - 1, j, qmx);
      load_q(p, Q, i, j + 1, qpy);
      load_q(p, Q, i, j - 1, qmy);
      orc_slopes(p, qc, qpx, qmx, qpy, qmy, dqx, dqy);
      /* slopes at (i-1,j) */
      load_q(p, Q, i - 1, j, qn);
      load_q(p, Q, i, j, a);
      load_q(p, Q, i - 2, j, b);
      load_q(p, Q, i - 1, j + 1, c4);
      load_q(p, Q, i - 1, j - 1, d4);
      orc_slopes(p, qn, a, b, c4, d4, dqxn, dqyn);
      orc_trace(p, qc, dqx, dqy, dtdx, dtdy, ORC_FACE_XMIN, qr);
      orc_trace(p, qn, dqxn, dqyn, dtdx, dtdy, ORC_FACE_XMAX, ql);
      orc_riemann(p, p->riemann, ql, qr, f);
      for (int v = 0; v < 4; ++v) Fx[IDX(p, i, j, v)] = f[v] * dtdx;
      /* slopes at (i,j-1) */
      load_q(p, Q, i, j - 1, qn);
      load_q(p, Q, i + 1, j - 1, a);
      load_q(p, Q, i - 1, j - 1, b);
      load_q(p, Q, i, j, c4);
      load_q(p, Q, i, j - 2, d4);
      orc_slopes(p, qn, a, b, c4, d4, dqxn, dqyn);
      orc_trace(p, qc, dqx, dqy, dtdx, dtdy, ORC_FACE_YMIN, qr);
      orc_trace(p, qn, dqxn, dqyn, dtdx, dtdy, ORC_FACE_YMAX, ql);
      double t;
      t = ql[ORC_IU]; ql[ORC_IU] = ql[ORC_IV]; ql[ORC_IV] = t;
      t = qr[ORC_IU]; qr[ORC_IU] = qr[ORC_IV]; qr[ORC_IV] = t;
      orc_riemann(p, p->riemann, ql, qr, f);
      t = f[ORC_IU]; f[ORC_IU] = f[ORC_IV]; f[ORC_IV] = t;
      for (int v = 0; v < 4; ++v) Fy[IDX(p, i, j, v)] = f[v] * dtdy;
    }

#pragma omp parallel for schedule(static)
  for (int j = g; j < jsize - g; ++j)
    for (int i = g; i < isize - g; ++i)
      for (int pass = 0; pass < 4; ++pass)
        for (int v = 0; v < 4; ++v) {
          double *dst = &u_out[IDX(p, i, j, v)];
          if (pass == 0) *dst += Fx[IDX(p, i, j, v)];
          if (pass == 1) *dst -= Fx[IDX(p, i + 1, j, v)];
          if (pass == 2) *dst += Fy[IDX(p, i, j, v)];
          if (pass == 3) *dst -= Fy[IDX(p, i, j + 1, v)];
        }
}

/* src/main.cpp:87-145: dt from the current state, clamped at t_end, the
 * U/U2 ping-pong of src/HydroRun.h:258-272. */
int orc_run(const orc_params *p, double *u, double *u2, int nstep_max, double t_end,
            double *dt_trace, double *t_out) {
  const size_t n = (size_t)p->isize * p->jsize;
  double *work = (double *)malloc(sizeof(double) * 12 * n);
  if (!work) return -1;
  double t = 0.0, dt;
  int ns = 0;
  orc_make_boundaries(p, u);
  orc_make_boundaries(p, u2);
  while (t < t_end && ns < nstep_max) {
    dt = orc_compute_dt(p, (ns % 2 == 0) ? u : u2);
    if (t + dt > t_end) dt = t_end - t;
    if (dt_trace) dt_trace[ns] = dt;
    if (ns % 2 == 0)
      orc_godunov_step(p, u, u2, dt, work);
    else
      orc_godunov_step(p, u2, u, dt, work);
    ns++;
    t += dt;
  }
  free(work);
  if (t_out) *t_out = t;
  return ns;
}

/* src/HydroRunFunctors.h:1375-1401 (InitImplodeFunctor).  reference_shape=1
 * uses the reference's x + y*y in (0.5, 1.5) region; 0 uses the x + y > 0.5
 * diagonal split of the classic implosion test. */
void orc_init_implode(const orc_params *p, double *u, int reference_shape) {
  const double gamma0 = p->gamma0;
  for (int j = 0; j < p->jsize; ++j)
    for (int i = 0; i < p->isize; ++i) {
      double x = p->xmin + p->dx / 2 + (i - p->ghost) * p->dx;
      double y = p->ymin + p->dy / 2 + (j - p->ghost) * p->dy;
      int inside;
      if (reference_shape) {
        double tmp = x + y * y;
        inside = (tmp > 0.5 && tmp < 1.5);
      } else {
        inside = (x + y > 0.5);
      }
      u[IDX(p, i, j, ORC_ID)] = inside ? 1.0 : 0.125;
      u[IDX(p, i, j, ORC_IP)] = inside ? 1.0 / (gamma0 - 1.0) : 0.14 / (gamma0 - 1.0);
      u[IDX(p, i, j, ORC_IU)] = 0.0;
      u[IDX(p, i, j, ORC_IV)] = 0.0;
    }
}

/* src/HydroRunFunctors.h:1451-1494 (InitBlastFunctor, regular init). */
/* src/ComputeRadialProfileFunctor.h:83-134 (apply) and :140-158 (operator()). */
void orc_radial_profile(const orc_params *p, const double *u, int nbins, double *distances,
                        double *profile, long long *counts) {
  const double cx = (p->xmin + p->xmax) / 2;
  const double cy = (p->ymin + p->ymax) / 2;
  const double Dx = (p->xmax - p->xmin) / 2;
  const double Dy = (p->ymax - p->ymin) / 2;
  const double rmax = sqrt(Dx * Dx + Dy * Dy);
  for (int b = 0; b < nbins; ++b) {
    profile[b] = 0.0;
    counts[b] = 0;
  }
  for (int j = 0; j < p->jsize; ++j)
    for (int i = 0; i < p->isize; ++i) {
      const double x = p->xmin + p->dx / 2 + (i - p->ghost) * p->dx;
      const double y = p->ymin + p->dy / 2 + (j - p->ghost) * p->dy;
      const double d = sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy));
      const int bin = (int)(d / rmax * nbins);
      if (bin < nbins) {
        counts[bin] += 1;
        profile[bin] += u[i + (long)p->isize * j];
      }
    }
  const double dr = rmax / nbins;
  for (int b = 0; b < nbins; ++b) {
    distances[b] = (b + 0.5) * dr;
    profile[b] /= (double)counts[b];
  }
}

void orc_init_blast(const orc_params *p, double *u, double radius, double cx, double cy,
                    double d_in, double d_out, double p_in, double p_out) {
  const double gamma0 = p->gamma0, r2 = radius * radius;
  for (int j = 0; j < p->jsize; ++j)
    for (int i = 0; i < p->isize; ++i) {
      double x = p->xmin + p->dx / 2 + (i - p->ghost) * p->dx;
      double y = p->ymin + p->dy / 2 + (j - p->ghost) * p->dy;
      double d2 = (x - cx) * (x - cx) + (y - cy) * (y - cy);
      int in = d2 < r2;
      u[IDX(p, i, j, ORC_ID)] = in ? d_in : d_out;
      u[IDX(p, i, j, ORC_IP)] = (in ? p_in : p_out) / (gamma0 - 1.0);
      u[IDX(p, i, j, ORC_IU)] = 0.0;
      u[IDX(p, i, j, ORC_IV)] = 0.0;
    }
}

/* src/HydroRunFunctors.h:1578-1665 (InitFourQuadrantFunctor).  prim holds
 * the (rho, p, u, v) states of regions 0..3 and (xt, yt) the split point
 * (the reference hard-codes 0.8, 0.8 and Lax-Liu case 3). */
void orc_init_four_quadrant(const orc_params *p, double *u, double xt, double yt,
                            const double prim[16]) {
  const double gamma0 = p->gamma0;
  double cons[4][4];
  for (int r = 0; r < 4; ++r) {
    double rho = prim[4 * r + 0], pr = prim[4 * r + 1], uu = prim[4 * r + 2], vv = prim[4 * r + 3];
    cons[r][ORC_ID] = rho;
    cons[r][ORC_IU] = uu * rho;
    cons[r][ORC_IV] = vv * rho;
    cons[r][ORC_IP] = pr / (gamma0 - 1.0) + rho * (uu * uu + vv * vv) * 0.5;
  }
  for (int j = 0; j < p->jsize; ++j)
    for (int i = 0; i < p->isize; ++i) {
      double x = p->xmin + p->dx / 2 + (i - p->ghost) * p->dx;
      double y = p->ymin + p->dy / 2 + (j - p->ghost) * p->dy;
      int r = (x < xt) ? ((y < yt) ? 2 : 1) : ((y < yt) ? 3 : 0);
      for (int v = 0; v < 4; ++v) u[IDX(p, i, j, v)] = cons[r][v];
    }
}
