// e2d_fp32c.cu -- FP32 step with a compensated (hi, lo) conservative update.
//
// The state keeps each conserved variable as an unevaluated sum hi + lo of
// two floats (~48 significant bits), so the small flux increments of a step
// are not rounded away; slopes, traces and Riemann fluxes are computed in FP32
// from hi.  The update adds the flux balance du to the low word (one FP32
// rounding, 2^-24 |du|: the size of du's own FP32 rounding) and renormalises
// the pair with Fast2Sum (Dekker, 1971), exact while |hi| >= |lo + du|; where
// a value crosses zero the pair keeps the correctly rounded sum, the accuracy
// of a plain FP32 update for that step.  The CFL maximum stays FP64: each warp selects its largest
// FP32 wave-speed term and, unless it is clearly below the running maximum,
// recomputes that cell's term in FP64 from hi + lo; warps combine with an
// FP64 max.
//
// k_step_f32c -- one launch per time step, a register march: each lane owns
// two adjacent columns, each warp a strip of 60 output columns (64 loaded:
// the 2-column halo on each side) by strip_h rows, and walks down the strip one row
// at a time keeping three rows of primitives, the previous row's face states
// and fluxes in registers.  Neighbour columns come from warp shuffles, and
// no block barrier is taken in the march.  Input rows reach the warp either
// as register loads one row ahead or (default variants) through a per-warp
// shared-memory ring filled by cp.async two rows ahead, ordered by one warp
// barrier per row; variant 6 fills the ring of interior strips by TMA copies
// (one per row) waited on with mbarriers, each wait bounded.  The two columns of a lane are computed together with
// Blackwell's packed FP32 instructions (FFMA2 / FADD2 / FMUL2 on float2).
// Ghost cells are read through the boundary map, so no fill pass runs and
// ghost cells of the arrays are never read.  Algorithmic traffic: 32 B read
// + 32 B written per cell.
#include "e2d_common.cuh"
#include "e2d_internal.h"
#include "e2d_tma.cuh"

#include <cudaTypedefs.h>

#include <cstdint>
#include <cstdlib>
#include <type_traits>

namespace e2d {
namespace {

constexpr int LANES = 32;
constexpr int OUTW = 60;   // output columns per warp strip (lanes 1..30)
constexpr int WPB = 4;     // warps (strips) per block
constexpr int CFL_UNIT_ROWS = 16;  // rows of a CFL fold unit (strip heights are multiples)
constexpr int NT = WPB * LANES;

// ------------------------------------------------------------ packed FP32
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);  // a + (-1)*b: one rounding, = a - b
}
__device__ __forceinline__ float2 operator*(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 max2(float2 a, float2 b) { return make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }
__device__ __forceinline__ float2 min2(float2 a, float2 b) { return make_float2(fminf(a.x, b.x), fminf(a.y, b.y)); }
__device__ __forceinline__ float2 abs2(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(1.0f / a.x, 1.0f / a.y); }
__device__ __forceinline__ float2 sqrt2(float2 a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }
__device__ __forceinline__ float2 sel2(bool cx, bool cy, float2 a, float2 b) {
  return make_float2(cx ? a.x : b.x, cy ? a.y : b.y);
}

// Constants broadcast to both halves of a float2.
struct C2 {
  float2 half, mhalf, smallr, smallp, smallc2, gamma0, gm1, entho, st;
  float2 ggm1, gsmallp;  // gamma (gamma - 1), gamma smallp
  float2 h2st, hst, mhst;  // 1 / (2 slope_type), slope_type / 2, -slope_type / 2
};

__device__ __forceinline__ C2 make_c2(const KPhys<float> &ph) {
  C2 k;
  k.half = f2(0.5f);
  k.mhalf = f2(-0.5f);
  k.smallr = f2(ph.smallr);
  k.smallp = f2(ph.smallp);
  k.smallc2 = f2(ph.smallc2);
  k.gamma0 = f2(ph.gamma0);
  k.gm1 = f2(ph.gm1);
  k.entho = f2(ph.entho);
  k.st = f2(ph.slope_type);
  k.ggm1 = f2(ph.gamma0 * ph.gm1);
  k.gsmallp = f2(ph.gamma0 * ph.smallp);
  k.h2st = f2(ph.slope_type > 0.0f ? 0.5f / ph.slope_type : 0.0f);
  k.hst = f2(0.5f * ph.slope_type);
  k.mhst = f2(-0.5f * ph.slope_type);
  return k;
}

// computePrimitives (src/HydroBaseFunctor.h:76-102) for two cells; `inv`
// receives 1 / d, which the trace reuses.
__device__ __forceinline__ void prims2(const C2 &k, float2 rho, float2 e, float2 mx, float2 my,
                                       float2 q[4], float2 &inv) {
  const float2 d = max2(rho, k.smallr);
  inv = rcp2(d);
  const float2 u = mx * inv, v = my * inv;
  const float2 ei = fma2(e, inv, k.mhalf * fma2(u, u, v * v));  // e/d - (u^2+v^2)/2
  q[E2D_ID] = d;
  q[E2D_IP] = max2(k.gm1 * d * ei, d * k.smallp);
  q[E2D_IU] = u;
  q[E2D_IV] = v;
}
__device__ __forceinline__ void prims2(const C2 &k, float2 rho, float2 e, float2 mx, float2 my,
                                       float2 q[4]) {
  float2 inv;
  prims2(k, rho, e, mx, my, q, inv);
}

// Three-input minimum and maximum (one instruction each on sm_100 and later).
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

// slope_unsplit_hydro_2d_scalar (src/HydroBaseFunctor.h:421-455), one
// direction, two cells; slope_type 0 is handled by the caller.  The
// reference's form -- zero when (q-qm)*(qp-q) <= 0, else
// sign(dcen) * min(st|q-qm|, st|qp-q|, |dcen|) -- is the minmod of the three
// differences a = st(q-qm), b = st(qp-q), c = dcen:
// the median of min(a,b,c), 0 and max(a,b,c), max(lo, min(hi, 0)).  When a
// and b have one sign, c (half their sum) has it too and the minmod is the
// one of smallest magnitude; when they differ it is 0.
__device__ __forceinline__ float2 minmod2(float2 a, float2 b, float2 c) {
  const float2 lo = make_float2(min3f(a.x, b.x, c.x), min3f(a.y, b.y, c.y));
  const float2 hi = make_float2(max3f(a.x, b.x, c.x), max3f(a.y, b.y, c.y));
  return max2(lo, min2(hi, f2(0.0f)));
}
// The slope divided by slope_type: minmod is homogeneous, so
// minmod(st a, st b, c) = st minmod(a, b, c / st); the callers carry the
// factor st in their constants (exact for slope_type 1 and 2).
__device__ __forceinline__ float2 slope2(const C2 &k, float2 q, float2 qp, float2 qm) {
  return minmod2(q - qm, qp - q, k.h2st * (qp - qm));
}

// riemann_hllc (src/HydroBaseFunctor.h:704-809) for two faces.
// The face states' densities arrive clamped to smallr by the trace, so the
// reference's clamp here would return them unchanged.
__device__ __forceinline__ void hllc2(const C2 &k, const float2 ql[4], const float2 qr[4], float2 f[4]) {
  const float2 rl = ql[E2D_ID], rr = qr[E2D_ID];
  const float2 pl = max2(ql[E2D_IP], rl * k.smallp), pr = max2(qr[E2D_IP], rr * k.smallp);
  const float2 ul = ql[E2D_IU], ur = qr[E2D_IU], vl = ql[E2D_IV], vr = qr[E2D_IV];
  const float2 cl = sqrt2(max2(k.gamma0 * pl * rcp2(rl), k.smallc2));
  const float2 cr = sqrt2(max2(k.gamma0 * pr * rcp2(rr), k.smallc2));
  const float2 cmax = max2(cl, cr);
  const float2 SL = min2(ul, ur) - cmax;
  const float2 SR = max2(ul, ur) + cmax;
  const float2 rcl = rl * (ul - SL);
  const float2 rcr = rr * (SR - ur);
  const float2 iden = rcp2(rcr + rcl);
  const float2 ustar = fma2(rcr, ur, fma2(rcl, ul, pl - pr)) * iden;
  const float2 ptotstar = fma2(rcr, pl, fma2(rcl, pr, rcl * rcr * (ul - ur))) * iden;
  const bool lx = ustar.x > 0.0f, ly = ustar.y > 0.0f;
  const float2 S = sel2(lx, ly, SL, SR);
  const float2 rs = sel2(lx, ly, rl, rr), us = sel2(lx, ly, ul, ur), ps = sel2(lx, ly, pl, pr);
  const float2 vs = sel2(lx, ly, vl, vr);
  // the total energy of the contact's side only (the other is never read)
  const float2 es = fma2(ps, k.entho, k.half * rs * fma2(us, us, vs * vs));
  const float2 sdu = S - us;
  const float2 isds = rcp2(S - ustar);
  const float2 rstar = rs * sdu * isds;
  const float2 etotstar = fma2(ptotstar, ustar, fma2(sdu, es, (ps * us) * f2(-1.0f))) * isds;
  // The reference samples: SL > 0: left state; else ustar > 0: left star;
  // else SR > 0: right star; else right state.  SL > 0 implies ustar > 0
  // (then rcl*ul > gamma*pl and rcr*ur > gamma*pr, so the numerator of ustar
  // exceeds (gamma+1)*pl + (gamma-1)*pr > 0), and SR <= 0 implies
  // ustar <= 0, so the choice is: the side's own state when its outer wave
  // S is on the far side of x/t = 0 ((S > 0) == (ustar > 0)), else its star
  // state.  (No branch around the selects: the x and y solves of a row stay
  // in one basic block.)
  const bool ox = (S.x > 0.0f) == lx, oy = (S.y > 0.0f) == ly;
  const float2 ro = sel2(ox, oy, rs, rstar);
  const float2 uo = sel2(ox, oy, us, ustar);
  const float2 po = sel2(ox, oy, ps, ptotstar);
  const float2 eo = sel2(ox, oy, es, etotstar);
  f[E2D_ID] = ro * uo;
  f[E2D_IU] = fma2(f[E2D_ID], uo, po);
  f[E2D_IP] = (eo + po) * uo;
  f[E2D_IV] = f[E2D_ID] * sel2(f[E2D_ID].x > 0.0f, f[E2D_ID].y > 0.0f, vl, vr);
}

// HLL flux (Toro eq. 10.21, riemann_hllc's wave speeds) for two faces.
__device__ __forceinline__ void hll2(const C2 &k, const float2 ql[4], const float2 qr[4], float2 f[4]) {
  const float2 rl = ql[E2D_ID], rr = qr[E2D_ID];  // clamped by the trace (hllc2)
  const float2 pl = max2(ql[E2D_IP], rl * k.smallp), pr = max2(qr[E2D_IP], rr * k.smallp);
  const float2 ul = ql[E2D_IU], ur = qr[E2D_IU], vl = ql[E2D_IV], vr = qr[E2D_IV];
  const float2 etotl = fma2(pl, k.entho, k.half * rl * fma2(ul, ul, vl * vl));
  const float2 etotr = fma2(pr, k.entho, k.half * rr * fma2(ur, ur, vr * vr));
  const float2 cmax = max2(sqrt2(max2(k.gamma0 * pl * rcp2(rl), k.smallc2)),
                           sqrt2(max2(k.gamma0 * pr * rcp2(rr), k.smallc2)));
  const float2 SL = min2(ul, ur) - cmax;
  const float2 SR = max2(ul, ur) + cmax;
  const float2 UL[4] = {rl, etotl, rl * ul, rl * vl};
  const float2 UR[4] = {rr, etotr, rr * ur, rr * vr};
  const float2 FL[4] = {UL[E2D_IU], (etotl + pl) * ul, fma2(UL[E2D_IU], ul, pl), UL[E2D_IU] * vl};
  const float2 FR[4] = {UR[E2D_IU], (etotr + pr) * ur, fma2(UR[E2D_IU], ur, pr), UR[E2D_IU] * vr};
  const float2 iden = rcp2(SR - SL);
  const float2 sls = SL * SR;
  const bool ax = SL.x > 0.0f, ay = SL.y > 0.0f, bx = SR.x <= 0.0f, by = SR.y <= 0.0f;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const float2 mid = fma2(sls, UR[v] - UL[v], SR * FL[v] - SL * FR[v]) * iden;
    f[v] = sel2(ax, ay, FL[v], sel2(bx, by, FR[v], mid));
  }
}

// riemann_approx (src/HydroBaseFunctor.h:558-693), one face, FP32.
__device__ __noinline__ void approx1(const KPhys<float> &ph, const float *ql, const float *qr, float *flux) {
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
__device__ __forceinline__ void riemann2(const KPhys<float> &ph, const C2 &k, const float2 ql[4],
                                         const float2 qr[4], float2 f[4]) {
  if (RS == E2D_RIEMANN_HLLC) {
    hllc2(k, ql, qr, f);
  } else if (RS == E2D_RIEMANN_HLL) {
    hll2(k, ql, qr, f);
  } else {
    float a[4], b[4], fa[4], fb[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) a[v] = ql[v].x, b[v] = qr[v].x;
    approx1(ph, a, b, fa);
#pragma unroll
    for (int v = 0; v < 4; ++v) a[v] = ql[v].y, b[v] = qr[v].y;
    approx1(ph, a, b, fb);
#pragma unroll
    for (int v = 0; v < 4; ++v) f[v] = make_float2(fa[v], fb[v]);
  }
}

// CFL term of src/HydroRunFunctors.h:56-72, FP64, from a compensated cell.
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

// The CFL term of two cells from their conserved values; idx = (1/dx, 1/dy).
__device__ __forceinline__ float2 cfl_term2(const C2 &k, float2 idx, const float2 u[4]) {
  // the primitives' u, v and internal energy e/d - (u^2+v^2)/2; the sound
  // speed from gamma p / d = gamma max((gamma-1) ei, smallp), p's cut-off
  // divided through by d
  const float2 inv = rcp2(max2(u[0], k.smallr));
  const float2 ux = u[2] * inv, uy = u[3] * inv;
  const float2 ei = fma2(u[1], inv, k.mhalf * fma2(ux, ux, uy * uy));
  const float2 c = sqrt2(max2(k.ggm1 * ei, k.gsmallp));
  return fma2(c + abs2(ux), f2(idx.x), (c + abs2(uy)) * f2(idx.y));
}

// Folds one candidate's FP64 CFL term into *target -- skipped when its FP32
// term is more than 1e-4 below the running maximum (FP32 terms are within
// ~1e-6 of the FP64 ones, so such a cell cannot hold the maximum; any value
// of the running maximum is a lower bound of the final one, so the final
// maximum does not depend on which candidates were skipped).
__device__ __forceinline__ void fold_candidate(const KParams32 &kp, float term, long long cell,
                                               const float *w, unsigned long long *target,
                                               unsigned int *status) {
  const double cur = __longlong_as_double((long long)(*(volatile unsigned long long *)target));
  if ((double)term < cur * (1.0 - 1e-4)) return;
  const long long P = kp.wplane;
  double u[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) u[v] = (double)w[cell + v * P] + (double)w[cell + (4 + v) * P];
  const double t64 = cfl_term64(kp.ph64, u[E2D_ID], u[E2D_IP], u[E2D_IU], u[E2D_IV]);
  if (t64 > 0.0 && !nonfinite64(t64))
    atomicMax(target, (unsigned long long)__double_as_longlong(t64));
  else
    atomicOr(status, nonfinite64(t64) ? (unsigned)E2D_FLAG_NONFINITE : (unsigned)E2D_FLAG_BAD_DT);
}

// Warp arg-max of an FP32 term (ties to the larger cell), then lane 0 folds
// the winner.
__device__ __forceinline__ void warp_cfl_fold(const KParams32 &kp, float term, long long cell,
                                              const float *w, unsigned long long *target,
                                              unsigned int *status) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float ot = __shfl_xor_sync(0xffffffffu, term, off);
    const long long oc = __shfl_xor_sync(0xffffffffu, cell, off);
    if (ot > term || (ot == term && oc > cell)) term = ot, cell = oc;
  }
  __syncwarp();  // the winner was written by a lane of this warp
  if ((threadIdx.x & 31) != 0 || cell < 0) return;
  fold_candidate(kp, term, cell, w, target, status);
}

// The same arg-max for a fold unit inside a strip march, with two warp
// reductions: `local` is the lane's best cell as its index in the strip,
// (row - rb) * 64 + (column - (cb - 2)), plus one (0: no candidate), which
// orders cells as their array offsets do.  CFL terms of valid cells are
// positive, so their bit patterns order like their values.
__device__ __forceinline__ int unit_argmax(float best, int local, float *term) {
  const unsigned int tb = local > 0 ? __float_as_uint(best) : 0u;
  const unsigned int m = __reduce_max_sync(0xffffffffu, tb);
  const unsigned int win = __reduce_max_sync(0xffffffffu, (m != 0u && tb == m) ? (unsigned int)local : 0u);
  *term = __uint_as_float(m);
  return (int)win;
}

// ------------------------------------------------------------ conversions
__global__ void k_f32c_from_f64(const KParams32 kp, const double *__restrict__ u, float *__restrict__ w) {
  const KGeom &g = kp.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.isize || j >= g.jsize) return;
  const long long s = i + (long long)g.isize * j, d = i + (long long)kp.wpitch * j;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const double x = u[s + v * g.plane];
    const float hi = (float)x;
    w[d + v * kp.wplane] = hi;
    w[d + (4 + v) * kp.wplane] = (float)(x - (double)hi);
  }
}

// hi + lo in FP64 for every cell; ghost cells through the boundary map (the
// state after make_boundaries).
__global__ void k_f32c_to_f64(const KParams32 kp, const float *__restrict__ w, double *__restrict__ u) {
  const KGeom &g = kp.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.isize || j >= g.jsize) return;
  bool fu, fv;
  const int si = ghost_source(i, g.nx, g.bc_xmin, g.bc_xmax, fu);
  const int sj = ghost_source(j, g.ny, g.bc_ymin, g.bc_ymax, fv);
  const long long s = si + (long long)kp.wpitch * sj, d = i + (long long)g.isize * j;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    double x = (double)w[s + v * kp.wplane] + (double)w[s + (4 + v) * kp.wplane];
    if ((v == E2D_IU && fu) || (v == E2D_IV && fv)) x = -x;
    u[d + v * g.plane] = x;
  }
}

// CFL maximum of a compensated state, folded per fold unit exactly as the
// step kernels fold it (same candidate cells, same order), so a dt computed
// here equals the one the previous step folded.
__global__ void __launch_bounds__(NT) k_f32c_dt(const KParams32 kp, const float *__restrict__ w,
                                                unsigned long long *target, unsigned int *status) {
  const KGeom &g = kp.g;
  const int lane = threadIdx.x & 31;
  const int nsx = (g.nx + OUTW - 1) / OUTW;
  const int nsy = (g.ny + CFL_UNIT_ROWS - 1) / CFL_UNIT_ROWS;
  const C2 k = make_c2(kp.ph);
  const float2 idx = make_float2(1.0f / kp.ph.dx, 1.0f / kp.ph.dy);
  for (int u = blockIdx.x * WPB + (threadIdx.x >> 5); u < nsx * nsy; u += gridDim.x * WPB) {
    const int sx = u % nsx, sy = u / nsx;
    const int cb = 2 + sx * OUTW;
    const int rb = 2 + sy * CFL_UNIT_ROWS;
    const int re = min(rb + CFL_UNIT_ROWS, g.ny + 2);
    const int c0 = cb - 2 + 2 * lane;
    const bool writer = (lane >= 1) && (lane <= 30) && (c0 < g.nx + 2);
    float best = -1.0f;
    long long bcell = -1;
    if (writer) {
      for (int r = rb; r < re; ++r) {
        const long long base = c0 + (long long)kp.wpitch * r;
        float2 h[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) h[v] = __ldg(reinterpret_cast<const float2 *>(w + base + v * kp.wplane));
        const float2 t = cfl_term2(k, idx, h);
        if (t.x > best) best = t.x, bcell = base;
        if (t.y > best && c0 + 1 < g.nx + 2) best = t.y, bcell = base + 1;
      }
    }
    warp_cfl_fold(kp, best, bcell, w, target, status);
  }
}

// ------------------------------------------------------------ the step
// Loads the 4 conserved hi values of array row r for the lane's two columns
// (c0, c0 + 1), ghosts mapped; `direct`: both columns are interior cells of
// an aligned pair, read as one float2 per variable.
__device__ __forceinline__ void load_row(const KParams32 &kp, const float *__restrict__ w, int r, int c0,
                                         bool direct, float2 out[4]) {
  const KGeom &g = kp.g;
  bool fv;
  const int rr = min(max(r, 0), g.jsize - 1);
  const int sr = ghost_source(rr, g.ny, g.bc_ymin, g.bc_ymax, fv);
  const float *row = w + (long long)sr * kp.wpitch;
  if (direct) {
#pragma unroll
    for (int v = 0; v < 4; ++v) out[v] = __ldg(reinterpret_cast<const float2 *>(row + v * kp.wplane + c0));
  } else {
    bool f0, f1;
    const int s0 = ghost_source(min(max(c0, 0), g.isize - 1), g.nx, g.bc_xmin, g.bc_xmax, f0);
    const int s1 = ghost_source(min(max(c0 + 1, 0), g.isize - 1), g.nx, g.bc_xmin, g.bc_xmax, f1);
#pragma unroll
    for (int v = 0; v < 4; ++v) out[v] = make_float2(__ldg(row + v * kp.wplane + s0), __ldg(row + v * kp.wplane + s1));
    if (f0) out[E2D_IU].x = -out[E2D_IU].x;
    if (f1) out[E2D_IU].y = -out[E2D_IU].y;
  }
  if (fv) out[E2D_IV] = neg2(out[E2D_IV]);
}

// Shared-memory row ring of the staged march: each warp copies the rows it
// will need PFD iterations ahead with cp.async (no registers held while the
// copies fly) into PFD + 3 slots (rows m-1 .. m+1+PFD); a slot holds the 8
// planes (hi, lo) x 64 columns of one row, each lane copying and later
// reading only its own two columns.  PFD = 0: rows loaded to registers.
constexpr int SLOT = 8 * 64;  // floats per slot
constexpr int kMaxSlots = 8;  // ring slots (PFD + 3) a warp may have
// (+128 bytes: the ring starts at the first 128-byte boundary of the
// dynamic shared memory, the alignment a tiled TMA destination needs)
constexpr size_t ring_bytes(int pfd) { return pfd > 0 ? sizeof(float) * WPB * (pfd + 3) * SLOT + 128 : 0; }

__device__ __forceinline__ void cp_async16(float *dst, const float *src) {
  const unsigned int d = (unsigned int)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
  const unsigned int d = (unsigned int)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// TMA row staging (interior strips of the staged variants): one
// cp.async.bulk.tensor per row and warp copies the 8 planes x 64 columns of
// a row (a box of 64 x 1 x 8 of the state's tensor map) into a ring slot,
// completing on the slot's mbarrier.  The box starts at a column multiple
// of 4 (x * 4 bytes a multiple of 16, as a tiled copy requires).  Each warp
// owns one mbarrier per ring slot; bit s of `phase` is the parity of slot
// s's next completion.
constexpr unsigned int kRowBytes = 8u * 64u * sizeof(float);

// The warp's ring barriers: initialised once per kernel, before any copy.
__device__ __forceinline__ void ring_bars_init(unsigned long long *bars, int nslots, int lane) {
  if (lane < nslots) mbar_init(bars + lane, 1u);
  mbar_init_fence();
  __syncwarp();
}

// Source row of array row r: itself, or through the boundary map when the
// strip touches a ghost row (`yghost`, warp-uniform); fv: negate IV.
__device__ __forceinline__ int source_row(const KGeom &g, int r, bool yghost, bool &fv) {
  fv = false;
  if (!yghost) return r;
  return ghost_source(min(max(r, 0), g.jsize - 1), g.ny, g.bc_ymin, g.bc_ymax, fv);
}

// Copies array row r into a ring slot.  `direct` strips (64 interior
// columns starting at array column cs, a multiple of 4) copy 16-byte chunks,
// lane l taking chunk l % 16 of planes l / 16, +2, +4, +6, so a lane reads
// columns another lane copied; other strips copy each lane's two columns
// s0, s1 (the boundary map of c0, c0 + 1) element by element.
__device__ __forceinline__ void stage_row(const KParams32 &kp, const float *__restrict__ w, int r, int cs,
                                          int lane, bool direct, bool yghost, int s0, int s1, float *slot) {
  bool fv;
  const float *row = w + (long long)source_row(kp.g, r, yghost, fv) * kp.wpitch;
  if (direct) {
    const int chunk = lane & 15;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int v = (lane >> 4) + 2 * k;
      cp_async16(slot + v * 64 + 4 * chunk, row + v * kp.wplane + cs + 4 * chunk);
    }
  } else {
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      cp_async4(slot + v * 64 + 2 * lane, row + v * kp.wplane + s0);
      cp_async4(slot + v * 64 + 2 * lane + 1, row + v * kp.wplane + s1);
    }
  }
}

// Copies array row r into a ring slot with one TMA copy (interior strips):
// lane 0 arms the slot's barrier for the row's bytes and issues the copy.
// The caller has passed a __syncwarp after every lane's last read of the
// slot; the proxy fence orders those reads before the copy engine's writes.
__device__ __forceinline__ void stage_row_tma(const KGeom &g, const CUtensorMap *map, int r, int cs, int lane,
                                              bool yghost, float *slot, unsigned long long *bar) {
  bool fv;
  const int sr = source_row(g, r, yghost, fv);
  fence_proxy_async_smem();
  if (lane == 0) {
    mbar_arrive_expect(bar, kRowBytes);
    tma_load_3d(slot, map, cs, sr, 0, bar);
  }
}

// One warp marches strip (sx, sy) of an instance: rows rb-2 .. re+1 are
// read, rows rb .. re-1 written.  With a target, the CFL term of the new
// state is folded into *target once per fold unit -- the strip's 60 output
// columns by 16 rows of the interior -- so that the set of FP64-recomputed
// candidates depends only on the grid, never on the strip height, the
// kernel or the batch (strip_h must be a multiple of CFL_UNIT_ROWS and at
// most 32 units).  Each unit's FP32 arg-max is parked in lane `unit`; the
// parked winners are recomputed in FP64 together when the strip ends.
template <int RS, int PFD, int TMA, bool INTERIOR, bool TGT>
__device__ __forceinline__ bool march_strip_t(const KParams32 &kp, const float *__restrict__ w_in,
                                            float *__restrict__ w_out, const float2 dtdx,
                                            const float2 dtdy, const int sx, const int sy,
                                            const int lane, unsigned long long *target,
                                            unsigned int *status, float *ring, const CUtensorMap *map,
                                            unsigned long long *bars, unsigned int &phase) {
  // sum of the lane's new conserved values over the strip: NaN or infinite
  // when one of them is (a sum that overflows FP32 reads as non-finite too)
  float2 nfacc = f2(0.0f);
  float best = -1.0f;      // the lane's largest CFL term in the current fold unit
  int blocal = 0;          // and its strip-local index + 1 (0: none)
  float pend_term = 0.0f;  // lane u: the winner of the strip's fold unit u
  int pend_local = 0;
  int unit = 0;
  const KGeom &g = kp.g;
  const KPhys<float> &ph = kp.ph;
  const int SH = kp.strip_h;
  const int cb = 2 + sx * OUTW;       // array column of the strip's first output column
  const int rb = 2 + sy * SH;         // array row of the strip's first output row
  const int re = min(rb + SH, g.ny + 2);
  const int c0 = cb - 2 + 2 * lane;   // the lane's columns: c0, c0 + 1
  const bool direct = INTERIOR || ((cb - 2 >= 2) && (cb + OUTW + 1 <= g.nx + 1));
  const bool writer = (lane >= 1) && (lane <= 30) && (c0 < g.nx + 2);
  const C2 k = make_c2(ph);
  const float2 idx = make_float2(1.0f / ph.dx, 1.0f / ph.dy);
  const int st_kind = (ph.slope_type == 2.0f) ? 2 : (ph.slope_type == 1.0f) ? 1 : 0;
  const float2 hdtdx = k.mhalf * dtdx, hdtdy = k.mhalf * dtdy;  // exact halvings
  // the same for slopes divided by slope_type (slope2)
  const float2 hdtdxs = hdtdx * k.st, hdtdys = hdtdy * k.st;

  float2 qa[4], qb[4];  // primitives of rows m-1 and m (m: row whose faces are built next)
  float2 ib;            // 1 / density of row m (from its primitives)
  float2 ymax_prev[4];  // YMAX states of row m-1
  float2 fx_prev[4];    // x-fluxes of row m-1: .x face (c0|c1), .y face (c1|c1+1)
  float2 fy_prev[4];    // y-flux of the face between rows m-2 and m-1
#pragma unroll
  for (int v = 0; v < 4; ++v) ymax_prev[v] = fx_prev[v] = fy_prev[v] = f2(0.0f);
  float2 pf[4];  // (register path) conserved hi of row m+1, loaded one iteration ahead
  // (staged path) the boundary map of the lane's columns and its ring slots
  bool f0 = false, f1 = false;
  int s0 = c0, s1 = c0 + 1;
  if ((PFD > 0) && !direct) {
    s0 = ghost_source(min(max(c0, 0), g.isize - 1), g.nx, g.bc_xmin, g.bc_xmax, f0);
    s1 = ghost_source(min(max(c0 + 1, 0), g.isize - 1), g.nx, g.bc_xmin, g.bc_xmax, f1);
  }
  constexpr int R = PFD + 3;  // ring slots; row r sits in slot (r - rb + 2) mod R
  static_assert(TMA != 2 || R == 6, "row pairs need a ring of three pairs");
  const bool yghost = !INTERIOR && ((rb - 2 < 2) || (re + 1 > g.ny + 1));
  // Staged variants: interior strips (`bulk`) fill the ring by TMA copies
  // and wait on the slots' barriers; boundary strips copy each lane's
  // boundary-mapped columns by cp.async and wait on commit groups.  With
  // TMA == 2 (`pairs`) an interior strip away from the ghost rows copies two
  // rows per TMA request (box 64 x 2 x 8 into a pair of slots laid out plane
  // by plane, [8][2][64]) and waits once per pair.
  const bool bulk = (TMA != 0) && (PFD > 0) && direct && !(TMA == 2 && yghost);
  const bool pairs = (TMA == 2) && bulk;
  const int ps = pairs ? 128 : 64;  // floats between the planes of a slot
  auto slot_of = [&](int sl) {
    return pairs ? ring + (sl >> 1) * (2 * SLOT) + (sl & 1) * 64 : ring + sl * SLOT;
  };
  auto wrap = [](int x) { return x >= R ? x - R : x; };
  int sm1 = 0;  // slot of row m-1 (the row being updated)
  // hi of a staged row, ghost flips applied
  auto staged_hi = [&](int r, int sl, float2 out[4]) {
    const float *p = slot_of(sl) + 2 * lane;
#pragma unroll
    for (int v = 0; v < 4; ++v) out[v] = *reinterpret_cast<const float2 *>(p + v * ps);
    if (f0) out[E2D_IU].x = -out[E2D_IU].x;
    if (f1) out[E2D_IU].y = -out[E2D_IU].y;
    bool fv;
    source_row(g, r, yghost, fv);
    if (fv) out[E2D_IV] = neg2(out[E2D_IV]);
  };
  unsigned int pending = 0u;  // slots (pairs: pair slots) with a TMA copy not yet waited for
  auto stage = [&](int r, int sl) {
    if (bulk && TMA == 1) {
      // wait_test: the first row of strip (1, 0) is never copied
      if (kp.wait_test && sx == 1 && sy == 0 && r == rb - 2) return;
      stage_row_tma(g, map, r, cb - 2, lane, yghost, slot_of(sl), bars + sl);
      pending |= 1u << sl;
    } else {
      stage_row(kp, w_in, r, cb - 2, lane, direct, yghost, s0, s1, slot_of(sl));
    }
  };
  auto wait_slot = [&](int sl) {
    const bool done = mbar_wait(bars + sl, (phase >> sl) & 1u);
    if (done) phase ^= 1u << sl, pending &= ~(1u << sl);
    return done;
  };
  // pairs: rows rb-2+2k and rb-1+2k into pair slot k mod 3 (its barrier k mod
  // 3); the caller has passed a __syncwarp after every lane's last read of
  // that pair.  A pair whose first row is past re+1 is not needed.
  auto stage_pair = [&](int k) {
    const int r = rb - 2 + 2 * k;
    if (r > re + 1) return;
    const int pp = k % 3;
    fence_proxy_async_smem();
    if (lane == 0) {
      mbar_arrive_expect(bars + pp, 2 * kRowBytes);
      tma_load_3d(ring + pp * (2 * SLOT), map, cb - 2, r, 0, bars + pp);
    }
    pending |= 1u << pp;
  };
  // a wait that ran out: flag it, let the copies in flight land (bounded
  // too) before the ring is reused or the block exits, leave the strip;
  // false if a copy may still be in flight (the ring must not be reused)
  auto give_up = [&]() {
    if (lane == 0) atomicOr(status, (unsigned)E2D_FLAG_TIMEOUT);
    for (int sl = 0; sl < R; ++sl)
      if (pending & (1u << sl)) wait_slot(sl);
    return pending == 0u;
  };
  if ((PFD > 0)) {
    // rows rb-2 .. rb+PFD-1 into slots 0 .. PFD+1 (one commit group each on
    // the cp.async path), after every lane is done with the ring's previous
    // strip
    __syncwarp();
    if (pairs) {
      stage_pair(0);
      stage_pair(1);
      if (!wait_slot(0)) return give_up();
    } else {
      for (int r = rb - 2; r < rb + PFD; ++r) {
        stage(r, r - rb + 2);
        if (!bulk) cp_async_commit();
      }
      if (bulk) {
        if (!(wait_slot(0) && wait_slot(1))) {
          return give_up();
        }
      } else {
        cp_async_wait<(PFD > 0 ? PFD : 0)>();
      }
    }
    __syncwarp();  // lanes read columns other lanes copied
    float2 u[4];
    staged_hi(rb - 2, 0, u);
    prims2(k, u[0], u[1], u[2], u[3], qa);
    staged_hi(rb - 1, 1, u);
    prims2(k, u[0], u[1], u[2], u[3], qb, ib);
  } else {
    float2 u[4];
    load_row(kp, w_in, rb - 2, c0, direct, u);
    prims2(k, u[0], u[1], u[2], u[3], qa);
    load_row(kp, w_in, rb - 1, c0, direct, u);
    prims2(k, u[0], u[1], u[2], u[3], qb, ib);
    load_row(kp, w_in, rb, c0, direct, pf);
  }
  // march: row n = m + 1 is loaded; faces of row m built; y-flux of face
  // (m-1|m); update of row m-1
  // unrolled by two: the row roll below becomes register renaming
  // (measured 0.75 % faster at 8192^2 than the rolled loop)
#pragma unroll 2
  for (int m = rb - 1; m <= re; ++m) {
    float2 qc[4], ic;
    if ((PFD > 0)) {
      // wait for row m+1 (rows m+2 .. m+PFD may still be in flight); the
      // barrier makes every lane's copies visible to the warp and orders
      // every lane's reads of row m-2 (previous iteration) before the copy
      // of row m+1+PFD into that slot
      if (pairs) {
        // row m+1 opens pair k = j/2 (j its index in the strip): wait for
        // it, then refill the pair of rows m-3 and m-2, now dead, with pair k+1
        const int j = m + 1 - (rb - 2);
        if (!(j & 1) && !wait_slot((j >> 1) % 3)) return give_up();
        __syncwarp();
        if (!(j & 1)) stage_pair((j >> 1) + 1);
      } else {
        if (bulk) {
          if (!wait_slot(wrap(sm1 + 2))) {
            return give_up();
          }
        } else {
          cp_async_wait<(PFD > 0 ? PFD - 1 : 0)>();
        }
        __syncwarp();
        const int rn = m + 1 + PFD;
        if (rn <= re + 1) stage(rn, wrap(sm1 + R - 1));
        if (!bulk) cp_async_commit();
      }
      float2 u[4];
      staged_hi(m + 1, wrap(sm1 + 2), u);
      prims2(k, u[0], u[1], u[2], u[3], qc, ic);
    } else {
      float2 u[4] = {pf[0], pf[1], pf[2], pf[3]};
      // issue the next row's loads before this row's arithmetic
      if (m + 2 <= re + 1) load_row(kp, w_in, m + 2, c0, direct, pf);
      prims2(k, u[0], u[1], u[2], u[3], qc, ic);
    }
    // the update of row m-1 reads its (hi, lo): issue those loads early too
    const bool upd = (m >= rb + 1) && writer;
    const long long ubase = c0 + (long long)kp.wpitch * (m - 1);
    float2 uhi[4], ulo[4];
    if (!(PFD > 0) && upd) {
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        uhi[v] = __ldg(reinterpret_cast<const float2 *>(w_in + ubase + v * kp.wplane));
        ulo[v] = __ldg(reinterpret_cast<const float2 *>(w_in + ubase + (4 + v) * kp.wplane));
      }
    }
    // slopes of row m (x from the neighbour lanes, y from rows m-1, m+1)
    float2 dqx[4], dqy[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const float left = __shfl_up_sync(0xffffffffu, qb[v].y, 1);
      const float right = __shfl_down_sync(0xffffffffu, qb[v].x, 1);
      if (st_kind == 0) {
        dqx[v] = f2(0.0f);
        dqy[v] = f2(0.0f);
      } else {
        dqx[v] = slope2(k, qb[v], make_float2(qb[v].y, right), make_float2(left, qb[v].x));
        dqy[v] = slope2(k, qb[v], qc[v], qa[v]);
      }
    }
    // trace sources (src/HydroBaseFunctor.h:246-249), negated and divided
    // by slope_type like the slopes: ns0 = -s0 / st; the half-step terms
    // below take -st/2 (exact for slope_type 1 and 2: a sign and a power of
    // two)
    float2 ns0[4];
    {
      const float2 r = qb[E2D_ID], p = qb[E2D_IP], u = qb[E2D_IU], v = qb[E2D_IV];
      const float2 div = dqx[E2D_IU] + dqy[E2D_IV];
      const float2 ir = ib;
      ns0[E2D_ID] = fma2(u, dqx[E2D_ID], fma2(v, dqy[E2D_ID], div * r));
      ns0[E2D_IP] = fma2(u, dqx[E2D_IP], fma2(v, dqy[E2D_IP], div * k.gamma0 * p));
      ns0[E2D_IU] = fma2(u, dqx[E2D_IU], fma2(v, dqy[E2D_IU], dqx[E2D_IP] * ir));
      ns0[E2D_IV] = fma2(u, dqx[E2D_IV], fma2(v, dqy[E2D_IV], dqy[E2D_IP] * ir));
    }
    // x faces of row m and y faces of row m (the flux of face (m-1|m) from
    // the saved YMAX of row m-1).  Both Riemann solves run on every row:
    // the loop body has no branch around them, so the two independent
    // solves can be scheduled together.  The update of row m-1 (m >= rb+1)
    // reads the x-fluxes of row m-1 and the y-fluxes of iterations m-1 and
    // m, so the solves of iteration rb-1 (and the x-solve of row re) are
    // never read.
    float2 xl[4], xr[4], ymin[4], ymax[4];
    // the source term first, ns0 * (-dt/(2dx)) added to q by one FMA, then
    // -/+ dq/2 by one FMA each (the halving is exact): the reference's
    // (q -/+ dq*0.5) + s0*0.5*dt/dx summed in another order
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const float2 bx = fma2(ns0[v], hdtdxs, qb[v]);  // q + s0 dt/(2dx)
      float2 xmin = fma2(dqx[v], k.mhst, bx);
      float2 xmax = fma2(dqx[v], k.hst, bx);
      if (v == E2D_ID) xmin = max2(xmin, k.smallr), xmax = max2(xmax, k.smallr);
      xl[v] = xmax;  // left states of faces (c0|c1) and (c1|c1+1)
      xr[v] = make_float2(xmin.y, __shfl_down_sync(0xffffffffu, xmin.x, 1));
      const float2 by = fma2(ns0[v], hdtdys, qb[v]);  // q + s0 dt/(2dy)
      ymin[v] = fma2(dqy[v], k.mhst, by);
      ymax[v] = fma2(dqy[v], k.hst, by);
    }
    ymin[E2D_ID] = max2(ymin[E2D_ID], k.smallr);
    ymax[E2D_ID] = max2(ymax[E2D_ID], k.smallr);
    float2 fx[4], fy[4];
    {
      // normal velocity first: swap IU/IV (src/HydroRunFunctors.h:628-632)
      float2 yl[4] = {ymax_prev[E2D_ID], ymax_prev[E2D_IP], ymax_prev[E2D_IV], ymax_prev[E2D_IU]};
      float2 yr[4] = {ymin[E2D_ID], ymin[E2D_IP], ymin[E2D_IV], ymin[E2D_IU]};
      float2 f[4];
      riemann2<RS>(ph, k, xl, xr, fx);
      riemann2<RS>(ph, k, yl, yr, f);
      // unscaled: dt/dx and dt/dy are applied in the update
      fy[E2D_ID] = f[E2D_ID];
      fy[E2D_IP] = f[E2D_IP];
      fy[E2D_IU] = f[E2D_IV];
      fy[E2D_IV] = f[E2D_IU];
    }
    // compensated update of row m-1
    if (m >= rb + 1) {
      float2 fxl[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) fxl[v] = make_float2(__shfl_up_sync(0xffffffffu, fx_prev[v].y, 1), fx_prev[v].x);
      if (upd) {
        const long long base = ubase;
        if ((PFD > 0)) {
          // row m-1 is interior: its slot holds it unflipped
          const float *sl = slot_of(sm1) + 2 * lane;
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            uhi[v] = *reinterpret_cast<const float2 *>(sl + v * ps);
            ulo[v] = *reinterpret_cast<const float2 *>(sl + (4 + v) * ps);
          }
        }
        float2 nh[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          // +Fx(i) -Fx(i+1) +Fy(j) -Fy(j+1)
          const float2 du = fma2(fxl[v] - fx_prev[v], dtdx, (fy_prev[v] - fy[v]) * dtdy);
          const float2 hi = uhi[v];
          const float2 tl = ulo[v] + du;        // the low word takes the update
          const float2 h2 = hi + tl;            // Fast2Sum(hi, tl)
          const float2 l2 = tl - (h2 - hi);
          *reinterpret_cast<float2 *>(w_out + base + v * kp.wplane) = h2;
          *reinterpret_cast<float2 *>(w_out + base + (4 + v) * kp.wplane) = l2;
          nh[v] = h2;
        }
        if (TGT || target) {
          const float2 t = cfl_term2(k, idx, nh);
          const int loc = (m - 1 - rb) * 64 + 2 * lane + 1;
          // non-finite states: a NaN term never wins the arg-max, and the
          // fmaxf cut-offs drop a NaN density or energy, so the new density
          // and energy are summed with the term, which a non-finite momentum
          // makes non-finite (tested at strip end)
          float2 chk = (nh[0] + nh[1]) + t;
          if (!(c0 + 1 < g.nx + 2)) chk.y = 0.0f;  // a ghost column: not a cell of the grid
          nfacc = nfacc + chk;
          if (t.x > best) best = t.x, blocal = loc;
          if (t.y > best && c0 + 1 < g.nx + 2) best = t.y, blocal = loc + 1;
        }
      }
      const int r = m - 1;  // >= rb >= 2, so the low bits of r - 2 are its remainder
      static_assert((CFL_UNIT_ROWS & (CFL_UNIT_ROWS - 1)) == 0, "fold units are a power of two rows");
      if ((TGT || target) && (((r - 2) & (CFL_UNIT_ROWS - 1)) == CFL_UNIT_ROWS - 1 || r == re - 1)) {
        float ut;
        const int win = unit_argmax(best, blocal, &ut);
        if (lane == unit) pend_term = ut, pend_local = win;
        ++unit;
        best = -1.0f;
        blocal = 0;
      }
    }
    // roll
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      qa[v] = qb[v];
      qb[v] = qc[v];
      ymax_prev[v] = ymax[v];
      fx_prev[v] = fx[v];
      fy_prev[v] = fy[v];
    }
    ib = ic;
    sm1 = wrap(sm1 + 1);
  }
  // the strip's fold-unit winners, one lane each, folded in parallel
  if (TGT || target) {
    const float kInf = __int_as_float(0x7f800000);
    const bool nonfin = !(fabsf(nfacc.x) < kInf) || !(fabsf(nfacc.y) < kInf);
    if (__any_sync(0xffffffffu, nonfin) && lane == 0) atomicOr(status, (unsigned)E2D_FLAG_NONFINITE);
    __syncwarp();  // the winners were written by lanes of this warp
    if (pend_local > 0) {
      const int L = pend_local - 1;
      const long long cell = (long long)kp.wpitch * (rb + L / 64) + (cb - 2) + (L % 64);
      fold_candidate(kp, pend_term, cell, w_out, target, status);
    }
  }
  return true;
}

// Interior strips (every column and row they read is a cell of the grid:
// no boundary map, no ghost flips) of the staged variants that fold the CFL
// maximum (every step of the device loop and of a batch) run an
// instantiation with those tests folded away; the others run the general
// one.  Same arithmetic, same bits.
template <int RS, int PFD, int TMA>
__device__ __forceinline__ bool march_strip(const KParams32 &kp, const float *__restrict__ w_in,
                                            float *__restrict__ w_out, const float2 dtdx,
                                            const float2 dtdy, const int sx, const int sy,
                                            const int lane, unsigned long long *target,
                                            unsigned int *status, float *ring, const CUtensorMap *map,
                                            unsigned long long *bars, unsigned int &phase) {
  const KGeom &g = kp.g;
  const int cb = 2 + sx * OUTW, rb = 2 + sy * kp.strip_h;
  const int re = min(rb + kp.strip_h, g.ny + 2);
  const bool interior = (cb - 2 >= 2) && (cb + OUTW + 1 <= g.nx + 1) && !(rb - 2 < 2) && !(re + 1 > g.ny + 1);
  if constexpr (PFD > 0) {
    if (interior && target)
      return march_strip_t<RS, PFD, TMA, true, true>(kp, w_in, w_out, dtdx, dtdy, sx, sy, lane, target, status,
                                                     ring, map, bars, phase);
  }
  return march_strip_t<RS, PFD, TMA, false, false>(kp, w_in, w_out, dtdx, dtdy, sx, sy, lane, target, status,
                                                   ring, map, bars, phase);
}

extern __shared__ __align__(16) float g_ring[];

// The warp's row ring: g_ring rounded up to 128 bytes (ring_bytes reserves
// the slack), then PFD + 3 slots of 2 KB per warp, so every slot is 128-byte
// aligned.
template <int PFD>
__device__ __forceinline__ float *warp_ring(int warp) {
  const unsigned int a = smem_u32(g_ring);
  return g_ring + ((128u - (a & 127u)) & 127u) / sizeof(float) + warp * (PFD + 3) * SLOT;
}

template <int RS, int MINB, int PFD, int TMA>
__global__ void __launch_bounds__(NT, MINB)
    k_step_f32c(const KParams32 kp, const float *__restrict__ w_in, float *__restrict__ w_out,
                const __grid_constant__ CUtensorMap tm_in, DevClock *clk, const int use_clock,
                const double host_dt) {
  const KGeom &g = kp.g;
  const int tid = threadIdx.x;
  const int lane = tid & 31;

  // dt of this step (FP64, src/main.cpp:128-134) by one thread per block
  __shared__ double s_dt[3];
  __shared__ int s_run, s_slot;
  __shared__ unsigned long long s_bars[TMA ? WPB * kMaxSlots : 1];  // ring slot barriers, per warp
  if (tid == 0) {
    double dt = host_dt;
    int run = 1, slot = 0;
    if (use_clock) {
      const double t = clk->t;
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
  const int slot = s_slot;
  const float2 dtdx = f2((float)s_dt[1]);
  const float2 dtdy = f2((float)s_dt[2]);

  const int nsx = (g.nx + OUTW - 1) / OUTW;
  const int SH = kp.strip_h;
  const int nsy = (g.ny + SH - 1) / SH;
  const int strip = blockIdx.x * WPB + (tid >> 5);
  unsigned long long *bars = s_bars + (TMA ? (tid >> 5) * kMaxSlots : 0);
  unsigned int phase = 0u;
  if (strip < nsx * nsy) {
    if (TMA && PFD > 0) ring_bars_init(bars, PFD + 3, lane);
    march_strip<RS, PFD, TMA>(kp, w_in, w_out, dtdx, dtdy, strip % nsx, strip / nsx, lane,
                         use_clock ? &clk->acc[slot ^ 1] : nullptr, &clk->status,
                         warp_ring<PFD>(tid >> 5), &tm_in, bars, phase);
  }
  if (!use_clock) return;

  // the last block to finish advances the loop state (src/main.cpp:139-143)
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned int nblocks = gridDim.x;
    const unsigned int ticket = atomicAdd(&clk->done_blocks, 1u);
    if (ticket == nblocks - 1) {
      __threadfence();
      const double dt = s_dt[0];
      const int ns = clk->nstep;
      const int tslot = ns - clk->trace_base;
      if (clk->trace && tslot >= 0 && tslot < clk->trace_cap) clk->trace[tslot] = dt;
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

// ------------------------------------------------------------ batches
// The loop-state advance of src/main.cpp:139-143 plus the next dt (:128-134)
// for one instance; run by the instance's last strip of an iteration.
__device__ __forceinline__ void batch_finalize(BatchInst &I) {
  const int n = I.nstep;
  const double dt = I.dt;
  if (!(dt > 0.0) || nonfinite64(dt)) I.status |= E2D_FLAG_BAD_DT;
  const double t = I.t + dt;
  I.t = t;
  I.nstep = n + 1;
  I.par ^= 1;
  I.acc[n & 1] = 0ull;
  const double inv_dt = __longlong_as_double((long long)I.acc[(n + 1) & 1]);
  double dtn = I.kp.ph64.cfl / inv_dt;
  if (t + dtn > I.t_end) dtn = I.t_end - t;
  I.dt = dtn;
  I.dtdx = (float)(dtn / I.kp.ph64.dx);
  I.dtdy = (float)(dtn / I.kp.ph64.dy);
  I.active = (t < I.t_end) && !(I.status & (E2D_FLAG_NONFINITE | E2D_FLAG_BAD_DT | E2D_FLAG_TIMEOUT));
  I.done = 0u;
}

// One iteration of a batch: every warp takes strips of the global strip list
// (instances concatenated) with a grid-sized stride, marches them with its
// instance's own dt, folds the instance's next CFL maximum, and the last
// strip of each instance advances that instance's loop state.  Results of an
// instance do not depend on the other instances in the batch.
template <int RS, int MINB, int PFD, int TMA>
__global__ void __launch_bounds__(NT, MINB)
    k_batch_f32c(BatchInst *__restrict__ insts, const int *__restrict__ list_slots,
                 const int *__restrict__ strip_begin, const int n_inst, const int total_strips) {
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * WPB;
  __shared__ unsigned long long s_bars[TMA ? WPB * kMaxSlots : 1];  // ring slot barriers, per warp
  unsigned long long *bars = s_bars + (TMA ? (threadIdx.x >> 5) * kMaxSlots : 0);
  unsigned int phase = 0u;  // carried across the warp's strips
  bool ring_ok = true;      // false after a TMA wait gave up with a copy maybe in flight
  if (TMA && PFD > 0) ring_bars_init(bars, PFD + 3, lane);
  for (int w = blockIdx.x * WPB + (threadIdx.x >> 5); w < total_strips; w += nwarps) {
    // instance k with strip_begin[k] <= w < strip_begin[k + 1]
    int lo = 0, hi = n_inst;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (strip_begin[mid] <= w)
        lo = mid;
      else
        hi = mid;
    }
    BatchInst &I = insts[list_slots[lo]];
    if (!I.active) continue;  // warp-uniform
    const KParams32 &kp = I.kp;
    const int par = I.par;
    const int strip = w - strip_begin[lo];
    if (ring_ok) {
      // the general march only: a persistent warp takes strips of many
      // instances, mostly boundary strips of small grids, and a second
      // instantiation in this loop measured 14 % slower on the 512-solve mix
      ring_ok = march_strip_t<RS, PFD, TMA, false, false>(kp, I.w[par], I.w[par ^ 1], f2(I.dtdx), f2(I.dtdy),
                                                          strip % I.nsx, strip / I.nsx, lane,
                                                          &I.acc[(I.nstep + 1) & 1], &I.status,
                                                          warp_ring<PFD>(threadIdx.x >> 5), &I.tm[par], bars, phase);
    } else if (lane == 0) {
      // a copy of an abandoned strip may still land in this warp's ring:
      // its remaining strips are not computed, their instances stop
      atomicOr(&I.status, (unsigned)E2D_FLAG_TIMEOUT);
    }
    if (lane == 0) {
      __threadfence();
      const unsigned int ticket = atomicAdd(&I.done, 1u);
      if (ticket == (unsigned)I.nstrips - 1u) {
        __threadfence();
        batch_finalize(I);
        __threadfence();
      }
    }
    __syncwarp();
  }
}

__global__ void k_batch_arm(BatchInst *I) {
  const double inv_dt = __longlong_as_double((long long)I->acc[I->nstep & 1]);
  double dt = I->kp.ph64.cfl / inv_dt;
  if (I->t + dt > I->t_end) dt = I->t_end - I->t;
  I->dt = dt;
  I->dtdx = (float)(dt / I->kp.ph64.dx);
  I->dtdy = (float)(dt / I->kp.ph64.dy);
  I->active = (I->t < I->t_end) && !(I->status & (E2D_FLAG_NONFINITE | E2D_FLAG_BAD_DT | E2D_FLAG_TIMEOUT));
  I->done = 0u;
}

}  // namespace

int strips_of(const KParams32 &kp) {
  const int nsx = (kp.g.nx + OUTW - 1) / OUTW;
  return nsx * ((kp.g.ny + kp.strip_h - 1) / kp.strip_h);
}

// Kernel variants: (MINB, PFD) = minimum resident blocks of 128 threads per
// SM (the register budget) and the row-staging distance (0: registers).
template <class F>
static void with_variant(int v, F &&f) {
  using std::integral_constant;
  using I0 = integral_constant<int, 0>;
  using I1 = integral_constant<int, 1>;
  switch (v) {
    case 0: f(integral_constant<int, 1>{}, I0{}, I0{}); break;
    case 2: f(integral_constant<int, 3>{}, I0{}, I0{}); break;
    case 3: f(integral_constant<int, 2>{}, I0{}, I0{}); break;
    case 4: f(integral_constant<int, 3>{}, integral_constant<int, 2>{}, I0{}); break;
    case 5: f(integral_constant<int, 4>{}, integral_constant<int, 2>{}, I0{}); break;
    case 6: f(integral_constant<int, 4>{}, integral_constant<int, 2>{}, I1{}); break;
    default: f(integral_constant<int, 4>{}, I0{}, I0{}); break;
  }
}
static_assert(kF32cVariants == 7, "with_variant covers variants 0..6");

// The single-grid step's variants: those of with_variant, plus variant 7
// (MINB 3, rows staged three ahead, interior strips by one TMA copy per two
// rows).  Batches keep variants 0..6: their instances' maps have one-row boxes.
template <class F>
static void with_step_variant(int v, F &&f) {
  if (v == 7) {
    f(std::integral_constant<int, 3>{}, std::integral_constant<int, 3>{}, std::integral_constant<int, 2>{});
    return;
  }
  with_variant(v, static_cast<F &&>(f));
}

template <int MINB, int PFD, int TMA>
static void launch_batch_v(int riemann, BatchInst *insts, const int *slots, const int *sb, int n, int total,
                           int grid, cudaStream_t s) {
  const size_t sm = ring_bytes(PFD);
  switch (riemann) {
    case E2D_RIEMANN_HLLC:
      k_batch_f32c<E2D_RIEMANN_HLLC, MINB, PFD, TMA><<<grid, NT, sm, s>>>(insts, slots, sb, n, total);
      break;
    case E2D_RIEMANN_HLL:
      k_batch_f32c<E2D_RIEMANN_HLL, MINB, PFD, TMA><<<grid, NT, sm, s>>>(insts, slots, sb, n, total);
      break;
    default:
      k_batch_f32c<E2D_RIEMANN_APPROX, MINB, PFD, TMA><<<grid, NT, sm, s>>>(insts, slots, sb, n, total);
      break;
  }
}

cudaError_t launch_batch_f32c(int riemann, int variant, BatchInst *insts, const int *list_slots,
                              const int *strip_begin, int n_inst, int total_strips, int grid_blocks,
                              cudaStream_t s) {
  if (n_inst <= 0 || total_strips <= 0) return cudaSuccess;
  with_variant(variant, [&](auto minb, auto pfd, auto tma) {
    launch_batch_v<decltype(minb)::value, decltype(pfd)::value, decltype(tma)::value>(riemann, insts, list_slots, strip_begin, n_inst,
                                                                total_strips, grid_blocks, s);
  });
  return cudaGetLastError();
}

cudaError_t launch_batch_arm(BatchInst *inst, cudaStream_t s) {
  k_batch_arm<<<1, 1, 0, s>>>(inst);
  return cudaGetLastError();
}

template <int RS>
static int batch_occupancy(int variant) {
  int n = 0;
  cudaError_t e = cudaErrorInvalidValue;
  with_variant(variant, [&](auto minb, auto pfd, auto tma) {
    constexpr int M = decltype(minb)::value, P = decltype(pfd)::value, T = decltype(tma)::value;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_f32c<RS, M, P, T>, NT, ring_bytes(P));
  });
  return (e == cudaSuccess && n > 0) ? n : 1;
}

int batch_blocks_per_sm(int riemann, int variant) {
  switch (riemann) {
    case E2D_RIEMANN_HLLC: return batch_occupancy<E2D_RIEMANN_HLLC>(variant);
    case E2D_RIEMANN_HLL: return batch_occupancy<E2D_RIEMANN_HLL>(variant);
    default: return batch_occupancy<E2D_RIEMANN_APPROX>(variant);
  }
}

// Rows per warp strip: the largest of 64, 32, 16 that still gives at least
// four waves of strips for the resident warps (152 SMs x 12 warps of the
// default variant): taller strips cost less halo ((h + 4) / h rows loaded per
// output row), more waves leave less of the last one idle.  Measured, FP32C
// HLLC: 8192^2 64 rows (55.4 Gcell/s; 32: 54.0), 4096^2 32 rows (48.5; 64:
// 46.8, 16: 45.2), 2048^2 all within 1 %.
int default_strip_h(int nx, int ny) {
  const long long nsx = (nx + OUTW - 1) / OUTW;
  for (int h = 64; h > 16; h /= 2)
    if (nsx * ((ny + h - 1) / h) >= 152LL * 12 * 4) return h;
  return 16;
}

void make_kparams32(const e2d_params &p, KParams32 *kp) {
  KParams64 k64;
  make_kparams(p, &k64);
  kp->g = k64.g;
  kp->ph64 = k64.ph;
  const KPhys<double> &d = k64.ph;
  kp->ph = KPhys<float>{(float)d.gamma0, (float)d.gamma6, (float)d.cfl, (float)d.slope_type,
                        (float)d.smallr, (float)d.smallc, (float)d.smallp, (float)d.smallpp,
                        (float)d.gm1, (float)d.entho, (float)d.smallc2, (float)d.dx, (float)d.dy};
  kp->wpitch = (p.isize + 3) & ~3;
  kp->wplane = (long long)kp->wpitch * p.jsize;
  kp->variant = 4;  // 3 blocks per SM, rows staged by cp.async (fastest at 8192^2)
  kp->strip_h = default_strip_h(p.nx, p.ny);
  const char *wt = std::getenv("E2D_TEST_WAIT_TIMEOUT");
  kp->wait_test = (wt && std::atoi(wt) != 0) ? 1 : 0;
}

// Dynamic plus static shared memory above 48 KB must be enabled per kernel
// before the first launch (and before any graph capture).
template <int RS>
static cudaError_t configure_rs() {
  cudaError_t e = cudaSuccess;
  for (int v = 0; v < kF32cVariants && e == cudaSuccess; ++v)
    with_variant(v, [&](auto minb, auto pfd, auto tma) {
      constexpr int M = decltype(minb)::value, P = decltype(pfd)::value, T = decltype(tma)::value;
      if (P > 0) {  // the kernels' static shared memory comes on top of the ring
        e = cudaFuncSetAttribute(k_step_f32c<RS, M, P, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ring_bytes(P));
        if (e == cudaSuccess)
          e = cudaFuncSetAttribute(k_batch_f32c<RS, M, P, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)ring_bytes(P));
      }
    });
  if (e == cudaSuccess)  // variant 7 (single-grid step only)
    e = cudaFuncSetAttribute(k_step_f32c<RS, 3, 3, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ring_bytes(3));
  return e;
}

cudaError_t configure_f32c_kernels() {
  cudaError_t e = configure_rs<E2D_RIEMANN_HLLC>();
  if (e == cudaSuccess) e = configure_rs<E2D_RIEMANN_HLL>();
  if (e == cudaSuccess) e = configure_rs<E2D_RIEMANN_APPROX>();
  return e;
}

cudaError_t launch_f32c_from_f64(const KParams32 &kp, const double *u, float *w, cudaStream_t s) {
  dim3 block(64, 4);
  dim3 grid((kp.g.isize + 63) / 64, (kp.g.jsize + 3) / 4);
  k_f32c_from_f64<<<grid, block, 0, s>>>(kp, u, w);
  return cudaGetLastError();
}

cudaError_t launch_f32c_to_f64(const KParams32 &kp, const float *w, double *u, cudaStream_t s) {
  dim3 block(64, 4);
  dim3 grid((kp.g.isize + 63) / 64, (kp.g.jsize + 3) / 4);
  k_f32c_to_f64<<<grid, block, 0, s>>>(kp, w, u);
  return cudaGetLastError();
}

cudaError_t launch_f32c_dt_to(const KParams32 &kp, const float *w, unsigned long long *target,
                              unsigned int *status, cudaStream_t s) {
  const long long units = (long long)((kp.g.nx + OUTW - 1) / OUTW) * ((kp.g.ny + CFL_UNIT_ROWS - 1) / CFL_UNIT_ROWS);
  long long blocks = (units + WPB - 1) / WPB;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_f32c_dt<<<(int)blocks, NT, 0, s>>>(kp, w, target, status);
  return cudaGetLastError();
}

cudaError_t launch_f32c_dt(const KParams32 &kp, const float *w, DevClock *clk, int slot, cudaStream_t s) {
  return launch_f32c_dt_to(kp, w, slot < 0 ? &clk->invdt_bits : &clk->acc[slot], &clk->status, s);
}

template <int MINB, int PFD, int TMA>
static void launch_step_v(const KParams32 &kp, int riemann, int blocks, const float *w_in, float *w_out,
                          const CUtensorMap &tm, DevClock *clk, int use_clock, double host_dt, cudaStream_t s) {
  const size_t sm = ring_bytes(PFD);
  switch (riemann) {
    case E2D_RIEMANN_HLLC:
      k_step_f32c<E2D_RIEMANN_HLLC, MINB, PFD, TMA><<<blocks, NT, sm, s>>>(kp, w_in, w_out, tm, clk, use_clock, host_dt);
      break;
    case E2D_RIEMANN_HLL:
      k_step_f32c<E2D_RIEMANN_HLL, MINB, PFD, TMA><<<blocks, NT, sm, s>>>(kp, w_in, w_out, tm, clk, use_clock, host_dt);
      break;
    default:
      k_step_f32c<E2D_RIEMANN_APPROX, MINB, PFD, TMA><<<blocks, NT, sm, s>>>(kp, w_in, w_out, tm, clk, use_clock,
                                                                        host_dt);
      break;
  }
}

cudaError_t launch_f32c_step(const KParams32 &kp, int riemann, const float *w_in, float *w_out,
                             const CUtensorMap &tm_in, DevClock *clk, int use_clock, double host_dt,
                             cudaStream_t s) {
  const int nsx = (kp.g.nx + OUTW - 1) / OUTW;
  const int nsy = (kp.g.ny + kp.strip_h - 1) / kp.strip_h;
  const int blocks = (nsx * nsy + WPB - 1) / WPB;
  with_step_variant(kp.variant, [&](auto minb, auto pfd, auto tma) {
    launch_step_v<decltype(minb)::value, decltype(pfd)::value, decltype(tma)::value>(kp, riemann, blocks, w_in, w_out, tm_in, clk,
                                                               use_clock, host_dt, s);
  });
  return cudaGetLastError();
}

// The TMA map of a state array: dimensions (wpitch, jsize, 8 planes), row
// and plane strides in bytes (multiples of 16: wpitch is a multiple of 4),
// box 64 x 1 x 8 (variant 7: 64 x 2 x 8, two rows per copy).  The encoder comes from the driver through the runtime's
// versioned entry point (no link against the driver library).
bool encode_f32c_map(CUtensorMap *map, const float *w, const KParams32 &kp) {
  // looked up once (thread-safe static initialisation); null if unavailable
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode) return false;
  if ((reinterpret_cast<uintptr_t>(w) & 15u) != 0 || (kp.wpitch & 3) != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)kp.wpitch, (cuuint64_t)kp.g.jsize, 8};
  const cuuint64_t strides[2] = {(cuuint64_t)kp.wpitch * sizeof(float), (cuuint64_t)kp.wplane * sizeof(float)};
  const cuuint32_t box[3] = {64, kp.variant == 7 ? 2u : 1u, 8};
  const cuuint32_t estr[3] = {1, 1, 1};
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(w), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace e2d
