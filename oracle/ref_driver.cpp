// C entry points around the reference euler2d solver, compiled from the
// reference's own unmodified sources against the host-only Kokkos stand-in in
// kokkos_compat/.  Test infrastructure only: it runs the reference so that
// the C restatement (e2d_oracle.c) and the golden fixtures can be checked
// against it.  Built by oracle/Makefile into oracle/_ref/libe2d_ref.so (the
// reference's FP64 build, USE_DOUBLE) and oracle/_ref/libe2d_ref32.so (its
// single-precision build).
//
// The run loop follows src/main.cpp:76-145 (compute_dt before the boundary
// fill, the loop condition, the dt clamp at tEnd, the U/U2 ping-pong) without
// the banner, the output and the timers' report.
#include "ComputeRadialProfileFunctor.h"
#include "HydroParams.h"
#include "HydroRun.h"
#include "config/ConfigMap.h"

#include <omp.h>
#include <unistd.h>

#include <cstring>

using namespace euler2d;
using Dev = Kokkos::Device<Kokkos::DefaultExecutionSpace, Kokkos::HostSpace>;

namespace
{
// Exposes the protected-by-convention numerical routines of
// HydroBaseFunctor (HydroBaseFunctor.h) to the C entry points below.
struct Probe : public HydroBaseFunctor
{
  explicit Probe(const HydroParams & p)
    : HydroBaseFunctor(p)
  {}
};

HydroState
load4(const double * v)
{
  HydroState s;
  for (int k = 0; k < 4; ++k)
    s[k] = v[k];
  return s;
}
void
store4(const HydroState & s, double * v)
{
  for (int k = 0; k < 4; ++k)
    v[k] = s[k];
}

// The reference's real_t is double under USE_DOUBLE (libe2d_ref.so) and
// float without it (libe2d_ref32.so); the entry points take and return FP64
// arrays either way (a plain copy in the double build).
void
to_real(real_t * dst, const double * src, long n)
{
  for (long k = 0; k < n; ++k)
    dst[k] = (real_t)src[k];
}
void
to_double(double * dst, const real_t * src, long n)
{
  for (long k = 0; k < n; ++k)
    dst[k] = (double)src[k];
}

HydroParams
params_from_ini(const char * ini)
{
  ConfigMap   cm{ std::string(ini) };
  HydroParams p;
  p.setup(cm);
  return p;
}
} // namespace

extern "C"
{

  // Scalars that HydroParams::setup/init derive from an ini file, in this
  // order: nx ny isize jsize dx dy gamma0 gamma6 cfl slope_type smallr smallc
  // smallp smallpp tEnd nStepmax bc_xmin bc_xmax bc_ymin bc_ymax riemann
  // problem impl xmin xmax ymin ymax.
  int
  ref_params(const char * ini, double * out)
  {
    HydroParams p = params_from_ini(ini);
    const double v[] = { (double)p.nx,
                         (double)p.ny,
                         (double)p.isize,
                         (double)p.jsize,
                         p.dx,
                         p.dy,
                         p.settings.gamma0,
                         p.settings.gamma6,
                         p.settings.cfl,
                         p.settings.slope_type,
                         p.settings.smallr,
                         p.settings.smallc,
                         p.settings.smallp,
                         p.settings.smallpp,
                         p.tEnd,
                         (double)p.nStepmax,
                         (double)p.boundary_type_xmin,
                         (double)p.boundary_type_xmax,
                         (double)p.boundary_type_ymin,
                         (double)p.boundary_type_ymax,
                         (double)p.riemannSolverType,
                         (double)p.problemType,
                         (double)p.implementationVersion,
                         p.xmin,
                         p.xmax,
                         p.ymin,
                         p.ymax };
    std::memcpy(out, v, sizeof(v));
    return (int)(sizeof(v) / sizeof(double));
  }

  // Full run as src/main.cpp does it.  If u0 is non-null it replaces the
  // initial condition (the whole isize*jsize*4 LayoutLeft array) before U2 is
  // copied from U.  nstep_limit >= 0 overrides nStepmax.  On return u_out
  // holds the current state (U after an even number of steps, else U2),
  // dt_trace[k] the dt used by step k, *nstep and *t the loop counters.
  int
  ref_run(const char * ini,
          const double * u0,
          int            nstep_limit,
          double *       u_out,
          double *       dt_trace,
          int *          nstep,
          double *       t_out)
  {
    ConfigMap   cm{ std::string(ini) };
    HydroParams params;
    params.setup(cm);
    if (nstep_limit >= 0)
      params.nStepmax = nstep_limit;
    params.enableOutput = false;

    HydroRun<Dev> hydro(params, cm);
    const long    n = (long)params.isize * params.jsize * 4;
    if (u0)
    {
      to_real(hydro.U.data(), u0, n);
      Kokkos::deep_copy(hydro.U2, hydro.U);
    }

    double t = 0, dt = 0;
    int    ns = 0;
    dt = hydro.compute_dt(ns % 2);
    hydro.make_boundaries(hydro.U);
    hydro.make_boundaries(hydro.U2);
    while (t < params.tEnd && ns < params.nStepmax)
    {
      dt = hydro.compute_dt(ns % 2);
      if (t + dt > params.tEnd)
        dt = params.tEnd - t;
      if (dt_trace)
        dt_trace[ns] = dt;
      hydro.godunov_unsplit(ns, dt);
      ns++;
      t += dt;
    }
    const real_t * cur = (ns % 2 == 0) ? hydro.U.data() : hydro.U2.data();
    if (u_out)
      to_double(u_out, cur, n);
    *nstep = ns;
    *t_out = t;
    return 0;
  }

  // The initial condition HydroRun's constructor builds for this ini
  // (src/HydroRun.h:185-214), before any boundary fill.
  int
  ref_initial_state(const char * ini, double * u_out)
  {
    ConfigMap   cm{ std::string(ini) };
    HydroParams params;
    params.setup(cm);
    HydroRun<Dev> hydro(params, cm);
    to_double(u_out, hydro.U.data(), (long)params.isize * params.jsize * 4);
    return 0;
  }

  // HydroRun::saveData -> saveVTK (src/HydroRun.h:486-609) of a
  // caller-supplied state: writes <outputDir>/<outputPrefix>_<iStep, 7
  // digits>.vti as the ini's [output] section names it.
  int
  ref_save_vtk(const char * ini, const double * u, int iStep)
  {
    ConfigMap   cm{ std::string(ini) };
    HydroParams params;
    params.setup(cm);
    HydroRun<Dev> hydro(params, cm);
    to_real(hydro.U.data(), u, (long)params.isize * params.jsize * 4);
    hydro.saveData(hydro.U, iStep, "U");
    return 0;
  }

  // make_boundaries (src/HydroRun.h:388-399) applied in place to u.
  int
  ref_make_boundaries(const char * ini, double * u)
  {
    ConfigMap   cm{ std::string(ini) };
    HydroParams params;
    params.setup(cm);
    HydroRun<Dev> hydro(params, cm);
    const long    n = (long)params.isize * params.jsize * 4;
    to_real(hydro.U.data(), u, n);
    hydro.make_boundaries(hydro.U);
    to_double(u, hydro.U.data(), n);
    return 0;
  }

  // The Sedov post-processing of src/main.cpp:175-179:
  // ComputeRadialProfileFunctor::apply (src/ComputeRadialProfileFunctor.h:83-134)
  // on a caller-supplied state.  It writes sedov_blast_radial_distances.npy
  // and sedov_blast_density_profile.npy into outdir.  Runs on one thread: the
  // stand-in View has no atomic accessor, and one thread also fixes the
  // summation order (j outer, i inner).
  int
  ref_radial_profile(const char * ini, const double * u, const char * outdir)
  {
    ConfigMap   cm{ std::string(ini) };
    HydroParams params;
    params.setup(cm);
    DataArray<Dev> U("U", params.isize, params.jsize);
    to_real(U.data(), u, (long)params.isize * params.jsize * 4);
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd) || chdir(outdir) != 0)
      return 1;
    const int threads = omp_get_max_threads();
    omp_set_num_threads(1);
    ComputeRadialProfileFunctor<Dev>::apply(params, U);
    omp_set_num_threads(threads);
    return chdir(cwd) == 0 ? 0 : 1;
  }

  // compute_dt (src/HydroRun.h:227-251) on a caller-supplied state.
  double
  ref_compute_dt(const char * ini, const double * u)
  {
    ConfigMap   cm{ std::string(ini) };
    HydroParams params;
    params.setup(cm);
    HydroRun<Dev> hydro(params, cm);
    to_real(hydro.U.data(), u, (long)params.isize * params.jsize * 4);
    return hydro.compute_dt(0);
  }

  // Batched per-function probes of HydroBaseFunctor, n states each.
  void
  ref_primitives(const char * ini, int n, const double * u, double * q, double * c)
  {
    Probe f(params_from_ini(ini));
    for (int k = 0; k < n; ++k)
    {
      HydroState qs;
      real_t     ck;
      f.computePrimitives(load4(u + 4 * k), &ck, qs);
      c[k] = ck;
      store4(qs, q + 4 * k);
    }
  }

  void
  ref_slopes(const char * ini, int n, const double * q5, double * dqx, double * dqy)
  {
    // q5 holds, per sample, 5 states: q, q(+x), q(-x), q(+y), q(-y).
    Probe f(params_from_ini(ini));
    for (int k = 0; k < n; ++k)
    {
      const double * s = q5 + 20 * k;
      HydroState     ax, ay;
      f.slope_unsplit_hydro_2d(
        load4(s), load4(s + 4), load4(s + 8), load4(s + 12), load4(s + 16), ax, ay);
      store4(ax, dqx + 4 * k);
      store4(ay, dqy + 4 * k);
    }
  }

  void
  ref_trace(const char *   ini,
            int            n,
            const double * q,
            const double * dqx,
            const double * dqy,
            double         dtdx,
            double         dtdy,
            int            face,
            double *       qface)
  {
    Probe f(params_from_ini(ini));
    for (int k = 0; k < n; ++k)
    {
      HydroState out;
      f.trace_unsplit_2d_along_dir(
        load4(q + 4 * k), load4(dqx + 4 * k), load4(dqy + 4 * k), dtdx, dtdy, face, out);
      store4(out, qface + 4 * k);
    }
  }

  void
  ref_riemann(const char * ini, int solver, int n, const double * ql, const double * qr, double * flux)
  {
    // solver: 0 = riemann_approx, 2 = riemann_hllc (the reference has no HLL).
    Probe f(params_from_ini(ini));
    for (int k = 0; k < n; ++k)
    {
      HydroState g, fl;
      if (solver == 0)
        f.riemann_approx(load4(ql + 4 * k), load4(qr + 4 * k), g, fl);
      else
        f.riemann_hllc(load4(ql + 4 * k), load4(qr + 4 * k), g, fl);
      store4(fl, flux + 4 * k);
    }
  }

} // extern "C"
