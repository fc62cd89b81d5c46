/*
 * e2d_oracle.h -- CPU restatement of the reference's MUSCL-Hancock unsplit
 * Godunov step (euler2d_kokkos, impl 0), in plain C, double precision.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity checker for the GPU path:
 * tests/, the smoke check and the benchmark's CPU-baseline leg may call it;
 * the product never does.  It is pinned against the reference itself
 * (oracle/_ref, built from the reference sources) by tests/golden/.
 *
 * Arrays are the reference's DataArray on its CUDA backend: LayoutLeft,
 * element (i, j, v) at i + isize * (j + jsize * v), v in {rho, E, mx, my}.
 */
#ifndef E2D_ORACLE_H
#define E2D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_ID = 0, ORC_IP = 1, ORC_IU = 2, ORC_IV = 3 };
enum { ORC_FACE_XMIN = 0, ORC_FACE_XMAX = 1, ORC_FACE_YMIN = 2, ORC_FACE_YMAX = 3 };
enum { ORC_BC_REFLECT = 1, ORC_BC_ABSORB = 2, ORC_BC_PERIODIC = 3 };
enum { ORC_RIEMANN_APPROX = 0, ORC_RIEMANN_HLL = 1, ORC_RIEMANN_HLLC = 2 };

typedef struct orc_params {
  int nx, ny, ghost, isize, jsize;
  double xmin, xmax, ymin, ymax, dx, dy;
  int bc_xmin, bc_xmax, bc_ymin, bc_ymax;
  double gamma0, gamma6, cfl, slope_type, smallr, smallc, smallp, smallpp;
  int riemann;
} orc_params;

/* HydroParams::init (src/HydroParams.cpp:160-190): derived sizes and cut-offs. */
void orc_params_init(orc_params *p);

void orc_primitives(const orc_params *p, const double u[4], double q[4], double *c);
void orc_slopes(const orc_params *p, const double q[4], const double qpx[4], const double qmx[4],
                const double qpy[4], const double qmy[4], double dqx[4], double dqy[4]);
void orc_trace(const orc_params *p, const double q[4], const double dqx[4], const double dqy[4],
               double dtdx, double dtdy, int face, double qface[4]);
void orc_riemann(const orc_params *p, int solver, const double ql[4], const double qr[4],
                 double flux[4]);

void orc_make_boundaries(const orc_params *p, double *u);
double orc_compute_dt(const orc_params *p, const double *u);
/* One godunov_unsplit_impl call (impl 0).  work holds 3 full arrays (Q, Fx, Fy). */
void orc_godunov_step(const orc_params *p, double *u_in, double *u_out, double dt, double *work);
/* The src/main.cpp:87-145 loop; returns the number of steps taken.  u and u2
 * are the two state arrays (u holds the initial condition); on return the
 * current state is u after an even number of steps, else u2. */
int orc_run(const orc_params *p, double *u, double *u2, int nstep_max, double t_end,
            double *dt_trace, double *t_out);

/* Initial conditions of src/HydroRunFunctors.h:1347-1827, parametrised. */
void orc_init_implode(const orc_params *p, double *u, int reference_shape);
/* ComputeRadialProfileFunctor (src/ComputeRadialProfileFunctor.h:83-165):
 * mean density in nbins rings about the box centre over every cell of the
 * array, ghosts included, summed j outer / i inner.  Cells whose ring index
 * is >= nbins (ghost corners) are not counted -- the reference writes them
 * past the end of its histograms.  An empty ring gives 0/0 (NaN), as there. */
void orc_radial_profile(const orc_params *p, const double *u, int nbins, double *distances,
                        double *profile, long long *counts);

void orc_init_blast(const orc_params *p, double *u, double radius, double cx, double cy,
                    double d_in, double d_out, double p_in, double p_out);
void orc_init_four_quadrant(const orc_params *p, double *u, double xt, double yt,
                            const double prim[16]);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
