/*
 * hydro_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of HydroCODE's Eulerian Godunov/GRP step (1D and 2D
 * structured, single-fluid, ideal gas) that the CUDA path is tested
 * against, and the timed CPU baseline ("port").  It is pinned against the
 * reference itself (oracle/_ref, built by oracle/Makefile) and against the
 * golden fixtures in tests/golden/.  Nothing in the product links it.
 *
 * The entry points have the same signatures as the ref_* functions of
 * ref_harness.c so tests can run either side on identical inputs.
 */
#ifndef HYDRO_ORACLE_H
#define HYDRO_ORACLE_H

#define ORC_NCONF 400

int orc_run_2d(int m, int n, double *rho, double *u, double *v, double *p, double *E,
               const double *cfg, int ncfg, int split, int threads,
               const double *plot_times, int nplot_in, double *snaps, int *nsnap_out,
               double *info);
int orc_run_1d(int m, double *rho, double *u, double *p, double *E_out,
               const double *cfg, int ncfg, int order, double *info);

void orc_riemann_exact(int cnt, const double *in, double eps, double tol, int N, double *out);
void orc_riemann_exact_ben(int cnt, const double *in, double eps, double tol, int N, double *out);
void orc_grp2d_flux(int cnt, const double *in, double tau, double eps, double *out);
/* GRP_2D_flux of the two-component (MULTIFLUID_BASICS) build: rows of 40 in, 19 out. */
void orc_grp2d_flux_mf(int cnt, const double *in, double tau, double eps, double gamma_a, double gamma_b,
                       int store_gamma, double *out);
void orc_q1d(int cnt, const double *in, double eps, double atc, double *out);
void orc_g2d(int cnt, const double *in, double eps, double atc, double *out);
int orc_run_1d_lag(int m, double *rho, double *u, double *p, double *E_out, double *X_out,
                   const double *cfg_in, int ncfg, int order, double *info);
void orc_lag(int cnt, const double *in, double eps, double atc, double *out);
void orc_grp1d(int cnt, const double *in, double eps, double atc, double *out);

/* Newton iteration count of the exact solver (same inputs as orc_riemann_exact);
 * out: cnt x 6 = u*, p*, CRW0, CRW1, gap, iterations. */
void orc_riemann_exact_iters(int cnt, const double *in, double eps, double tol, int N, double *out);

#endif
