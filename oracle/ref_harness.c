/*
 * ref_harness.c -- TEST INFRASTRUCTURE ONLY (the oracle's checker side).
 *
 * Flat C entry points around the reference's own, unmodified hot-path sources
 * (compiled from their place in the reference tree by oracle/Makefile).  The
 * harness owns the global `config[]` the reference reads, builds the
 * reference's x-major `struct cell_var_stru` arrays, calls the reference's
 * scheme entry points and point solvers, and hands back raw float64 results
 * (the reference's own writers print only `%.10g`).
 *
 * Nothing in the product links this file.  It exists to pin the C restatement
 * in oracle/hydro_oracle.c and to generate the golden fixtures under
 * tests/golden/.
 *
 * Mirrors the driver set-up of src/hydrocode_2D/hydrocode.c:164-274 and
 * src/hydrocode_1D/hydrocode.c:150-273 (config[] defaults to INFINITY,
 * E initialisation, CV[0] filled, N_plot/time_plot from time_plot_read
 * src/file_io/io_control.c:288-335 when no time_plot file exists).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdbool.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "var_struc.h"
#include "finite_volume.h"
#include "riemann_solver.h"
#include "flux_calc.h"

double config[N_CONF];

/* Silent replacement for the progress bar in src/tools/sys_pro.c:37 (the
 * reference's version writes escape sequences on every step). */
void DispPro(const double pro, const int step) { (void)pro; (void)step; }

static double wall(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return (double)clock() / CLOCKS_PER_SEC;
#endif
}

static void load_config(const double *cfg, int ncfg)
{
    int k;
    for (k = 0; k < N_CONF; ++k)
        config[k] = INFINITY;
    for (k = 0; k < ncfg && k < N_CONF; ++k)
        config[k] = cfg[k];
}

static void set_threads(int threads)
{
#ifdef _OPENMP
    if (threads > 0)
        omp_set_num_threads(threads);
#else
    (void)threads;
#endif
}

static double **alloc2(int a, int b)
{
    double **p = (double **)malloc(a * sizeof(double *));
    for (int j = 0; j < a; ++j)
        p[j] = (double *)malloc((b > 0 ? b : 1) * sizeof(double));
    return p;
}

static void free2(double **p, int a)
{
    if (!p)
        return;
    for (int j = 0; j < a; ++j)
        free(p[j]);
    free(p);
}

/*
 * 2D run.  Arrays are x-major flat: value of cell (x=j, y=i) at [j*n + i].
 * cfg[0..ncfg) is copied into config[] (missing entries stay INFINITY), so the
 * caller passes an already checked configuration (config_check semantics are
 * the caller's job, as configurate() runs before the scheme in the driver).
 * plot_times (nplot_in entries, may be NULL) play the role of a time_plot file.
 * snaps (may be NULL) receives every stored snapshot CV[0..N_plot-1] as
 * 5 planes (RHO,U,V,P,E) each; nsnap_out gets N_plot.
 * info: [0]=config[5] written back, [1]=time_plot[N_plot-1],
 *       [2]=cpu_time[N_plot-1] (the reference's own timer), [3]=wall seconds.
 */
int ref_run_2d(int m, int n, double *rho, double *u, double *v, double *p, double *E,
               const double *cfg, int ncfg, int split, int threads,
               const double *plot_times, int nplot_in, double *snaps, int *nsnap_out,
               double *info)
{
    int j, i, k;
    load_config(cfg, ncfg);
    set_threads(threads);
    config[0] = 2.0;
    const double gamma = config[6];

    int N_plot = (plot_times && nplot_in > 0) ? nplot_in + 2 : 2;
    double *time_plot = (double *)malloc(N_plot * sizeof(double));
    time_plot[0] = 0.0;
    time_plot[N_plot - 1] = config[1];
    for (k = 0; k < N_plot - 2; ++k)
        time_plot[k + 1] = plot_times[k];
    int N_T = N_plot < 5 ? N_plot : 5;

    struct cell_var_stru *CV = (struct cell_var_stru *)calloc(N_T, sizeof(struct cell_var_stru));
    for (k = 0; k < N_T; ++k) {
        CV[k].RHO = alloc2(m, n);
        CV[k].U = alloc2(m, n);
        CV[k].V = alloc2(m, n);
        CV[k].P = alloc2(m, n);
        CV[k].E = alloc2(m, n);
    }
    double **X = alloc2(m + 1, n + 1), **Y = alloc2(m + 1, n + 1);
    for (j = 0; j <= m; ++j)
        for (i = 0; i <= n; ++i) {
            X[j][i] = j * config[10];
            Y[j][i] = i * config[11];
        }
    for (j = 0; j < m; ++j)
        for (i = 0; i < n; ++i) {
            CV[0].RHO[j][i] = rho[j * n + i];
            CV[0].U[j][i] = u[j * n + i];
            CV[0].V[j][i] = v[j * n + i];
            CV[0].P[j][i] = p[j * n + i];
            CV[0].E[j][i] = 0.5 * CV[0].U[j][i] * CV[0].U[j][i] + CV[0].P[j][i] / (gamma - 1.0) / CV[0].RHO[j][i];
            CV[0].E[j][i] += 0.5 * CV[0].V[j][i] * CV[0].V[j][i];
        }
    double *cpu_time = (double *)calloc(N_T, sizeof(double));

    double t0 = wall();
    if (split)
        GRP_solver_2D_split_EUL_source(m, n, CV, X, Y, cpu_time, "oracle", N_T, &N_plot, time_plot);
    else
        GRP_solver_2D_EUL_source(m, n, CV, X, Y, cpu_time, "oracle", N_T, &N_plot, time_plot);
    double t1 = wall();

    int last = N_plot - 1;
    for (j = 0; j < m; ++j)
        for (i = 0; i < n; ++i) {
            rho[j * n + i] = CV[last].RHO[j][i];
            u[j * n + i] = CV[last].U[j][i];
            v[j * n + i] = CV[last].V[j][i];
            p[j * n + i] = CV[last].P[j][i];
            if (E)
                E[j * n + i] = CV[last].E[j][i];
        }
    if (snaps)
        for (k = 0; k < N_plot; ++k)
            for (j = 0; j < m; ++j)
                for (i = 0; i < n; ++i) {
                    size_t b = (size_t)k * 5 * m * n + (size_t)j * n + i;
                    snaps[b + 0 * (size_t)m * n] = CV[k].RHO[j][i];
                    snaps[b + 1 * (size_t)m * n] = CV[k].U[j][i];
                    snaps[b + 2 * (size_t)m * n] = CV[k].V[j][i];
                    snaps[b + 3 * (size_t)m * n] = CV[k].P[j][i];
                    snaps[b + 4 * (size_t)m * n] = CV[k].E[j][i];
                }
    if (nsnap_out)
        *nsnap_out = N_plot;
    if (info) {
        info[0] = config[5];
        info[1] = time_plot[last];
        info[2] = cpu_time[last];
        info[3] = t1 - t0;
    }
    for (k = 0; k < N_T; ++k) {
        free2(CV[k].RHO, m);
        free2(CV[k].U, m);
        free2(CV[k].V, m);
        free2(CV[k].P, m);
        free2(CV[k].E, m);
    }
    free(CV);
    free2(X, m + 1);
    free2(Y, m + 1);
    free(cpu_time);
    free(time_plot);
    return 0;
}

/*
 * 1D run (order 1 = Godunov, order 2 = GRP), Eulerian.  rho/u/p in, final
 * state out; E_out may be NULL.  info as in ref_run_2d.
 */
int ref_run_1d(int m, double *rho, double *u, double *p, double *E_out,
               const double *cfg, int ncfg, int order, double *info)
{
    int j, k;
    load_config(cfg, ncfg);
    config[0] = 1.0;
    config[8] = 0.0;
    const double gamma = config[6];
    int N_plot = 2;
    double time_plot[2] = {0.0, config[1]};
    int N = 2;
    struct cell_var_stru CV;
    memset(&CV, 0, sizeof(CV));
    CV.RHO = alloc2(N, m);
    CV.U = alloc2(N, m);
    CV.P = alloc2(N, m);
    CV.E = alloc2(N, m);
    for (j = 0; j < m; ++j) {
        CV.RHO[0][j] = rho[j];
        CV.U[0][j] = u[j];
        CV.P[0][j] = p[j];
        CV.E[0][j] = 0.5 * CV.U[0][j] * CV.U[0][j] + CV.P[0][j] / (gamma - 1.0) / CV.RHO[0][j];
    }
    double cpu_time[2] = {0.0, 0.0};
    double t0 = wall();
    if (order == 1)
        Godunov_solver_EUL_source(m, CV, cpu_time, &N_plot, time_plot);
    else
        GRP_solver_EUL_source(m, CV, cpu_time, &N_plot, time_plot);
    double t1 = wall();
    int last = N_plot - 1;
    for (j = 0; j < m; ++j) {
        rho[j] = CV.RHO[last][j];
        u[j] = CV.U[last][j];
        p[j] = CV.P[last][j];
        if (E_out)
            E_out[j] = CV.E[last][j];
    }
    if (info) {
        info[0] = config[5];
        info[1] = time_plot[last];
        info[2] = cpu_time[last];
        info[3] = t1 - t0;
    }
    free2(CV.RHO, N);
    free2(CV.U, N);
    free2(CV.P, N);
    free2(CV.E, N);
    (void)k;
    return 0;
}

/* Exact two-gamma Riemann solver (src/riemann_solver/riemann_solver_exact_Ben.c:30).
 * in: cnt x 8 = gammaL,gammaR,u_L,u_R,p_L,p_R,c_L,c_R; out: cnt x 5 = u*,p*,CRW0,CRW1,gap. */
void ref_riemann_exact(int cnt, const double *in, double eps, double tol, int N, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 8 * q;
        double us, ps;
        _Bool CRW[2];
        double gap = Riemann_solver_exact(&us, &ps, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], CRW, eps, tol, N);
        double *o = out + 5 * q;
        o[0] = us;
        o[1] = ps;
        o[2] = CRW[0];
        o[3] = CRW[1];
        o[4] = gap;
    }
}

/* Single-gamma exact solver (riemann_solver_exact_Ben.c:230).
 * in: cnt x 7 = gamma,u_L,u_R,p_L,p_R,c_L,c_R; out as above. */
void ref_riemann_exact_ben(int cnt, const double *in, double eps, double tol, int N, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 7 * q;
        double us, ps;
        _Bool CRW[2];
        double gap = Riemann_solver_exact_Ben(&us, &ps, a[0], a[1], a[2], a[3], a[4], a[5], a[6], CRW, eps, tol, N);
        double *o = out + 5 * q;
        o[0] = us;
        o[1] = ps;
        o[2] = CRW[0];
        o[3] = CRW[1];
        o[4] = gap;
    }
}

/* One side of an interface: RHO,U,V,P,d_rho,d_u,d_v,d_p,t_rho,t_u,t_v,t_p. */
static void fill_side(struct i_f_var *f, const double *s)
{
    f->RHO = s[0];
    f->U = s[1];
    f->V = s[2];
    f->P = s[3];
    f->d_rho = s[4];
    f->d_u = s[5];
    f->d_v = s[6];
    f->d_p = s[7];
    f->t_rho = s[8];
    f->t_u = s[9];
    f->t_v = s[10];
    f->t_p = s[11];
}

/* GRP_2D_flux (src/flux_calc/flux_solver.c:158) on cnt interfaces.
 * in: cnt x 27 = n_x,n_y,gamma, left side (12), right side (12).
 * out: cnt x 9 = F_rho,F_u,F_v,F_e,RHO_int,U_int,V_int,P_int,retval. */
void ref_grp2d_flux(int cnt, const double *in, double tau, double eps, double *out)
{
    config[4] = eps;
    config[8] = 0.0;
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 27 * q;
        struct i_f_var L, R;
        memset(&L, 0, sizeof(L));
        memset(&R, 0, sizeof(R));
        L.n_x = R.n_x = a[0];
        L.n_y = R.n_y = a[1];
        L.gamma = R.gamma = a[2];
        fill_side(&L, a + 3);
        fill_side(&R, a + 15);
        int rv = GRP_2D_flux(&L, &R, tau);
        double *o = out + 9 * q;
        o[0] = L.F_rho;
        o[1] = L.F_u;
        o[2] = L.F_v;
        o[3] = L.F_e;
        o[4] = L.RHO_int;
        o[5] = L.U_int;
        o[6] = L.V_int;
        o[7] = L.P_int;
        o[8] = rv;
    }
}

/* linear_GRP_solver_Edir_Q1D (linear_grp_solver_Edir_Q1D.c:38) in the normal frame.
 * in: cnt x 25 = gamma, left (12), right (12) with lambda_u = lambda_v = 0.
 * out: cnt x 14 = wave_speed[2], D[0..3], U[0..3], U_star[0],U_star[1],U_star[2],U_star[3]. */
void ref_q1d(int cnt, const double *in, double eps, double atc, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 25 * q;
        struct i_f_var L, R;
        memset(&L, 0, sizeof(L));
        memset(&R, 0, sizeof(R));
        L.gamma = R.gamma = a[0];
        fill_side(&L, a + 1);
        fill_side(&R, a + 13);
        double ws[2], D[6], U[6], S[6];
        linear_GRP_solver_Edir_Q1D(ws, D, U, S, &L, &R, eps, atc);
        double *o = out + 14 * q;
        o[0] = ws[0];
        o[1] = ws[1];
        for (int k = 0; k < 4; ++k) {
            o[2 + k] = D[k];
            o[6 + k] = U[k];
            o[10 + k] = S[k];
        }
    }
}

/*
 * 1D Lagrangian run (order 1 = Godunov_solver_LAG_source, 2 = GRP_solver_LAG_source),
 * set up as src/hydrocode_1D/hydrocode.c:196-247 does for "LAG": node
 * coordinates X[0][j] = j h, config[8] = 1.  rho/u/p in, final state out;
 * E_out and X_out (m+1 node coordinates) may be NULL.  info as in ref_run_1d.
 */
int ref_run_1d_lag(int m, double *rho, double *u, double *p, double *E_out, double *X_out,
                   const double *cfg, int ncfg, int order, double *info)
{
    int j;
    load_config(cfg, ncfg);
    config[0] = 1.0;
    config[8] = 1.0;
    const double gamma = config[6], h = config[10];
    int N_plot = 2;
    double time_plot[2] = {0.0, config[1]};
    int N = 2;
    struct cell_var_stru CV;
    memset(&CV, 0, sizeof(CV));
    CV.RHO = alloc2(N, m);
    CV.U = alloc2(N, m);
    CV.P = alloc2(N, m);
    CV.E = alloc2(N, m);
    double **X = alloc2(N, m + 1);
    for (j = 0; j <= m; ++j)
        X[0][j] = h * j;
    for (j = 0; j < m; ++j) {
        CV.RHO[0][j] = rho[j];
        CV.U[0][j] = u[j];
        CV.P[0][j] = p[j];
        CV.E[0][j] = 0.5 * CV.U[0][j] * CV.U[0][j] + CV.P[0][j] / (gamma - 1.0) / CV.RHO[0][j];
    }
    double cpu_time[2] = {0.0, 0.0};
    double t0 = wall();
    if (order == 1)
        Godunov_solver_LAG_source(m, CV, X, cpu_time, &N_plot, time_plot);
    else
        GRP_solver_LAG_source(m, CV, X, cpu_time, &N_plot, time_plot);
    double t1 = wall();
    int last = N_plot - 1;
    for (j = 0; j < m; ++j) {
        rho[j] = CV.RHO[last][j];
        u[j] = CV.U[last][j];
        p[j] = CV.P[last][j];
        if (E_out)
            E_out[j] = CV.E[last][j];
    }
    if (X_out)
        for (j = 0; j <= m; ++j)
            X_out[j] = X[last][j];
    if (info) {
        info[0] = config[5];
        info[1] = time_plot[last];
        info[2] = cpu_time[last];
        info[3] = t1 - t0;
    }
    free2(CV.RHO, N);
    free2(CV.U, N);
    free2(CV.P, N);
    free2(CV.E, N);
    free2(X, N);
    return 0;
}

/* linear_GRP_solver_LAG (linear_grp_solver_LAG.c:32) on cnt interfaces.
 * in: cnt x 13 = gamma, left rho,u,p,t_rho,t_u,t_p (material derivatives),
 * right the same.  out: cnt x 8 = D[0..3], U[0..3]. */
void ref_lag(int cnt, const double *in, double eps, double atc, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 13 * q;
        struct i_f_var L, R;
        memset(&L, 0, sizeof(L));
        memset(&R, 0, sizeof(R));
        L.gamma = R.gamma = a[0];
        L.RHO = a[1]; L.U = a[2]; L.P = a[3]; L.t_rho = a[4]; L.t_u = a[5]; L.t_p = a[6];
        R.RHO = a[7]; R.U = a[8]; R.P = a[9]; R.t_rho = a[10]; R.t_u = a[11]; R.t_p = a[12];
        double D[4], U[4];
        linear_GRP_solver_LAG(D, U, &L, &R, eps, atc);
        double *o = out + 8 * q;
        for (int k = 0; k < 4; ++k) {
            o[k] = D[k];
            o[4 + k] = U[k];
        }
    }
}

/* linear_GRP_solver_Edir_G2D (linear_grp_solver_Edir_G2D.c:48); layout as ref_q1d. */
void ref_g2d(int cnt, const double *in, double eps, double atc, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 25 * q;
        struct i_f_var L, R;
        memset(&L, 0, sizeof(L));
        memset(&R, 0, sizeof(R));
        L.gamma = R.gamma = a[0];
        fill_side(&L, a + 1);
        fill_side(&R, a + 13);
        double ws[2], D[6], U[6], S[6];
        linear_GRP_solver_Edir_G2D(ws, D, U, S, &L, &R, eps, atc);
        double *o = out + 14 * q;
        o[0] = ws[0];
        o[1] = ws[1];
        for (int k = 0; k < 4; ++k) {
            o[2 + k] = D[k];
            o[6 + k] = U[k];
            o[10 + k] = S[k];
        }
    }
}

/* linear_GRP_solver_Edir (linear_grp_solver_Edir.c:33), 1D.
 * in: cnt x 13 = gamma, left rho,u,p,d_rho,d_u,d_p, right same.
 * out: cnt x 6 = D[0..2], U[0..2]. */
void ref_grp1d(int cnt, const double *in, double eps, double atc, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 13 * q;
        struct i_f_var L, R;
        memset(&L, 0, sizeof(L));
        memset(&R, 0, sizeof(R));
        L.gamma = R.gamma = a[0];
        L.RHO = a[1]; L.U = a[2]; L.P = a[3]; L.d_rho = a[4]; L.d_u = a[5]; L.d_p = a[6];
        R.RHO = a[7]; R.U = a[8]; R.P = a[9]; R.d_rho = a[10]; R.d_u = a[11]; R.d_p = a[12];
        double D[3], U[3];
        linear_GRP_solver_Edir(D, U, &L, &R, eps, atc);
        double *o = out + 6 * q;
        for (int k = 0; k < 3; ++k) {
            o[k] = D[k];
            o[3 + k] = U[k];
        }
    }
}
