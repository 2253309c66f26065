/*
 * ref_mf_harness.c -- TEST INFRASTRUCTURE ONLY (the oracle's checker side).
 *
 * Flat entry point around the reference's GRP_2D_flux compiled, unmodified,
 * with MULTIFLUID_BASICS defined (oracle/Makefile, target
 * _ref/libhydro_ref_mf.so): the two-component interface flux
 * (src/flux_calc/flux_solver.c:158-237) over the two-component
 * linear_GRP_solver_Edir_Q1D (src/riemann_solver/linear_grp_solver_Edir_Q1D.c:55-62).
 * This file is compiled with the same macro, so struct i_f_var has the
 * two-component layout (src/include/var_struc.h:116-142).
 *
 * Row layout (in: 40 doubles, out: 19) as orc_grp2d_flux_mf in hydro_oracle.c.
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "var_struc.h"
#include "flux_calc.h"

double config[N_CONF];

static void fill(struct i_f_var *s, const double *a, const double *x)
{
    s->RHO = a[0]; s->U = a[1]; s->V = a[2]; s->P = a[3];
    s->d_rho = a[4]; s->d_u = a[5]; s->d_v = a[6]; s->d_p = a[7];
    s->t_rho = a[8]; s->t_u = a[9]; s->t_v = a[10]; s->t_p = a[11];
    s->Z_a = x[0]; s->d_z_a = x[1]; s->t_z_a = x[2];
    s->PHI = x[3]; s->d_phi = x[4]; s->t_phi = x[5];
}

void ref_grp2d_flux_mf(int cnt, const double *in, double tau, double eps, double gamma_a, double gamma_b,
                       int store_gamma, double *out)
{
    int k;
    for (k = 0; k < N_CONF; ++k)
        config[k] = INFINITY;
    config[4] = eps;
    config[6] = gamma_a;
    config[8] = 0.0;
    config[60] = store_gamma ? 1.0 : 0.0;
    config[106] = gamma_b;
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 40 * q;
        struct i_f_var L, R;
        memset(&L, 0, sizeof(L));
        memset(&R, 0, sizeof(R));
        L.n_x = R.n_x = a[0];
        L.n_y = R.n_y = a[1];
        L.gamma = a[2];
        fill(&L, a + 3, a + 15);
        R.gamma = a[21];
        fill(&R, a + 22, a + 34);
        int rv = GRP_2D_flux(&L, &R, tau);
        double *o = out + 19 * q;
        o[0] = L.F_rho; o[1] = L.F_u; o[2] = L.F_v; o[3] = L.F_e;
        o[4] = L.RHO_int; o[5] = L.U_int; o[6] = L.V_int; o[7] = L.P_int;
        o[8] = L.F_phi; o[9] = L.F_gamma; o[10] = L.F_e_a; o[11] = L.PHI; o[12] = L.Z_a;
        o[13] = L.U_qt_add_c; o[14] = L.V_qt_add_c; o[15] = L.U_qt_star; o[16] = L.V_qt_star;
        o[17] = L.P_star;
        o[18] = rv;
    }
}
