/*
 * hydro_oracle.c -- TEST INFRASTRUCTURE ONLY: the oracle.
 *
 * A CPU restatement, in plain C99 + OpenMP, of HydroCODE's Eulerian
 * Godunov/GRP finite-volume step for the 1D and 2D structured single-fluid
 * ideal-gas solver.  The CUDA path is tested against it (tests/, smoke() and
 * bench.py's cpu_baseline only) and never part of the product.
 *
 * Every floating-point expression keeps the reference's operand order, so the
 * restatement is bit-identical to the reference built from its own sources
 * (oracle/_ref, pinned by tests/test_oracle_pin.py and by the fixtures in
 * tests/golden/).  Function-level citations name the reference file:line each
 * routine follows.
 *
 * Deliberate difference: when the star-state /
 * time-derivative check of an interface fails, the reference returns before
 * writing that interface's flux and leaves whatever the previous interface on
 * the same OpenMP thread produced; here the flux is still assembled from the
 * (rejected) solution so the value is deterministic.  The run stops after that
 * step in both.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "hydro_oracle.h"

/* ------------------------------------------------------------------------- */
/* small helpers                                                              */
/* ------------------------------------------------------------------------- */

typedef struct {
    double rho, u, v, p;     /* primitive values at the interface (t_n)   */
    double drho, du, dv, dp; /* normal derivatives                        */
    double trho, tu, tv, tp; /* tangential derivatives                    */
} orc_side;

/* Passive scalars of the two-component build (MULTIFLUID_BASICS): volume
 * fraction z and mass fraction phi of one side, each with its normal and
 * tangential derivative (struct i_f_var Z_a/d_z_a/t_z_a, PHI/d_phi/t_phi,
 * src/include/var_struc.h:129-130). */
typedef struct {
    double z, dz, tz;
    double phi, dphi, tphi;
} orc_scal;

/* Ghost cell of one boundary row/column, same fields as the reference's
 * struct b_f_var (src/include/var_struc.h:146-151). */
typedef struct {
    double rho, p, u, v;     /* ghost values                 */
    double srho, sp, su, sv; /* x-derivatives of the ghost   */
    double trho, tp, tu, tv; /* y-derivatives of the ghost   */
} orc_ghost;

static double wall_clock(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return (double)clock() / CLOCKS_PER_SEC;
#endif
}

/* minmod of two slopes: src/include/tools.h:44-55 */
static double orc_minmod2(double sL, double sR)
{
    if (sL * sR <= 0.0)
        return 0.0;
    if (sR > 0.0 && sR < sL)
        return sR;
    if (sR <= 0.0 && sR > sL)
        return sR;
    return sL;
}

/* minmod of three slopes: src/include/tools.h:60-73 */
static double orc_minmod3(double sL, double sR, double sm)
{
    if (sL * sm <= 0.0 || sR * sm <= 0.0)
        return 0.0;
    if (sm > 0.0 && sm < sL && sm < sR)
        return sm;
    if (sm <= 0.0 && sm > sL && sm > sR)
        return sm;
    if (sR > 0.0 && sR < sL)
        return sR;
    if (sR <= 0.0 && sR > sL)
        return sR;
    return sL;
}

/* ------------------------------------------------------------------------- */
/* exact Riemann solver                                                       */
/* ------------------------------------------------------------------------- */

/* Velocity reached on the left (1-wave) curve through (uL,pL) at pressure pp:
 * shock branch for pp > pL, rarefaction branch otherwise.
 * riemann_solver_exact_Ben.c:50-62 and :96-108. */
static double orc_curve_left(double pp, double uL, double pL, double cL, double g, double mu, double nu)
{
    double w;
    if (pp > pL) {
        double dp = pp - pL;
        w = sqrt(1.0 + nu * dp / pL);
        w = dp * cL / g / pL / w;
        return uL - w;
    }
    w = pow(pp / pL, mu) - 1.0;
    w = 2.0 * cL * w / (g - 1.0);
    return uL - w;
}

/* Same for the right (3-wave) curve: riemann_solver_exact_Ben.c:64-76, :109-121. */
static double orc_curve_right(double pp, double uR, double pR, double cR, double g, double mu, double nu)
{
    double w;
    if (pp > pR) {
        double dp = pp - pR;
        w = sqrt(1.0 + nu * dp / pR);
        w = dp * cR / g / pR / w;
        return uR + w;
    }
    w = pow(pp / pR, mu) - 1.0;
    w = 2.0 * cR * w / (g - 1.0);
    return uR + w;
}

/*
 * Exact two-gamma Riemann solver: wave classification, a starting pressure at
 * half the intersection of the two tangent lines, then Newton on the velocity
 * gap with an absolute tolerance.  riemann_solver_exact_Ben.c:30-211
 * (Riemann_solver_exact; the single-gamma Riemann_solver_exact_Ben at :230 is
 * the same arithmetic with gL == gR).
 */
static double orc_exact(double gL, double gR, double uL, double uR, double pL, double pR,
                        double cL, double cR, double eps, double tol, int N,
                        double *u_star, double *p_star, int crw[2], int *iters)
{
    const double muL = (gL - 1.0) / (2.0 * gL), nuL = (gL + 1.0) / (2.0 * gL);
    const double muR = (gR - 1.0) / (2.0 * gR), nuR = (gR + 1.0) / (2.0 * gR);
    double k1, k3, p_int, p_new, vL, vR, gap;
    int it = 0;

    /* wave types, :48-84 */
    double uLR = orc_curve_left(pR, uL, pL, cL, gL, muL, nuL);
    double uRL = orc_curve_right(pL, uR, pR, cR, gR, muR, nuR);
    crw[1] = (uLR > uR + eps) ? 0 : 1;
    crw[0] = (uRL > uL - eps) ? 1 : 0;

    /* starting pressure, :86-93 */
    k1 = -cL / pL / gL;
    k3 = cR / pR / gR;
    p_int = (k1 * pL - k3 * pR - uL + uR) / (k1 - k3);
    if (p_int < 0)
        p_int = (pL < pR) ? pL : pR;
    p_int = 0.5 * p_int;

    vL = orc_curve_left(p_int, uL, pL, cL, gL, muL, nuL);
    vR = orc_curve_right(p_int, uR, pR, cR, gR, muR, nuR);
    gap = fabs(vL - vR);

    /* trivial case, :124-130 */
    if (fabs(uL - uR) < tol && fabs(pL - pR) < tol) {
        *p_star = 0.5 * (pL + pR);
        *u_star = 0.5 * (uL + uR);
        if (iters)
            *iters = 0;
        return fabs(uL - uR);
    }

    /* Newton, :133-203 */
    while ((gap > tol) && (it != N)) {
        double t1, t2, t3;
        if (p_int > pL) {
            double dp = p_int - pL;
            t1 = 1.0 / sqrt(1.0 + nuL * dp / pL);
            t2 = cL / gL / pL;
            t3 = 0.5 * t2 * nuL / pL;
            k1 = t3 * dp * pow(t1, 3.0) - t2 * t1;
        } else {
            t2 = cL / gL / pL;
            t1 = 1.0 / pow(p_int / pL, nuL);
            k1 = -t1 * t2;
        }
        if (p_int > pR) {
            double dp = p_int - pR;
            t1 = 1.0 / sqrt(1.0 + nuR * dp / pR);
            t2 = cR / gR / pR;
            t3 = 0.5 * t2 * nuR / pR;
            k3 = t2 * t1 - t3 * dp * pow(t1, 3.0);
        } else {
            t2 = cR / gR / pR;
            t1 = 1.0 / pow(p_int / pR, nuR);
            k3 = t1 * t2;
        }
        p_new = p_int + (vR - vL) / (k1 - k3);
        if (p_new < 0.0)
            p_int = 0.5 * p_int;
        else
            p_int = p_new;
        ++it;
        vL = orc_curve_left(p_int, uL, pL, cL, gL, muL, nuL);
        vR = orc_curve_right(p_int, uR, pR, cR, gR, muR, nuR);
        gap = fabs(vL - vR);
    }
    *u_star = k1 * (vR - vL) / (k1 - k3) + vL; /* :205 */
    *p_star = p_int;
    if (iters)
        *iters = it;
    return gap;
}

/* ------------------------------------------------------------------------- */
/* quasi-1D direct Eulerian GRP solver (2D path)                              */
/* ------------------------------------------------------------------------- */

/* Star region and wave speeds of one interface, as both direct Eulerian GRP
 * solvers compute them (Q1D :93-134, G2D :109-153). */
typedef struct {
    double c_L, c_R, u_star, p_star, rho_star_L, rho_star_R, c_star_L, c_star_R, speed_L, speed_R;
    int CRW[2];
} orc_star;

/*
 * linear_GRP_solver_Edir_Q1D, src/riemann_solver/linear_grp_solver_Edir_Q1D.c:38-554,
 * single-fluid (the volume/mass-fraction slots are constants and are dropped),
 * frame velocity lambda = 0 as set by GRP_2D_flux.
 * Outputs: ws = wave speeds, D = (rho,u,v,p)_t, U = (rho,u,v,p) on the t-axis,
 * S = (rho*_L, u*, rho*_R, p*).
 */
static void orc_g2d_nonacoustic(double gL, double gR, const orc_side *Ls, const orc_side *Rs, double eps,
                                const orc_star *st, double D[4], double U[4]);

/* The scalars' t-axis values UX = (z, phi) and derivatives DX when taken from
 * one side's states as they stand (the states left/right of all waves):
 * linear_grp_solver_Edir_Q1D.c:147-154, 162-169, 264-271, 279-286. */
static void orc_scal_side(const orc_scal *X, double u, double v, double lu, double lv, double DX[2], double UX[2])
{
    UX[0] = X->z;
    UX[1] = X->phi;
    DX[0] = -(u - lu) * X->dz - (v - lv) * X->tz;
    DX[1] = -(u - lu) * X->dphi - (v - lv) * X->tphi;
}

/* Scalars: XL/XR the two sides' (z, phi) with derivatives, DX/UX their outputs;
 * all NULL for the single-fluid build (the reference's constant slots). */
static void orc_q1d_solve_x(double gL, double gR, const orc_side *Ls, const orc_side *Rs,
                            const orc_scal *XL, const orc_scal *XR,
                            double eps, double atc, double ws[2], double D[4], double U[4], double S[4],
                            double DX[2], double UX[2], int *newton_iters, int g2d);

static void orc_q1d_solve(double gL, double gR, const orc_side *Ls, const orc_side *Rs,
                          double eps, double atc, double ws[2], double D[4], double U[4], double S[4],
                          int *newton_iters, int g2d)
{
    orc_q1d_solve_x(gL, gR, Ls, Rs, NULL, NULL, eps, atc, ws, D, U, S, NULL, NULL, newton_iters, g2d);
}

static void orc_q1d_solve_x(double gL, double gR, const orc_side *Ls, const orc_side *Rs,
                            const orc_scal *XL, const orc_scal *XR,
                            double eps, double atc, double ws[2], double D[4], double U[4], double S[4],
                            double DX[2], double UX[2], int *newton_iters, int g2d)
{
    const int sc = XL != NULL;
    const double lu = 0.0, lv = 0.0;
    const double rho_L = Ls->rho, rho_R = Rs->rho;
    const double d_rho_L = Ls->drho, d_rho_R = Rs->drho;
    const double t_rho_L = Ls->trho, t_rho_R = Rs->trho;
    const double u_L = Ls->u, u_R = Rs->u;
    const double d_u_L = Ls->du, d_u_R = Rs->du;
    const double t_u_L = Ls->tu, t_u_R = Rs->tu;
    const double v_L = Ls->v, v_R = Rs->v;
    const double d_v_L = Ls->dv, d_v_R = Rs->dv;
    const double t_v_L = Ls->tv, t_v_R = Rs->tv;
    const double p_L = Ls->p, p_R = Rs->p;
    const double d_p_L = Ls->dp, d_p_R = Rs->dp;
    const double t_p_L = Ls->tp, t_p_R = Rs->tp;

    int CRW[2] = {0, 0};
    double C = 0.0, c_frac;
    double TdS, d_Psi, d_Phi, VAR;
    double D_rho, D_u, D_v, D_p, T_rho, T_u, T_v, T_p;
    double u_star, p_star, rho_star_L, rho_star_R, c_star_L, c_star_R;
    double H1, H2, H3, a_L, b_L, d_L, a_R, b_R, d_R, detA, L_u, L_p, L_rho;
    double u_t_mat, p_t_mat, SmUs, SmUL, SmUR, rho_x, f, speed_L, speed_R;
    const double zetaL = (gL - 1.0) / (gL + 1.0);
    const double zetaR = (gR - 1.0) / (gR + 1.0);

    if (newton_iters)
        *newton_iters = -1;
    double c_L = sqrt(gL * p_L / rho_L);
    double c_R = sqrt(gR * p_R / rho_R);
    /* the genuinely-2D solver also counts the tangential velocity jump
       (linear_grp_solver_Edir_G2D.c:112) */
    double dist = g2d ? sqrt((rho_L - rho_R) * (rho_L - rho_R) + (u_L - u_R) * (u_L - u_R) +
                             (v_L - v_R) * (v_L - v_R) + (p_L - p_R) * (p_L - p_R))
                      : sqrt((rho_L - rho_R) * (rho_L - rho_R) + (u_L - u_R) * (u_L - u_R) + (p_L - p_R) * (p_L - p_R));

    if (dist < atc && atc < 2 * eps) { /* :96-106 */
        u_star = 0.5 * (u_R + u_L);
        p_star = 0.5 * (p_R + p_L);
        rho_star_L = rho_L;
        c_star_L = c_L;
        speed_L = u_star - c_star_L;
        rho_star_R = rho_R;
        c_star_R = c_R;
        speed_R = u_star + c_star_R;
    } else { /* :107-134 */
        int it;
        orc_exact(gL, gR, u_L, u_R, p_L, p_R, c_L, c_R, eps, eps, 500, &u_star, &p_star, CRW, &it);
        if (newton_iters)
            *newton_iters = it;
        if (CRW[0]) {
            rho_star_L = rho_L * pow(p_star / p_L, 1.0 / gL);
            c_star_L = c_L * pow(p_star / p_L, 0.5 * (gL - 1.0) / gL);
            speed_L = u_L - c_L;
        } else {
            rho_star_L = rho_L * (p_star + zetaL * p_L) / (p_L + zetaL * p_star);
            c_star_L = sqrt(gL * p_star / rho_star_L);
            speed_L = u_L - c_L * sqrt(0.5 * ((gL + 1.0) * (p_star / p_L) + (gL - 1.0)) / gL);
        }
        if (CRW[1]) {
            rho_star_R = rho_R * pow(p_star / p_R, 1.0 / gR);
            c_star_R = c_R * pow(p_star / p_R, 0.5 * (gR - 1.0) / gR);
            speed_R = u_R + c_R;
        } else {
            rho_star_R = rho_R * (p_star + zetaR * p_R) / (p_R + zetaR * p_star);
            c_star_R = sqrt(gR * p_star / rho_star_R);
            speed_R = u_R + c_R * sqrt(0.5 * ((gR + 1.0) * (p_star / p_R) + (gR - 1.0)) / gR);
        }
    }
    ws[0] = speed_L;
    ws[1] = speed_R;
    S[0] = rho_star_L;
    S[1] = u_star;
    S[2] = rho_star_R;
    S[3] = p_star;

    if (dist < atc) { /* acoustic case, :139-254 */
        if (speed_L > lu) {
            U[0] = rho_L; U[1] = u_L; U[2] = v_L; U[3] = p_L;
            D[0] = -(u_L - lu) * d_rho_L - (v_L - lv) * t_rho_L - rho_L * (d_u_L + t_v_L);
            D[1] = -(u_L - lu) * d_u_L - (v_L - lv) * t_u_L - d_p_L / rho_L;
            D[2] = -(u_L - lu) * d_v_L - (v_L - lv) * t_v_L - t_p_L / rho_L;
            D[3] = -(u_L - lu) * d_p_L - (v_L - lv) * t_p_L - rho_L * c_L * c_L * (d_u_L + t_v_L);
            if (sc)
                orc_scal_side(XL, u_L, v_L, lu, lv, DX, UX);
        } else if (speed_R < lu) {
            U[0] = rho_R; U[1] = u_R; U[2] = v_R; U[3] = p_R;
            D[0] = -(u_R - lu) * d_rho_R - (v_R - lv) * t_rho_R - rho_R * (d_u_R + t_v_R);
            D[1] = -(u_R - lu) * d_u_R - (v_R - lv) * t_u_R - d_p_R / rho_R;
            D[2] = -(u_R - lu) * d_v_R - (v_R - lv) * t_v_R - t_p_R / rho_R;
            D[3] = -(u_R - lu) * d_p_R - (v_R - lv) * t_p_R - rho_R * c_R * c_R * (d_u_R + t_v_R);
            if (sc)
                orc_scal_side(XR, u_R, v_R, lu, lv, DX, UX);
        } else {
            if (CRW[0] && ((u_star - c_star_L) > lu)) {
                U[1] = zetaL * (u_L + 2.0 * (c_L + lu) / (gL - 1.0));
                C = U[1] - lu;
                U[3] = pow(C / c_L, 2.0 * gL / (gL - 1.0)) * p_L;
                U[0] = gL * U[3] / C / C;
                U[2] = v_L;
            } else if (CRW[1] && ((u_star + c_star_R) < lu)) {
                U[1] = zetaR * (u_R - 2.0 * (c_R - lu) / (gR - 1.0));
                C = lu - U[1];
                U[3] = pow(C / c_R, 2.0 * gR / (gR - 1.0)) * p_R;
                U[0] = gR * U[3] / C / C;
                U[2] = v_R;
            } else if (u_star > lu) {
                U[0] = rho_star_L; U[1] = u_star; U[2] = v_L; U[3] = p_star;
                C = c_star_L;
            } else {
                U[0] = rho_star_R; U[1] = u_star; U[2] = v_R; U[3] = p_star;
                C = c_star_R;
            }
            D_p = 0.5 * ((d_u_L * (U[0] * C) + d_p_L) - (d_u_R * (U[0] * C) - d_p_R));
            T_p = 0.5 * ((t_u_L * (U[0] * C) + t_p_L) - (t_u_R * (U[0] * C) - t_p_R));
            D_u = 0.5 * (d_u_L + d_p_L / (U[0] * C) + d_u_R - d_p_R / (U[0] * C));
            T_u = 0.5 * (t_u_L + t_p_L / (U[0] * C) + t_u_R - t_p_R / (U[0] * C));
            if (u_star > lu) {
                D_v = d_v_L;
                T_v = t_v_L;
                D_rho = d_rho_L - d_p_L / (C * C) + D_p / (C * C);
                T_rho = t_rho_L - t_p_L / (C * C) + T_p / (C * C);
            } else {
                D_v = d_v_R;
                T_v = t_v_R;
                D_rho = d_rho_R - d_p_R / (C * C) + D_p / (C * C);
                T_rho = t_rho_R - t_p_R / (C * C) + T_p / (C * C);
            }
            D[0] = -(U[1] - lu) * D_rho - (U[2] - lv) * T_rho - U[0] * (D_u + T_v);
            D[1] = -(U[1] - lu) * D_u - (U[2] - lv) * T_u - D_p / U[0];
            D[2] = -(U[1] - lu) * D_v - (U[2] - lv) * T_v - T_p / U[0];
            D[3] = -(U[1] - lu) * D_p - (U[2] - lv) * T_p - U[0] * C * C * (D_u + T_v);
            if (sc) { /* :180-210 (the side of the t-axis state), :220-245 */
                const orc_scal *Xu = (CRW[0] && ((u_star - c_star_L) > lu)) ? XL
                                   : (CRW[1] && ((u_star + c_star_R) < lu)) ? XR
                                   : (u_star > lu) ? XL : XR;
                const orc_scal *Xd = (u_star > lu) ? XL : XR;
                UX[0] = Xu->z;
                UX[1] = Xu->phi;
                DX[0] = -(U[1] - lu) * Xd->dz - (U[2] - lv) * Xd->tz;
                DX[1] = -(U[1] - lu) * Xd->dphi - (U[2] - lv) * Xd->tphi;
            }
        }
        return;
    }

    if (g2d) { /* the acoustic case above is the same in both solvers (G2D :156-271) */
        orc_star st = {c_L, c_R, u_star, p_star, rho_star_L, rho_star_R, c_star_L, c_star_R,
                       speed_L, speed_R, {CRW[0], CRW[1]}};
        orc_g2d_nonacoustic(gL, gR, Ls, Rs, eps, &st, D, U);
        return;
    }

    /* non-acoustic case, :256-547 */
    if (speed_L > lu) {
        U[0] = rho_L; U[1] = u_L; U[2] = v_L; U[3] = p_L;
        D[0] = -(u_L - lu) * d_rho_L - (v_L - lv) * t_rho_L - rho_L * (d_u_L + t_v_L);
        D[1] = -(u_L - lu) * d_u_L - (v_L - lv) * t_u_L - d_p_L / rho_L;
        D[2] = -(u_L - lu) * d_v_L - (v_L - lv) * t_v_L - t_p_L / rho_L;
        D[3] = -(u_L - lu) * d_p_L - (v_L - lv) * t_p_L - rho_L * c_L * c_L * (d_u_L + t_v_L);
        if (sc)
            orc_scal_side(XL, u_L, v_L, lu, lv, DX, UX);
        return;
    }
    if (speed_R < lu) {
        U[0] = rho_R; U[1] = u_R; U[2] = v_R; U[3] = p_R;
        D[0] = -(u_R - lu) * d_rho_R - (v_R - lv) * t_rho_R - rho_R * (d_u_R + t_v_R);
        D[1] = -(u_R - lu) * d_u_R - (v_R - lv) * t_u_R - d_p_R / rho_R;
        D[2] = -(u_R - lu) * d_v_R - (v_R - lv) * t_v_R - t_p_R / rho_R;
        D[3] = -(u_R - lu) * d_p_R - (v_R - lv) * t_p_R - rho_R * c_R * c_R * (d_u_R + t_v_R);
        if (sc)
            orc_scal_side(XR, u_R, v_R, lu, lv, DX, UX);
        return;
    }
    if (CRW[0] && ((u_star - c_star_L) > lu)) { /* sonic point in the 1-rarefaction, :290-314 */
        U[1] = zetaL * (u_L + 2.0 * (c_L + lu) / (gL - 1.0));
        C = U[1] - lu;
        U[3] = pow(C / c_L, 2.0 * gL / (gL - 1.0)) * p_L;
        U[0] = gL * U[3] / C / C;
        U[2] = v_L;
        c_frac = C / c_L;
        TdS = (d_p_L - d_rho_L * c_L * c_L) / (gL - 1.0) / rho_L;
        d_Psi = d_u_L + (gL * d_p_L / c_L - c_L * d_rho_L) / (gL - 1.0) / rho_L;
        D[1] = ((1.0 + zetaL) * pow(c_frac, 0.5 / zetaL) + zetaL * pow(c_frac, (1.0 + zetaL) / zetaL));
        D[1] = D[1] / (1.0 + 2.0 * zetaL) * TdS;
        D[1] = D[1] - c_L * pow(c_frac, 0.5 / zetaL) * d_Psi;
        D[3] = U[0] * (U[1] - lu) * D[1];
        D[0] = U[0] * (U[1] - lu) * pow(c_frac, (1.0 + zetaL) / zetaL) * TdS * (gL - 1.0);
        D[0] = (D[0] + D[3]) / C / C;
        D[2] = -(U[1] - lu) * d_v_L * U[0] / rho_L;
        if (sc) {
            UX[0] = XL->z;
            UX[1] = XL->phi;
            DX[0] = -(U[1] - lu) * XL->dz * U[0] / rho_L;
            DX[1] = -(U[1] - lu) * XL->dphi * U[0] / rho_L;
        }
    } else if (CRW[1] && ((u_star + c_star_R) < lu)) { /* sonic point in the 3-rarefaction, :315-339 */
        U[1] = zetaR * (u_R - 2.0 * (c_R - lu) / (gR - 1.0));
        C = lu - U[1];
        U[3] = pow(C / c_R, 2.0 * gR / (gR - 1.0)) * p_R;
        U[0] = gR * U[3] / C / C;
        U[2] = v_R;
        c_frac = C / c_R;
        TdS = (d_p_R - d_rho_R * c_R * c_R) / (gR - 1.0) / rho_R;
        d_Phi = d_u_R - (gR * d_p_R / c_R - c_R * d_rho_R) / (gR - 1.0) / rho_R;
        D[1] = ((1.0 + zetaR) * pow(c_frac, 0.5 / zetaR) + zetaR * pow(c_frac, (1.0 + zetaR) / zetaR));
        D[1] = D[1] / (1.0 + 2.0 * zetaR) * TdS;
        D[1] = D[1] + c_R * pow(c_frac, 0.5 / zetaR) * d_Phi;
        D[3] = U[0] * (U[1] - lu) * D[1];
        D[0] = U[0] * (U[1] - lu) * pow(c_frac, (1.0 + zetaR) / zetaR) * TdS * (gR - 1.0);
        D[0] = (D[0] + D[3]) / C / C;
        D[2] = -(U[1] - lu) * d_v_R * U[0] / rho_R;
        if (sc) {
            UX[0] = XR->z;
            UX[1] = XR->phi;
            DX[0] = -(U[1] - lu) * XR->dz * U[0] / rho_R;
            DX[1] = -(U[1] - lu) * XR->dphi * U[0] / rho_R;
        }
    } else { /* non-sonic case, :340-523 */
        if (u_star < lu) {
            U[0] = rho_star_R; U[1] = u_star; U[2] = v_R; U[3] = p_star;
            C = c_star_R;
        } else {
            U[0] = rho_star_L; U[1] = u_star; U[2] = v_L; U[3] = p_star;
            C = c_star_L;
        }
        if (sc) {
            const orc_scal *Xu = (u_star < lu) ? XR : XL;
            UX[0] = Xu->z;
            UX[1] = Xu->phi;
        }
        if (CRW[0]) {
            a_L = 1.0;
            b_L = 1.0 / rho_star_L / c_star_L;
            c_frac = c_star_L / c_L;
            TdS = (d_p_L - d_rho_L * c_L * c_L) / (gL - 1.0) / rho_L;
            d_Psi = d_u_L + (gL * d_p_L / c_L - c_L * d_rho_L) / (gL - 1.0) / rho_L;
            d_L = ((1.0 + zetaL) * pow(c_frac, 0.5 / zetaL) + zetaL * pow(c_frac, (1.0 + zetaL) / zetaL));
            d_L = d_L / (1.0 + 2.0 * zetaL) * TdS;
            d_L = d_L - c_L * pow(c_frac, 0.5 / zetaL) * d_Psi;
        } else {
            SmUs = -sqrt(0.5 * ((gL + 1.0) * p_L + (gL - 1.0) * p_star) / rho_star_L);
            SmUL = -sqrt(0.5 * ((gL + 1.0) * p_star + (gL - 1.0) * p_L) / rho_L);
            VAR = sqrt((1 - zetaL) / (rho_L * (p_star + zetaL * p_L)));
            H1 = 0.5 * VAR * (p_star + (1.0 + 2.0 * zetaL) * p_L) / (p_star + zetaL * p_L);
            H2 = -0.5 * VAR * ((2.0 + zetaL) * p_star + zetaL * p_L) / (p_star + zetaL * p_L);
            H3 = -0.5 * VAR * (p_star - p_L) / rho_L;
            L_p = -1.0 / rho_L - SmUL * H2;
            L_u = SmUL + rho_L * (c_L * c_L * H2 + H3);
            L_rho = -SmUL * H3;
            a_L = 1.0 - rho_star_L * SmUs * H1;
            b_L = -SmUs / (rho_star_L * c_star_L * c_star_L) + H1;
            d_L = L_rho * d_rho_L + L_u * d_u_L + L_p * d_p_L;
        }
        if (CRW[1]) {
            a_R = 1.0;
            b_R = -1.0 / rho_star_R / c_star_R;
            c_frac = c_star_R / c_R;
            TdS = (d_p_R - d_rho_R * c_R * c_R) / (gR - 1.0) / rho_R;
            d_Phi = d_u_R - (gR * d_p_R / c_R - c_R * d_rho_R) / (gR - 1.0) / rho_R;
            d_R = ((1.0 + zetaR) * pow(c_frac, 0.5 / zetaR) + zetaR * pow(c_frac, (1.0 + zetaR) / zetaR));
            d_R = d_R / (1.0 + 2.0 * zetaR) * TdS;
            d_R = d_R + c_R * pow(c_frac, 0.5 / zetaR) * d_Phi;
        } else {
            SmUs = sqrt(0.5 * ((gR + 1.0) * p_R + (gR - 1.0) * p_star) / rho_star_R);
            SmUR = sqrt(0.5 * ((gR + 1.0) * p_star + (gR - 1.0) * p_R) / rho_R);
            VAR = sqrt((1.0 - zetaR) / (rho_R * (p_star + zetaR * p_R)));
            H1 = 0.5 * VAR * (p_star + (1 + 2.0 * zetaR) * p_R) / (p_star + zetaR * p_R);
            H2 = -0.5 * VAR * ((2.0 + zetaR) * p_star + zetaR * p_R) / (p_star + zetaR * p_R);
            H3 = -0.5 * VAR * (p_star - p_R) / rho_R;
            L_p = -1.0 / rho_R + SmUR * H2;
            L_u = SmUR - rho_R * (c_R * c_R * H2 + H3);
            L_rho = SmUR * H3;
            a_R = 1.0 + rho_star_R * SmUs * H1;
            b_R = -(SmUs / (rho_star_R * c_star_R * c_star_R) + H1);
            d_R = L_rho * d_rho_R + L_u * d_u_R + L_p * d_p_R;
        }
        detA = a_L * b_R - b_L * a_R;
        u_t_mat = (b_R * d_L - b_L * d_R) / detA;
        p_t_mat = (a_L * d_R - a_R * d_L) / detA;
        D[1] = u_t_mat + (u_star - lu) / U[0] / C / C * p_t_mat;
        D[3] = p_t_mat + (u_star - lu) * U[0] * u_t_mat;
        if (u_star < lu) {
            if (CRW[1]) {
                D[0] = rho_star_R * (u_star - lu) * pow(c_star_R / c_R, (1.0 + zetaR) / zetaR) * (d_p_R - d_rho_R * c_R * c_R) / rho_R;
                D[0] = (D[0] + D[3]) / c_star_R / c_star_R;
                D[2] = -U[1] * d_v_R * U[0] / rho_R;
                D[2] = D[2] + lu * d_v_R;
                if (sc) {
                    DX[0] = -U[1] * XR->dz * U[0] / rho_R;
                    DX[0] = DX[0] + lu * XR->dz;
                    DX[1] = -U[1] * XR->dphi * U[0] / rho_R;
                    DX[1] = DX[1] + lu * XR->dphi;
                }
            } else {
                SmUs = sqrt(0.5 * ((gR + 1.0) * p_R + (gR - 1.0) * p_star) / rho_star_R);
                SmUR = sqrt(0.5 * ((gR + 1.0) * p_star + (gR - 1.0) * p_R) / rho_R);
                VAR = p_R + zetaR * p_star;
                H1 = rho_R * p_R * (1.0 - zetaR * zetaR) / VAR / VAR;
                H2 = rho_R * p_star * (zetaR * zetaR - 1.0) / VAR / VAR;
                H3 = (p_star + zetaR * p_R) / VAR;
                L_rho = SmUR * H3 * d_rho_R;
                L_u = -rho_R * (H2 * c_R * c_R + H3) * d_u_R;
                L_p = H2 * SmUR * d_p_R;
                D[0] = ((u_star + SmUs) / c_star_R / c_star_R - u_star * H1) * p_t_mat + rho_star_R * u_star * SmUs * H1 * u_t_mat;
                D[0] = (D[0] - u_star * (L_p + L_rho + L_u)) / SmUs;
                f = SmUR * (H2 * d_p_R + H3 * d_rho_R) - rho_R * (H2 * c_R * c_R + H3) * d_u_R;
                rho_x = (f + H1 * (p_t_mat - rho_star_R * SmUs * u_t_mat) - D[0]) / (SmUR + u_R);
                D[0] = D[0] + lu * rho_x;
                D[2] = -U[1] * SmUR * d_v_R / SmUs;
                D[2] = D[2] + lu * d_v_R;
                if (sc) {
                    DX[0] = -U[1] * SmUR * XR->dz / SmUs;
                    DX[0] = DX[0] + lu * XR->dz;
                    DX[1] = -U[1] * SmUR * XR->dphi / SmUs;
                    DX[1] = DX[1] + lu * XR->dphi;
                }
            }
        } else {
            if (CRW[0]) {
                D[0] = rho_star_L * (u_star - lu) * pow(c_star_L / c_L, (1.0 + zetaL) / zetaL) * (d_p_L - d_rho_L * c_L * c_L) / rho_L;
                D[0] = (D[0] + D[3]) / c_star_L / c_star_L;
                D[2] = -U[1] * d_v_L * U[0] / rho_L;
                D[2] = D[2] + lu * d_v_L;
                if (sc) {
                    DX[0] = -U[1] * XL->dz * U[0] / rho_L;
                    DX[0] = DX[0] + lu * XL->dz;
                    DX[1] = -U[1] * XL->dphi * U[0] / rho_L;
                    DX[1] = DX[1] + lu * XL->dphi;
                }
            } else {
                SmUs = -sqrt(0.5 * ((gL + 1.0) * p_L + (gL - 1.0) * p_star) / rho_star_L);
                SmUL = -sqrt(0.5 * ((gL + 1.0) * p_star + (gL - 1.0) * p_L) / rho_L);
                VAR = p_L + zetaL * p_star;
                H1 = rho_L * p_L * (1.0 - zetaL * zetaL) / VAR / VAR;
                H2 = rho_L * p_star * (zetaL * zetaL - 1.0) / VAR / VAR;
                H3 = (p_star + zetaL * p_L) / VAR;
                L_rho = SmUL * H3 * d_rho_L;
                L_u = -rho_L * (H2 * c_L * c_L + H3) * d_u_L;
                L_p = H2 * SmUL * d_p_L;
                D[0] = ((u_star + SmUs) / c_star_L / c_star_L - H1 * u_star) * p_t_mat + rho_star_L * u_star * SmUs * H1 * u_t_mat;
                D[0] = (D[0] - u_star * (L_p + L_rho + L_u)) / SmUs;
                f = SmUL * (H2 * d_p_L + H3 * d_rho_L) - rho_L * (H2 * c_L * c_L + H3) * d_u_L;
                rho_x = (f + H1 * (p_t_mat - rho_star_L * SmUs * u_t_mat) - D[0]) / (SmUL + u_L);
                D[0] = D[0] + lu * rho_x;
                D[2] = -U[1] * SmUL * d_v_L / SmUs;
                D[2] = D[2] + lu * d_v_L;
                if (sc) {
                    DX[0] = -U[1] * SmUL * XL->dz / SmUs;
                    DX[0] = DX[0] + lu * XL->dz;
                    DX[1] = -U[1] * SmUL * XL->dphi / SmUs;
                    DX[1] = DX[1] + lu * XL->dphi;
                }
            }
        }
    }
    /* transversal terms, :524-545 */
    T_p = 0.5 * ((t_u_L * (U[0] * C) + t_p_L) - (t_u_R * (U[0] * C) - t_p_R));
    T_u = 0.5 * (t_u_L + t_p_L / (U[0] * C) + t_u_R - t_p_R / (U[0] * C));
    if (u_star > lu) {
        T_rho = t_rho_L - t_p_L / (C * C) + T_p / (C * C);
        D[0] = D[0] - (U[2] - lv) * T_rho - U[0] * t_v_L;
        D[1] = D[1] - (U[2] - lv) * T_u;
        D[2] = D[2] - (U[2] - lv) * t_v_L - T_p / U[0];
        D[3] = D[3] - (U[2] - lv) * T_p - U[0] * C * C * t_v_L;
        if (sc) {
            DX[0] = DX[0] - (U[2] - lv) * XL->tz;
            DX[1] = DX[1] - (U[2] - lv) * XL->tphi;
        }
    } else {
        T_rho = t_rho_R - t_p_R / (C * C) + T_p / (C * C);
        D[0] = D[0] - (U[2] - lv) * T_rho - U[0] * t_v_R;
        D[1] = D[1] - (U[2] - lv) * T_u;
        D[2] = D[2] - (U[2] - lv) * t_v_R - T_p / U[0];
        D[3] = D[3] - (U[2] - lv) * T_p - U[0] * C * C * t_v_R;
        if (sc) {
            DX[0] = DX[0] - (U[2] - lv) * XR->tz;
            DX[1] = DX[1] - (U[2] - lv) * XR->tphi;
        }
    }
}

/* Q of the rarefaction-side transversal correction (G2D :367-370): the
 * closed form has a removable singularity at gamma = 3. */
static double orc_g2d_q(double gam, double zeta, double c_frac, double eps)
{
    if (gam < 3.0 - eps || gam > 3.0 + eps)
        return (c_frac * (zeta - 1.0) + pow(c_frac, 0.5 / zeta) * zeta) / (2.0 * zeta - 1.0);
    return 0.5 * c_frac + pow(c_frac, 0.5 / zeta) * (0.5 - 0.25 / zeta * log(c_frac));
}

/*
 * Non-acoustic case of linear_GRP_solver_Edir_G2D,
 * src/riemann_solver/linear_grp_solver_Edir_G2D.c:273-629, single-fluid,
 * EXACT_TANGENT_DERIVATIVE off (the reference defines it only for its
 * documentation build, :16-18), frame velocities lambda_u = lambda_v = 0 as
 * GRP_2D_flux and flux_generator_x/_y leave them (flux_solver.c:163,
 * flux_generator_x.c:35-36).  Unlike the quasi-1D solver, the tangential
 * derivatives enter the characteristic relations of both waves (L_v, the Q
 * term of a rarefaction, and the v T_u / v T_p corrections of d_L, d_R).
 * c_frac is one variable across the branches, as in the reference: with two
 * rarefactions the 3-wave's value is the one the 1-side D[2] sees (:588).
 */
static void orc_g2d_nonacoustic(double gL, double gR, const orc_side *Ls, const orc_side *Rs, double eps,
                                const orc_star *st, double D[4], double U[4])
{
    const double lu = 0.0, lv = 0.0;
    const double rho_L = Ls->rho, rho_R = Rs->rho;
    const double d_rho_L = Ls->drho, d_rho_R = Rs->drho;
    const double t_rho_L = Ls->trho, t_rho_R = Rs->trho;
    const double u_L = Ls->u, u_R = Rs->u;
    const double d_u_L = Ls->du, d_u_R = Rs->du;
    const double t_u_L = Ls->tu, t_u_R = Rs->tu;
    const double v_L = Ls->v, v_R = Rs->v;
    const double d_v_L = Ls->dv, d_v_R = Rs->dv;
    const double t_v_L = Ls->tv, t_v_R = Rs->tv;
    const double p_L = Ls->p, p_R = Rs->p;
    const double d_p_L = Ls->dp, d_p_R = Rs->dp;
    const double t_p_L = Ls->tp, t_p_R = Rs->tp;
    const double c_L = st->c_L, c_R = st->c_R;
    const double u_star = st->u_star, p_star = st->p_star;
    const double rho_star_L = st->rho_star_L, rho_star_R = st->rho_star_R;
    const double c_star_L = st->c_star_L, c_star_R = st->c_star_R;
    const int *CRW = st->CRW;
    const double zetaL = (gL - 1.0) / (gL + 1.0);
    const double zetaR = (gR - 1.0) / (gR + 1.0);
    double C, c_frac = 1.0, TdS, d_Psi, d_Phi, VAR, Q;
    double T_rho, T_u, T_v, T_p;
    double H1, H2, H3, a_L, b_L, d_L, a_R, b_R, d_R, detA, L_u, L_p, L_rho, L_v;
    double u_t_mat, p_t_mat, D0_p_tau, D0_u_tau, SmUs, SmUL, SmUR, rho_x, f;

    /* trivial cases: the t-axis lies outside the wave fan (:274-304) */
    if (st->speed_L > lu) {
        U[0] = rho_L; U[1] = u_L; U[2] = v_L; U[3] = p_L;
        D[0] = -(u_L - lu) * d_rho_L - (v_L - lv) * t_rho_L - rho_L * (d_u_L + t_v_L);
        D[1] = -(u_L - lu) * d_u_L - (v_L - lv) * t_u_L - d_p_L / rho_L;
        D[2] = -(u_L - lu) * d_v_L - (v_L - lv) * t_v_L - t_p_L / rho_L;
        D[3] = -(u_L - lu) * d_p_L - (v_L - lv) * t_p_L - rho_L * c_L * c_L * (d_u_L + t_v_L);
        return;
    }
    if (st->speed_R < lu) {
        U[0] = rho_R; U[1] = u_R; U[2] = v_R; U[3] = p_R;
        D[0] = -(u_R - lu) * d_rho_R - (v_R - lv) * t_rho_R - rho_R * (d_u_R + t_v_R);
        D[1] = -(u_R - lu) * d_u_R - (v_R - lv) * t_u_R - d_p_R / rho_R;
        D[2] = -(u_R - lu) * d_v_R - (v_R - lv) * t_v_R - t_p_R / rho_R;
        D[3] = -(u_R - lu) * d_p_R - (v_R - lv) * t_p_R - rho_R * c_R * c_R * (d_u_R + t_v_R);
        return;
    }

    /* tangential derivatives from the acoustic relations across the star side
     * that holds the t-axis (:337-349, the #else branch) */
    if (u_star < lu) {
        T_p = 0.5 * ((t_u_L - t_u_R) * rho_star_R * c_star_R + t_p_L + t_p_R);
        T_u = 0.5 * (t_u_L + t_u_R + (t_p_L - t_p_R) / rho_star_R / c_star_R);
        T_rho = t_rho_R - t_p_R / (c_star_R * c_star_R) + T_p / (c_star_R * c_star_R);
    } else {
        T_p = 0.5 * ((t_u_L - t_u_R) * rho_star_L * c_star_L + t_p_L + t_p_R);
        T_u = 0.5 * (t_u_L + t_u_R + (t_p_L - t_p_R) / rho_star_L / c_star_L);
        T_rho = t_rho_L - t_p_L / (c_star_L * c_star_L) + T_p / (c_star_L * c_star_L);
    }

    if (CRW[0] && ((u_star - c_star_L) > lu)) { /* t-axis inside the 1-rarefaction (:351-384) */
        U[1] = zetaL * (u_L + 2.0 * (c_L + lu) / (gL - 1.0));
        C = U[1] - lu;
        U[3] = pow(C / c_L, 2.0 * gL / (gL - 1.0)) * p_L;
        U[0] = gL * U[3] / C / C;
        U[2] = v_L;
        c_frac = C / c_L;
        TdS = (d_p_L - d_rho_L * c_L * c_L) / (gL - 1.0) / rho_L;
        d_Psi = d_u_L + (gL * d_p_L / c_L - c_L * d_rho_L) / (gL - 1.0) / rho_L;
        D[1] = ((1.0 + zetaL) * pow(c_frac, 0.5 / zetaL) + zetaL * pow(c_frac, (1.0 + zetaL) / zetaL));
        D[1] = D[1] / (1.0 + 2.0 * zetaL) * TdS;
        D[1] = D[1] - c_L * pow(c_frac, 0.5 / zetaL) * d_Psi;
        Q = orc_g2d_q(gL, zetaL, c_frac, eps);
        D[1] = D[1] - c_L * t_v_L * Q;
        D[3] = U[0] * (U[1] - lu) * D[1];
        D[0] = U[0] * (U[1] - lu) * pow(c_frac, (1.0 + zetaL) / zetaL) * TdS * (gL - 1.0);
        D[0] = (D[0] + D[3]) / C / C - (U[2] - lv) * T_rho;
        D[2] = -(U[1] - lu) * d_v_L * U[0] / rho_L - (U[2] - lv) * t_v_L - T_p / U[0];
        D[2] = D[2] - (zetaL - 1.0) * (pow(c_frac, 2.0 / zetaL - 1.0) - 1.0) / (zetaL - 2.0) / U[0] * t_p_L;
        D[3] = D[3] - (U[2] - lv) * T_p;
        D[1] = D[1] - (U[2] - lv) * T_u + U[1] * t_v_L;
        return;
    }
    if (CRW[1] && ((u_star + c_star_R) < lu)) { /* t-axis inside the 3-rarefaction (:385-418) */
        U[1] = zetaR * (u_R - 2.0 * (c_R - lu) / (gR - 1.0));
        C = lu - U[1];
        U[3] = pow(C / c_R, 2.0 * gR / (gR - 1.0)) * p_R;
        U[0] = gR * U[3] / C / C;
        U[2] = v_R;
        c_frac = C / c_R;
        TdS = (d_p_R - d_rho_R * c_R * c_R) / (gR - 1.0) / rho_R;
        d_Phi = d_u_R - (gR * d_p_R / c_R - c_R * d_rho_R) / (gR - 1.0) / rho_R;
        D[1] = ((1.0 + zetaR) * pow(c_frac, 0.5 / zetaR) + zetaR * pow(c_frac, (1.0 + zetaR) / zetaR));
        D[1] = D[1] / (1.0 + 2.0 * zetaR) * TdS;
        D[1] = D[1] + c_R * pow(c_frac, 0.5 / zetaR) * d_Phi;
        Q = orc_g2d_q(gR, zetaR, c_frac, eps);
        D[1] = D[1] + c_R * t_v_R * Q;
        D[3] = U[0] * (U[1] - lu) * D[1];
        D[0] = U[0] * (U[1] - lu) * pow(c_frac, (1.0 + zetaR) / zetaR) * TdS * (gR - 1.0);
        D[0] = (D[0] + D[3]) / C / C - (U[2] - lv) * T_rho;
        D[2] = -(U[1] - lu) * d_v_R * U[0] / rho_R - (U[2] - lv) * t_v_R - T_p / U[0];
        D[2] = D[2] - (zetaR - 1.0) * (pow(c_frac, 2.0 / zetaR - 1.0) - 1.0) / (zetaR - 2.0) / U[0] * t_p_R;
        D[3] = D[3] - (U[2] - lv) * T_p;
        D[1] = D[1] - (U[2] - lv) * T_u + U[1] * t_v_R;
        return;
    }

    /* non-sonic case (:419-627): the t-axis is in the star region */
    if (u_star < lu) {
        U[0] = rho_star_R; U[1] = u_star; U[2] = v_R; U[3] = p_star;
        C = c_star_R;
        T_v = t_v_R;
    } else {
        U[0] = rho_star_L; U[1] = u_star; U[2] = v_L; U[3] = p_star;
        C = c_star_L;
        T_v = t_v_L;
    }
    /* characteristic relation across the 1-wave: a_L u_t + b_L p_t = d_L (:444-481) */
    if (CRW[0]) {
        a_L = 1.0;
        b_L = 1.0 / rho_star_L / c_star_L;
        c_frac = c_star_L / c_L;
        TdS = (d_p_L - d_rho_L * c_L * c_L) / (gL - 1.0) / rho_L;
        d_Psi = d_u_L + (gL * d_p_L / c_L - c_L * d_rho_L) / (gL - 1.0) / rho_L;
        d_L = ((1.0 + zetaL) * pow(c_frac, 0.5 / zetaL) + zetaL * pow(c_frac, (1.0 + zetaL) / zetaL));
        d_L = d_L / (1.0 + 2.0 * zetaL) * TdS;
        d_L = d_L - c_L * pow(c_frac, 0.5 / zetaL) * d_Psi;
        Q = orc_g2d_q(gL, zetaL, c_frac, eps);
        d_L = d_L - c_L * t_v_L * Q;
    } else {
        SmUs = -sqrt(0.5 * ((gL + 1.0) * p_L + (gL - 1.0) * p_star) / rho_star_L);
        SmUL = -sqrt(0.5 * ((gL + 1.0) * p_star + (gL - 1.0) * p_L) / rho_L);
        VAR = sqrt((1 - zetaL) / (rho_L * (p_star + zetaL * p_L)));
        H1 = 0.5 * VAR * (p_star + (1.0 + 2.0 * zetaL) * p_L) / (p_star + zetaL * p_L);
        H2 = -0.5 * VAR * ((2.0 + zetaL) * p_star + zetaL * p_L) / (p_star + zetaL * p_L);
        H3 = -0.5 * VAR * (p_star - p_L) / rho_L;
        L_p = -1.0 / rho_L - SmUL * H2;
        L_u = SmUL + rho_L * (c_L * c_L * H2 + H3);
        L_rho = -SmUL * H3;
        L_v = SmUs + rho_L * (c_L * c_L * H2 + H3);
        a_L = 1.0 - rho_star_L * SmUs * H1;
        b_L = -SmUs / (rho_star_L * c_star_L * c_star_L) + H1;
        d_L = L_rho * d_rho_L + L_u * d_u_L + L_p * d_p_L + L_v * t_v_L;
    }
    d_L = d_L - a_L * v_L * T_u - b_L * v_L * T_p;
    /* and across the 3-wave (:482-519) */
    if (CRW[1]) {
        a_R = 1.0;
        b_R = -1.0 / rho_star_R / c_star_R;
        c_frac = c_star_R / c_R;
        TdS = (d_p_R - d_rho_R * c_R * c_R) / (gR - 1.0) / rho_R;
        d_Phi = d_u_R - (gR * d_p_R / c_R - c_R * d_rho_R) / (gR - 1.0) / rho_R;
        d_R = ((1.0 + zetaR) * pow(c_frac, 0.5 / zetaR) + zetaR * pow(c_frac, (1.0 + zetaR) / zetaR));
        d_R = d_R / (1.0 + 2.0 * zetaR) * TdS;
        d_R = d_R + c_R * pow(c_frac, 0.5 / zetaR) * d_Phi;
        Q = orc_g2d_q(gR, zetaR, c_frac, eps);
        d_R = d_R + c_R * t_v_R * Q;
    } else {
        SmUs = sqrt(0.5 * ((gR + 1.0) * p_R + (gR - 1.0) * p_star) / rho_star_R);
        SmUR = sqrt(0.5 * ((gR + 1.0) * p_star + (gR - 1.0) * p_R) / rho_R);
        VAR = sqrt((1.0 - zetaR) / (rho_R * (p_star + zetaR * p_R)));
        H1 = 0.5 * VAR * (p_star + (1 + 2.0 * zetaR) * p_R) / (p_star + zetaR * p_R);
        H2 = -0.5 * VAR * ((2.0 + zetaR) * p_star + zetaR * p_R) / (p_star + zetaR * p_R);
        H3 = -0.5 * VAR * (p_star - p_R) / rho_R;
        L_p = -1.0 / rho_R + SmUR * H2;
        L_u = SmUR - rho_R * (c_R * c_R * H2 + H3);
        L_rho = SmUR * H3;
        L_v = SmUs - rho_R * (c_R * c_R * H2 + H3);
        a_R = 1.0 + rho_star_R * SmUs * H1;
        b_R = -(SmUs / (rho_star_R * c_star_R * c_star_R) + H1);
        d_R = L_rho * d_rho_R + L_u * d_u_R + L_p * d_p_R + L_v * t_v_R;
    }
    d_R = d_R - a_R * v_R * T_u - b_R * v_R * T_p;
    detA = a_L * b_R - b_L * a_R;
    u_t_mat = (b_R * d_L - b_L * d_R) / detA;
    p_t_mat = (a_L * d_R - a_R * d_L) / detA;
    D0_p_tau = p_t_mat + U[2] * T_p;
    D0_u_tau = u_t_mat + U[2] * T_u;
    /* total derivatives along the t-axis (:521-530) */
    D[1] = u_t_mat + (u_star - lu) / U[0] / C / C * D0_p_tau + (u_star - lu) * T_v;
    D[3] = p_t_mat + (u_star - lu) * U[0] * D0_u_tau;
    if (u_star < lu) {
        if (CRW[1]) { /* :533-546 */
            D[0] = rho_star_R * (u_star - lu) * pow(c_star_R / c_R, (1.0 + zetaR) / zetaR) * (d_p_R - d_rho_R * c_R * c_R) / rho_R;
            D[0] = (D[0] + D[3] + U[2] * T_p) / c_star_R / c_star_R - (U[2] - lv) * T_rho;
            D[2] = -U[1] * d_v_R * U[0] / rho_R - (U[2] - lv) * t_v_R - T_p / U[0];
            D[2] = D[2] + lu * d_v_R;
            D[2] = D[2] + u_star / c_star_R * (zetaR - 1.0) * (pow(c_frac, 2.0 / zetaR - 1.0) - 1.0) / (zetaR - 2.0) / U[0] * t_p_R;
        } else { /* :547-577 */
            SmUs = sqrt(0.5 * ((gR + 1.0) * p_R + (gR - 1.0) * p_star) / rho_star_R);
            SmUR = sqrt(0.5 * ((gR + 1.0) * p_star + (gR - 1.0) * p_R) / rho_R);
            VAR = p_R + zetaR * p_star;
            H1 = rho_R * p_R * (1.0 - zetaR * zetaR) / VAR / VAR;
            H2 = rho_R * p_star * (zetaR * zetaR - 1.0) / VAR / VAR;
            H3 = (p_star + zetaR * p_R) / VAR;
            L_rho = SmUR * H3 * d_rho_R;
            L_u = -rho_R * (H2 * c_R * c_R + H3) * d_u_R;
            L_p = H2 * SmUR * d_p_R;
            L_v = -rho_R * (H2 * c_R * c_R + H3) * t_v_R;
            D[0] = ((u_star + SmUs) / c_star_R / c_star_R - u_star * H1) * D0_p_tau + rho_star_R * u_star * SmUs * H1 * D0_u_tau;
            D[0] = (D[0] - u_star * (L_p + L_rho + L_u + L_v)) / SmUs;
            D[0] = D[0] - (U[2] - lv) * T_rho;
            f = SmUR * (H2 * d_p_R + H3 * d_rho_R) - rho_R * (H2 * c_R * c_R + H3) * d_u_R;
            rho_x = (f + H1 * (p_t_mat - rho_star_R * SmUs * u_t_mat) - D[0]) / (SmUR + u_R);
            D[0] = D[0] + lu * rho_x;
            D[2] = -(U[1] * (SmUR * d_v_R - t_p_R / rho_R) + (u_star + SmUs) * T_p / U[0]) / SmUs;
            D[2] = D[2] + lu * d_v_R - (U[2] - lv) * t_v_R;
        }
    } else {
        if (CRW[0]) { /* :580-593 */
            D[0] = rho_star_L * (u_star - lu) * pow(c_star_L / c_L, (1.0 + zetaL) / zetaL) * (d_p_L - d_rho_L * c_L * c_L) / rho_L;
            D[0] = (D[0] + D[3] + U[2] * T_p) / c_star_L / c_star_L - (U[2] - lv) * T_rho;
            D[2] = -U[1] * d_v_L * U[0] / rho_L - (U[2] - lv) * t_v_L - T_p / U[0];
            D[2] = D[2] + lu * d_v_L;
            D[2] = D[2] - u_star / c_star_L * (zetaL - 1.0) * (pow(c_frac, 2.0 / zetaL - 1.0) - 1.0) / (zetaL - 2.0) / U[0] * t_p_L;
        } else { /* :594-624 */
            SmUs = -sqrt(0.5 * ((gL + 1.0) * p_L + (gL - 1.0) * p_star) / rho_star_L);
            SmUL = -sqrt(0.5 * ((gL + 1.0) * p_star + (gL - 1.0) * p_L) / rho_L);
            VAR = p_L + zetaL * p_star;
            H1 = rho_L * p_L * (1.0 - zetaL * zetaL) / VAR / VAR;
            H2 = rho_L * p_star * (zetaL * zetaL - 1.0) / VAR / VAR;
            H3 = (p_star + zetaL * p_L) / VAR;
            L_rho = SmUL * H3 * d_rho_L;
            L_u = -rho_L * (H2 * c_L * c_L + H3) * d_u_L;
            L_p = H2 * SmUL * d_p_L;
            L_v = -rho_L * (H2 * c_L * c_L + H3) * t_v_L;
            D[0] = ((u_star + SmUs) / c_star_L / c_star_L - u_star * H1) * D0_p_tau + rho_star_L * u_star * SmUs * H1 * D0_u_tau;
            D[0] = (D[0] - u_star * (L_p + L_rho + L_u + L_v)) / SmUs;
            D[0] = D[0] - (U[2] - lv) * T_rho;
            f = SmUL * (H2 * d_p_L + H3 * d_rho_L) - rho_L * (H2 * c_L * c_L + H3) * d_u_L;
            rho_x = (f + H1 * (p_t_mat - rho_star_L * SmUs * u_t_mat) - D[0]) / (SmUL + u_L);
            D[0] = D[0] + lu * rho_x;
            D[2] = -(U[1] * (SmUL * d_v_L - t_p_L / rho_L) + (u_star + SmUs) * T_p / U[0]) / SmUs;
            D[2] = D[2] + lu * d_v_L - (U[2] - lv) * t_v_L;
        }
    }
    D[1] = D[1] + lv * T_u;
    D[3] = D[3] + lv * T_p;
}

static int orc_isfinite4(const double x[4])
{
    return isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]) && isfinite(x[3]);
}

/*
 * GRP_2D_flux, src/flux_calc/flux_solver.c:158-237: rotate both states to the
 * interface normal (n_x, n_y), solve the quasi-1D GRP, check the solution
 * (star_dire_check, src/inter_process/fluid_var_check.c:65-131, dim 2), form the
 * mid-time flux and the t+tau interface values.
 * out[0..3] = F_rho,F_u,F_v,F_e; out[4..7] = RHO_int,U_int,V_int,P_int.
 */
static int orc_grp2d_flux_one(double n_x, double n_y, double gamma, orc_side L, orc_side R,
                              double tau, double eps, double out[8], int *newton_iters, int g2d)
{
    double u = L.u * n_x + L.v * n_y;
    double u_R = R.u * n_x + R.v * n_y;
    double d_u = L.du * n_x + L.dv * n_y;
    double d_u_R = R.du * n_x + R.dv * n_y;
    double t_u = L.tu * n_x + L.tv * n_y;
    double t_u_R = R.tu * n_x + R.tv * n_y;
    L.v = -L.u * n_y + L.v * n_x;
    R.v = -R.u * n_y + R.v * n_x;
    L.dv = -L.du * n_y + L.dv * n_x;
    R.dv = -R.du * n_y + R.dv * n_x;
    L.tv = -L.tu * n_y + L.tv * n_x;
    R.tv = -R.tu * n_y + R.tv * n_x;
    L.u = u;
    R.u = u_R;
    L.du = d_u;
    R.du = d_u_R;
    L.tu = t_u;
    R.tu = t_u_R;

    double ws[2], dire[4], mid[4], star[4];
    orc_q1d_solve(gamma, gamma, &L, &R, eps, eps, ws, dire, mid, star, newton_iters, g2d);

    int retval = 0;
    if (mid[3] < eps || mid[0] < eps)
        retval = 1;
    else if (!orc_isfinite4(mid))
        retval = 2;
    else if (!orc_isfinite4(dire))
        retval = 3;

    double rho_mid = mid[0] + 0.5 * tau * dire[0];
    double u_mid = (mid[1] + 0.5 * tau * dire[1]) * n_x - (mid[2] + 0.5 * tau * dire[2]) * n_y;
    double v_mid = (mid[1] + 0.5 * tau * dire[1]) * n_y + (mid[2] + 0.5 * tau * dire[2]) * n_x;
    double p_mid = mid[3] + 0.5 * tau * dire[3];
    double F_rho = rho_mid * (u_mid * n_x + v_mid * n_y);
    double F_u = F_rho * u_mid + p_mid * n_x;
    double F_v = F_rho * v_mid + p_mid * n_y;
    double F_e = (gamma / (gamma - 1.0)) * p_mid / rho_mid + 0.5 * (u_mid * u_mid + v_mid * v_mid);
    F_e = F_rho * F_e;
    out[0] = F_rho;
    out[1] = F_u;
    out[2] = F_v;
    out[3] = F_e;
    out[5] = (mid[1] + tau * dire[1]) * n_x - (mid[2] + tau * dire[2]) * n_y;
    out[6] = (mid[1] + tau * dire[1]) * n_y + (mid[2] + tau * dire[2]) * n_x;
    out[4] = mid[0] + tau * dire[0];
    out[7] = mid[3] + tau * dire[3];
    return retval;
}

/* ifvar_check, src/inter_process/fluid_var_check.c:21-51, dim 2. */
static int orc_ifvar_check2(const orc_side *L, const orc_side *R, double eps)
{
    if (L->p < eps || R->p < eps || L->rho < eps || R->rho < eps)
        return 1;
    if (!isfinite(L->dp) || !isfinite(R->dp) || !isfinite(L->du) || !isfinite(R->du) ||
        !isfinite(L->dv) || !isfinite(R->dv) || !isfinite(L->drho) || !isfinite(R->drho))
        return 2;
    if (!isfinite(L->tp) || !isfinite(R->tp) || !isfinite(L->tu) || !isfinite(R->tu) ||
        !isfinite(L->tv) || !isfinite(R->tv) || !isfinite(L->trho) || !isfinite(R->trho))
        return 2;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* 1D direct Eulerian GRP solver                                              */
/* ------------------------------------------------------------------------- */

/* linear_GRP_solver_Edir, src/riemann_solver/linear_grp_solver_Edir.c:33-337.
 * in: rho,u,p,s_rho,s_u,s_p per side. D = (rho,u,p)_t, U = (rho,u,p) on the t-axis. */
static void orc_grp1d_solve(double gamma, const double Ls[6], const double Rs[6], double eps, double atc,
                            double D[3], double U[3])
{
    const double rho_L = Ls[0], u_L = Ls[1], p_L = Ls[2], s_rho_L = Ls[3], s_u_L = Ls[4], s_p_L = Ls[5];
    const double rho_R = Rs[0], u_R = Rs[1], p_R = Rs[2], s_rho_R = Rs[3], s_u_R = Rs[4], s_p_R = Rs[5];
    int CRW[2] = {0, 0};
    double u_star, p_star, rho_star_L, rho_star_R, c_star_L, c_star_R;
    double PI, H1, H2, H3, a_L, b_L, d_L, a_R, b_R, d_R, L_u, L_p, L_rho, u_t_mat, p_t_mat;
    double shk_spd, g_rho, g_u, g_p, f, speed_L, speed_R;
    const double zeta = (gamma - 1.0) / (gamma + 1.0), zts = zeta * zeta;

    double c_L = sqrt(gamma * p_L / rho_L);
    double c_R = sqrt(gamma * p_R / rho_R);
    double dist = sqrt((u_L - u_R) * (u_L - u_R) + (p_L - p_R) * (p_L - p_R));
    if (dist < atc && atc < 2 * eps) {
        rho_star_L = rho_L;
        rho_star_R = rho_R;
        c_star_L = c_L;
        c_star_R = c_R;
        u_star = 0.5 * (u_R + u_L);
        p_star = 0.5 * (p_R + p_L);
    } else {
        orc_exact(gamma, gamma, u_L, u_R, p_L, p_R, c_L, c_R, eps, eps, 50, &u_star, &p_star, CRW, NULL);
        if (p_star > p_L)
            rho_star_L = rho_L * (p_star + zeta * p_L) / (p_L + zeta * p_star);
        else
            rho_star_L = rho_L * pow(p_star / p_L, 1.0 / gamma);
        if (p_star > p_R)
            rho_star_R = rho_R * (p_star + zeta * p_R) / (p_R + zeta * p_star);
        else
            rho_star_R = rho_R * pow(p_star / p_R, 1.0 / gamma);
        c_star_L = sqrt(gamma * p_star / rho_star_L);
        c_star_R = sqrt(gamma * p_star / rho_star_R);
    }

    if (dist < atc) { /* acoustic case, :86-144 */
        if (u_L - c_L > 0.0) {
            D[0] = -s_rho_L * u_L - rho_L * s_u_L;
            D[1] = (D[0] * u_L + s_rho_L * u_L * u_L + 2.0 * rho_L * u_L * s_u_L + s_p_L) / -rho_L;
            D[2] = -(gamma - 1.0) * (0.5 * D[0] * u_L * u_L + rho_L * u_L * D[1]);
            D[2] = D[2] - s_u_L * (gamma * p_L + 0.5 * (gamma - 1.0) * rho_L * u_L * u_L);
            D[2] = D[2] - u_L * (gamma * s_p_L + (gamma - 1.0) * (0.5 * s_rho_L * u_L * u_L + rho_L * u_L * s_u_L));
            U[0] = rho_L; U[1] = u_L; U[2] = p_L;
        } else if (u_R + c_R < 0.0) {
            D[0] = -s_rho_R * u_R - rho_R * s_u_R;
            D[1] = (D[0] * u_R + s_rho_R * u_R * u_R + 2.0 * rho_R * u_R * s_u_R + s_p_R) / -rho_R;
            D[2] = -(gamma - 1.0) * (0.5 * D[0] * u_R * u_R + rho_R * u_R * D[1]);
            D[2] = D[2] - s_u_R * (gamma * p_R + 0.5 * (gamma - 1.0) * rho_R * u_R * u_R);
            D[2] = D[2] - u_R * (gamma * s_p_R + (gamma - 1.0) * (0.5 * s_rho_R * u_R * u_R + rho_R * u_R * s_u_R));
            U[0] = rho_R; U[1] = u_R; U[2] = p_R;
        } else if (u_star > 0.0) {
            U[0] = rho_star_L; U[1] = u_star; U[2] = p_star;
            PI = (u_star + c_star_R) * rho_star_L * c_star_L * c_star_L / (u_star - c_star_L) / rho_star_R / c_star_R / c_star_R;
            D[1] = (s_p_L / rho_L + c_L * s_u_L) * PI / (1.0 - PI) + (s_p_R / rho_R - c_R * s_u_R) / (PI - 1.0);
            D[2] = ((u_star + c_star_R) / rho_star_R / c_star_R / c_star_R) - ((u_star - c_star_L) / rho_star_L / c_star_L / c_star_L);
            D[2] = (s_p_R / rho_R - c_R * s_u_R - s_p_L / rho_L - c_L * s_u_L) / D[2];
            D[2] = D[2] * (1.0 - (u_star * u_star / c_star_L / c_star_L)) + rho_star_L * u_star * D[1];
            D[0] = (u_star * (s_p_L - s_rho_L * c_star_L * c_star_L) + D[2]) / c_star_L / c_star_L;
        } else {
            U[0] = rho_star_R; U[1] = u_star; U[2] = p_star;
            PI = (u_star + c_star_R) * rho_star_L * c_star_L * c_star_L / (u_star - c_star_L) / rho_star_R / c_star_R / c_star_R;
            D[1] = (s_p_L / rho_L + c_L * s_u_L) * PI / (1.0 - PI) + (s_p_R / rho_R - c_R * s_u_R) / (PI - 1.0);
            D[2] = ((u_star + c_star_R) / rho_star_R / c_star_R / c_star_R) - ((u_star - c_star_L) / rho_star_L / c_star_L / c_star_L);
            D[2] = (s_p_R / rho_R - c_R * s_u_R - s_p_L / rho_L - c_L * s_u_L) / D[2];
            D[2] = D[2] * (1.0 - (u_star * u_star / c_star_R / c_star_R)) + rho_star_R * u_star * D[1];
            D[0] = (u_star * (s_p_R - s_rho_R * c_star_R * c_star_R) + D[2]) / c_star_R / c_star_R;
        }
        return;
    }

    /* non-acoustic case, :146-336 */
    if (CRW[0])
        speed_L = u_L - c_L;
    else
        speed_L = (rho_star_L * u_star - rho_L * u_L) / (rho_star_L - rho_L);
    if (CRW[1])
        speed_R = u_R + c_R;
    else
        speed_R = (rho_star_R * u_star - rho_R * u_R) / (rho_star_R - rho_R);

    if (speed_L > 0.0) {
        D[0] = -s_rho_L * u_L - rho_L * s_u_L;
        D[1] = (D[0] * u_L + s_rho_L * u_L * u_L + 2.0 * rho_L * u_L * s_u_L + s_p_L) / -rho_L;
        D[2] = (s_u_L * p_L + u_L * s_p_L) * gamma / (1.0 - gamma) - 0.5 * s_rho_L * u_L * u_L * u_L - 1.5 * rho_L * u_L * u_L * s_u_L;
        D[2] = D[2] - 0.5 * D[0] * u_L * u_L - rho_L * u_L * D[1];
        D[2] = D[2] * (gamma - 1.0);
        U[0] = rho_L; U[1] = u_L; U[2] = p_L;
    } else if (speed_R < 0.0) {
        D[0] = -s_rho_R * u_R - rho_R * s_u_R;
        D[1] = (D[0] * u_R + s_rho_R * u_R * u_R + 2.0 * rho_R * u_R * s_u_R + s_p_R) / -rho_R;
        D[2] = -(gamma - 1.0) * (0.5 * D[0] * u_R * u_R + rho_R * u_R * D[1]);
        D[2] = D[2] - s_u_R * (gamma * p_R + 0.5 * (gamma - 1.0) * rho_R * u_R * u_R);
        D[2] = D[2] - u_R * (gamma * s_p_R + (gamma - 1.0) * (0.5 * s_rho_R * u_R * u_R + rho_R * u_R * s_u_R));
        U[0] = rho_R; U[1] = u_R; U[2] = p_R;
    } else if ((CRW[0]) && ((u_star - c_star_L) > 0.0)) {
        U[1] = zeta * (u_L + 2.0 * c_L / (gamma - 1.0));
        U[2] = U[1] * U[1] * rho_L / gamma / pow(p_L, 1.0 / gamma);
        U[2] = pow(U[2], gamma / (gamma - 1.0));
        U[0] = gamma * U[2] / U[1] / U[1];
        D[1] = 0.5 * (pow(U[1] / c_L, 0.5 / zeta) * (1.0 + zeta) + pow(U[1] / c_L, (1.0 + zeta) / zeta) * zeta) / (0.5 + zeta);
        D[1] = D[1] * (s_p_L - s_rho_L * c_L * c_L) / (gamma - 1.0) / rho_L;
        D[1] = D[1] - c_L * pow(U[1] / c_L, 0.5 / zeta) * (s_u_L + (gamma * s_p_L / c_L - c_L * s_rho_L) / (gamma - 1.0) / rho_L);
        D[2] = U[0] * U[1] * D[1];
        D[0] = U[0] * U[1] * pow(U[1] / c_L, (1.0 + zeta) / zeta) * (s_p_L - s_rho_L * c_L * c_L) / rho_L;
        D[0] = (D[0] + D[2]) / U[1] / U[1];
    } else if ((CRW[1]) && ((u_star + c_star_R) < 0.0)) {
        U[1] = zeta * (u_R - 2.0 * c_R / (gamma - 1.0));
        U[2] = U[1] * U[1] * rho_R / gamma / pow(p_R, 1.0 / gamma);
        U[2] = pow(U[2], gamma / (gamma - 1.0));
        U[0] = gamma * U[2] / U[1] / U[1];
        D[1] = 0.5 * (pow(-U[1] / c_R, 0.5 / zeta) * (1.0 + zeta) + pow(-U[1] / c_R, (1.0 + zeta) / zeta) * zeta) / (0.5 + zeta);
        D[1] = D[1] * (s_p_R - s_rho_R * c_R * c_R) / (gamma - 1.0) / rho_R;
        D[1] = D[1] + c_R * pow(-U[1] / c_R, 0.5 / zeta) * (s_u_R - (gamma * s_p_R / c_R - c_R * s_rho_R) / (gamma - 1.0) / rho_R);
        D[2] = U[0] * U[1] * D[1];
        D[0] = U[0] * U[1] * pow(-U[1] / c_R, (1.0 + zeta) / zeta) * (s_p_R - s_rho_R * c_R * c_R) / rho_R;
        D[0] = (D[0] + D[2]) / U[1] / U[1];
    } else {
        if (CRW[0]) {
            a_L = 1.0;
            b_L = 1.0 / rho_star_L / c_star_L;
            d_L = 0.5 * (pow(c_star_L / c_L, 0.5 / zeta) * (1.0 + zeta) + pow(c_star_L / c_L, (1.0 + zeta) / zeta) * zeta) / (0.5 + zeta);
            d_L = d_L * (s_p_L - s_rho_L * c_L * c_L) / (gamma - 1.0) / rho_L;
            d_L = d_L - c_L * pow(c_star_L / c_L, 0.5 / zeta) * (s_u_L + (gamma * s_p_L / c_L - c_L * s_rho_L) / (gamma - 1.0) / rho_L);
        } else {
            H1 = 0.5 * sqrt((1.0 - zeta) / (rho_L * (p_star + zeta * p_L))) * (p_star + (1.0 + 2.0 * zeta) * p_L) / (p_star + zeta * p_L);
            H2 = -0.5 * sqrt((1.0 - zeta) / (rho_L * (p_star + zeta * p_L))) * ((2.0 + zeta) * p_star + zeta * p_L) / (p_star + zeta * p_L);
            H3 = -0.5 * sqrt((1.0 - zeta) / (rho_L * (p_star + zeta * p_L))) * (p_star - p_L) / rho_L;
            shk_spd = (rho_star_L * u_star - rho_L * u_L) / (rho_star_L - rho_L);
            a_L = 1.0 - rho_star_L * (shk_spd - u_star) * H1;
            b_L = (u_star - shk_spd) / rho_star_L / c_star_L / c_star_L + H1;
            L_rho = (u_L - shk_spd) * H3;
            L_u = shk_spd - u_L + rho_L * c_L * c_L * H2 + rho_L * H3;
            L_p = (u_L - shk_spd) * H2 - 1.0 / rho_L;
            d_L = L_rho * s_rho_L + L_u * s_u_L + L_p * s_p_L;
        }
        if (CRW[1]) {
            a_R = 1.0;
            b_R = -1.0 / rho_star_R / c_star_R;
            d_R = 0.5 * (pow(c_star_R / c_R, 0.5 / zeta) * (1.0 + zeta) + pow(c_star_R / c_R, (1.0 + zeta) / zeta) * zeta) / (0.5 + zeta);
            d_R = d_R * (s_p_R - s_rho_R * c_R * c_R) / (gamma - 1.0) / rho_R;
            d_R = d_R + c_R * pow(c_star_R / c_R, 0.5 / zeta) * (s_u_R - (gamma * s_p_R / c_R - c_R * s_rho_R) / (gamma - 1.0) / rho_R);
        } else {
            H1 = 0.5 * sqrt((1.0 - zeta) / (rho_R * (p_star + zeta * p_R))) * (p_star + (1.0 + 2.0 * zeta) * p_R) / (p_star + zeta * p_R);
            H2 = -0.5 * sqrt((1.0 - zeta) / (rho_R * (p_star + zeta * p_R))) * ((2.0 + zeta) * p_star + zeta * p_R) / (p_star + zeta * p_R);
            H3 = -0.5 * sqrt((1.0 - zeta) / (rho_R * (p_star + zeta * p_R))) * (p_star - p_R) / rho_R;
            shk_spd = (rho_star_R * u_star - rho_R * u_R) / (rho_star_R - rho_R);
            a_R = 1.0 + rho_star_R * (shk_spd - u_star) * H1;
            b_R = (u_star - shk_spd) / rho_star_R / c_star_R / c_star_R - H1;
            L_rho = (shk_spd - u_R) * H3;
            L_u = shk_spd - u_R - rho_R * c_R * c_R * H2 - rho_R * H3;
            L_p = (shk_spd - u_R) * H2 - 1.0 / rho_R;
            d_R = L_rho * s_rho_R + L_u * s_u_R + L_p * s_p_R;
        }
        p_t_mat = (d_L * a_R / a_L - d_R) / (b_L * a_R / a_L - b_R);
        u_t_mat = (d_L - b_L * p_t_mat) / a_L;
        if (u_star < 0.0) {
            U[0] = rho_star_R; U[1] = u_star; U[2] = p_star;
            D[1] = u_t_mat + u_star * p_t_mat / rho_star_R / c_star_R / c_star_R;
            D[2] = p_t_mat + rho_star_R * u_star * u_t_mat;
            if (CRW[1]) {
                D[0] = rho_star_R * u_star * pow(c_star_R / c_R, (1.0 + zeta) / zeta) * (s_p_R - s_rho_R * c_R * c_R) / rho_R;
                D[0] = (D[0] + D[2]) / c_star_R / c_star_R;
            } else {
                shk_spd = (rho_star_R * u_star - rho_R * u_R) / (rho_star_R - rho_R);
                H1 = rho_R * p_R * (1.0 - zts) / (p_R + zeta * p_star) / (p_R + zeta * p_star);
                H2 = rho_R * p_star * (zts - 1.0) / (p_R + zeta * p_star) / (p_R + zeta * p_star);
                H3 = (p_star + zeta * p_R) / (p_R + zeta * p_star);
                g_rho = u_star - shk_spd;
                g_u = u_star * rho_star_R * (shk_spd - u_star) * H1;
                g_p = shk_spd / c_star_R / c_star_R - u_star * H1;
                f = (shk_spd - u_R) * (H2 * s_p_R + H3 * s_rho_R) - rho_R * (H2 * c_R * c_R + H3) * s_u_R;
                D[0] = (f * u_star - g_p * p_t_mat - g_u * u_t_mat) / g_rho;
            }
        } else {
            U[0] = rho_star_L; U[1] = u_star; U[2] = p_star;
            D[1] = u_t_mat + u_star * p_t_mat / rho_star_L / c_star_L / c_star_L;
            D[2] = p_t_mat + rho_star_L * u_star * u_t_mat;
            if (CRW[0]) {
                D[0] = rho_star_L * u_star * pow(c_star_L / c_L, (1.0 + zeta) / zeta) * (s_p_L - s_rho_L * c_L * c_L) / rho_L;
                D[0] = (D[0] + D[2]) / c_star_L / c_star_L;
            } else {
                shk_spd = (rho_star_L * u_star - rho_L * u_L) / (rho_star_L - rho_L);
                H1 = rho_L * p_L * (1.0 - zts) / (p_L + zeta * p_star) / (p_L + zeta * p_star);
                H2 = rho_L * p_star * (zts - 1.0) / (p_L + zeta * p_star) / (p_L + zeta * p_star);
                H3 = (p_star + zeta * p_L) / (p_L + zeta * p_star);
                g_rho = u_star - shk_spd;
                g_u = u_star * rho_star_L * (shk_spd - u_star) * H1;
                g_p = shk_spd / c_star_L / c_star_L - u_star * H1;
                f = (shk_spd - u_L) * (H2 * s_p_L + H3 * s_rho_L) - rho_L * (H2 * c_L * c_L + H3) * s_u_L;
                D[0] = (f * u_star - g_p * p_t_mat - g_u * u_t_mat) / g_rho;
            }
        }
    }
}

/* star_dire_check dim 1, el = 0 (fluid_var_check.c:92-108). */
static int orc_star_dire_check1(const double mid[3], const double dire[3], double eps)
{
    if (mid[2] < eps || mid[0] < eps)
        return 1;
    if (!isfinite(mid[1]) || !isfinite(mid[2]) || !isfinite(mid[0]))
        return 2;
    if (!isfinite(dire[1]) || !isfinite(dire[2]) || !isfinite(dire[0]))
        return 3;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* 2D time loops                                                              */
/* ------------------------------------------------------------------------- */

typedef struct {
    int m, n;
    double gamma, eps, hx, hy, alpha;
    int bx, by;
    int g2d; /* interface solver: 0 = quasi-1D (the reference's), 1 = genuinely 2D (config[301] = 1) */
    double *snap[5][5]; /* snap[k][var]: var = rho,u,v,p,E; k < N_T */
    double *s[4], *t[4];                  /* x- and y-slopes (rho,u,v,p), [j*n+i] */
    double *F[4], *Ix[4];                 /* x-faces, [j*n+i], j = 0..m           */
    double *G[4], *Iy[4];                 /* y-faces, [j*(n+1)+i], i = 0..n       */
    unsigned char *cx, *cy;               /* per-face error codes                  */
    orc_ghost *gL, *gR, *gD, *gU;
} orc2d;

#define AT(j, i) ((size_t)(j) * n + (i))
#define ATY(j, i) ((size_t)(j) * (n + 1) + (i))

/* Ghost values along x: bound_cond_slope_limiter_x.c:34-82. cur = working state,
 * ini = CV[0]. Returns 0 for an unknown boundary code. */
static int orc_bc_values_x(orc2d *c, double *const cur[5], double *const ini[5], int found)
{
    const int m = c->m, n = c->n;
    for (int i = 0; i < n; ++i) {
        orc_ghost *L = &c->gL[i], *R = &c->gR[i];
        size_t a = AT(0, i), b = AT(m - 1, i);
        switch (c->bx) {
        case -1:
            if (found)
                break;
            L->u = ini[1][a]; R->u = ini[1][b];
            L->v = ini[2][a]; R->v = ini[2][b];
            L->p = ini[3][a]; R->p = ini[3][b];
            L->rho = ini[0][a]; R->rho = ini[0][b];
            break;
        case -2:
            L->u = -cur[1][a]; R->u = -cur[1][b];
            L->v = cur[2][a]; R->v = cur[2][b];
            L->p = cur[3][a]; R->p = cur[3][b];
            L->rho = cur[0][a]; R->rho = cur[0][b];
            break;
        case -4:
            L->u = cur[1][a]; R->u = cur[1][b];
            L->v = cur[2][a]; R->v = cur[2][b];
            L->p = cur[3][a]; R->p = cur[3][b];
            L->rho = cur[0][a]; R->rho = cur[0][b];
            break;
        case -7:
            L->u = cur[1][b]; R->u = cur[1][a];
            L->v = cur[2][b]; R->v = cur[2][a];
            L->p = cur[3][b]; R->p = cur[3][a];
            L->rho = cur[0][b]; R->rho = cur[0][a];
            break;
        case -24:
            L->u = -cur[1][a]; R->u = cur[1][b];
            L->v = cur[2][a]; R->v = cur[2][b];
            L->p = cur[3][a]; R->p = cur[3][b];
            L->rho = cur[0][a]; R->rho = cur[0][b];
            break;
        default:
            return 0;
        }
    }
    return 1;
}

/* bound_cond_slope_limiter_y.c:34-82 */
static int orc_bc_values_y(orc2d *c, double *const cur[5], double *const ini[5], int found)
{
    const int m = c->m, n = c->n;
    for (int j = 0; j < m; ++j) {
        orc_ghost *D = &c->gD[j], *U = &c->gU[j];
        size_t a = AT(j, 0), b = AT(j, n - 1);
        switch (c->by) {
        case -1:
            if (found)
                break;
            D->u = ini[1][a]; U->u = ini[1][b];
            D->v = ini[2][a]; U->v = ini[2][b];
            D->p = ini[3][a]; U->p = ini[3][b];
            D->rho = ini[0][a]; U->rho = ini[0][b];
            break;
        case -2:
            D->u = cur[1][a]; U->u = cur[1][b];
            D->v = -cur[2][a]; U->v = -cur[2][b];
            D->p = cur[3][a]; U->p = cur[3][b];
            D->rho = cur[0][a]; U->rho = cur[0][b];
            break;
        case -4:
            D->u = cur[1][a]; U->u = cur[1][b];
            D->v = cur[2][a]; U->v = cur[2][b];
            D->p = cur[3][a]; U->p = cur[3][b];
            D->rho = cur[0][a]; U->rho = cur[0][b];
            break;
        case -7:
            D->u = cur[1][b]; U->u = cur[1][a];
            D->v = cur[2][b]; U->v = cur[2][a];
            D->p = cur[3][b]; U->p = cur[3][a];
            D->rho = cur[0][b]; U->rho = cur[0][a];
            break;
        case -24:
            D->u = cur[1][a]; U->u = cur[1][b];
            D->v = -cur[2][a]; U->v = cur[2][b];
            D->p = cur[3][a]; U->p = cur[3][b];
            D->rho = cur[0][a]; U->rho = cur[0][b];
            break;
        default:
            return 0;
        }
    }
    return 1;
}

static double ghost_val(const orc_ghost *g, int var)
{
    switch (var) {
    case 0: return g->rho;
    case 1: return g->u;
    case 2: return g->v;
    default: return g->p;
    }
}

/* minmod_limiter_2D_x (slope_limiter_2D_x.c:32-84) on every row, then the ghost
 * x-slopes (bound_cond_slope_limiter_x.c:94-126). */
static void orc_limit_x(orc2d *c, double *const cur[5], int found)
{
    const int m = c->m, n = c->n;
    const double h = c->hx, alpha = c->alpha;
    int i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < n; ++i)
        for (int var = 0; var < 4; ++var) {
            const double *U = cur[var];
            double *s = c->s[var];
            const double UL = ghost_val(&c->gL[i], var), UR = ghost_val(&c->gR[i], var);
            for (int j = 0; j < m; ++j) {
                double sL, sR;
                if (j)
                    sL = (U[AT(j, i)] - U[AT(j - 1, i)]) / h;
                else
                    sL = (U[AT(j, i)] - UL) / h;
                if (j < m - 1)
                    sR = (U[AT(j + 1, i)] - U[AT(j, i)]) / h;
                else
                    sR = (UR - U[AT(j, i)]) / h;
                if (found)
                    s[AT(j, i)] = orc_minmod3(alpha * sL, alpha * sR, s[AT(j, i)]);
                else
                    s[AT(j, i)] = orc_minmod2(sL, sR);
            }
        }
    for (i = 0; i < n; ++i) {
        orc_ghost *L = &c->gL[i], *R = &c->gR[i];
        switch (c->bx) {
        case -2:
            L->su = c->s[1][AT(0, i)]; R->su = c->s[1][AT(m - 1, i)];
            break;
        case -7:
            L->su = c->s[1][AT(m - 1, i)]; R->su = c->s[1][AT(0, i)];
            L->sv = c->s[2][AT(m - 1, i)]; R->sv = c->s[2][AT(0, i)];
            L->sp = c->s[3][AT(m - 1, i)]; R->sp = c->s[3][AT(0, i)];
            L->srho = c->s[0][AT(m - 1, i)]; R->srho = c->s[0][AT(0, i)];
            break;
        case -24:
            L->su = c->s[1][AT(0, i)];
            break;
        }
    }
    for (int j = 0; j < m; ++j) {
        orc_ghost *D = &c->gD[j], *U = &c->gU[j];
        switch (c->by) {
        case -2: case -4: case -24:
            D->su = c->s[1][AT(j, 0)]; U->su = c->s[1][AT(j, n - 1)];
            D->sv = c->s[2][AT(j, 0)]; U->sv = c->s[2][AT(j, n - 1)];
            D->sp = c->s[3][AT(j, 0)]; U->sp = c->s[3][AT(j, n - 1)];
            D->srho = c->s[0][AT(j, 0)]; U->srho = c->s[0][AT(j, n - 1)];
            break;
        case -7:
            D->su = c->s[1][AT(j, n - 1)]; U->su = c->s[1][AT(j, 0)];
            D->sv = c->s[2][AT(j, n - 1)]; U->sv = c->s[2][AT(j, 0)];
            D->sp = c->s[3][AT(j, n - 1)]; U->sp = c->s[3][AT(j, 0)];
            D->srho = c->s[0][AT(j, n - 1)]; U->srho = c->s[0][AT(j, 0)];
            break;
        }
    }
}

/* minmod_limiter (slope_limiter.c:31-83) along every column, then the ghost
 * y-slopes (bound_cond_slope_limiter_y.c:94-126). */
static void orc_limit_y(orc2d *c, double *const cur[5], int found)
{
    const int m = c->m, n = c->n;
    const double h = c->hy, alpha = c->alpha;
    int j;
#pragma omp parallel for schedule(static)
    for (j = 0; j < m; ++j)
        for (int var = 0; var < 4; ++var) {
            const double *U = cur[var] + AT(j, 0);
            double *t = c->t[var] + AT(j, 0);
            const double UL = ghost_val(&c->gD[j], var), UR = ghost_val(&c->gU[j], var);
            for (int i = 0; i < n; ++i) {
                double sL, sR;
                if (i)
                    sL = (U[i] - U[i - 1]) / h;
                else
                    sL = (U[i] - UL) / h;
                if (i < n - 1)
                    sR = (U[i + 1] - U[i]) / h;
                else
                    sR = (UR - U[i]) / h;
                if (found)
                    t[i] = orc_minmod3(alpha * sL, alpha * sR, t[i]);
                else
                    t[i] = orc_minmod2(sL, sR);
            }
        }
    for (j = 0; j < m; ++j) {
        orc_ghost *D = &c->gD[j], *U = &c->gU[j];
        switch (c->by) {
        case -2:
            D->tv = c->t[2][AT(j, 0)]; U->tv = c->t[2][AT(j, n - 1)];
            break;
        case -7:
            D->tu = c->t[1][AT(j, n - 1)]; U->tu = c->t[1][AT(j, 0)];
            D->tv = c->t[2][AT(j, n - 1)]; U->tv = c->t[2][AT(j, 0)];
            D->tp = c->t[3][AT(j, n - 1)]; U->tp = c->t[3][AT(j, 0)];
            D->trho = c->t[0][AT(j, n - 1)]; U->trho = c->t[0][AT(j, 0)];
            break;
        case -24:
            D->tv = c->t[2][AT(j, 0)];
            break;
        }
    }
    for (int i = 0; i < n; ++i) {
        orc_ghost *L = &c->gL[i], *R = &c->gR[i];
        switch (c->bx) {
        case -2: case -4: case -24:
            L->tu = c->t[1][AT(0, i)]; R->tu = c->t[1][AT(m - 1, i)];
            L->tv = c->t[2][AT(0, i)]; R->tv = c->t[2][AT(m - 1, i)];
            L->tp = c->t[3][AT(0, i)]; R->tp = c->t[3][AT(m - 1, i)];
            L->trho = c->t[0][AT(0, i)]; R->trho = c->t[0][AT(m - 1, i)];
            break;
        case -7:
            L->tu = c->t[1][AT(m - 1, i)]; R->tu = c->t[1][AT(0, i)];
            L->tv = c->t[2][AT(m - 1, i)]; R->tv = c->t[2][AT(0, i)];
            L->tp = c->t[3][AT(m - 1, i)]; R->tp = c->t[3][AT(0, i)];
            L->trho = c->t[0][AT(m - 1, i)]; R->trho = c->t[0][AT(0, i)];
            break;
        }
    }
}

/* Resolve per-face codes the way the reference's serial loop leaves its return
 * value: the code of the last failing face in loop order wins. */
static int orc_last_code(const unsigned char *code, size_t count)
{
    int r = 0;
    for (size_t q = 0; q < count; ++q)
        if (code[q])
            r = code[q];
    return r;
}

/* flux_generator_x, src/flux_calc/flux_generator_x.c:31-165. */
static int orc_flux_x(orc2d *c, double *const cur[5], double tau, int transversal)
{
    const int m = c->m, n = c->n;
    const double hh = 0.5 * c->hx;
    int i;
    (void)hh;
#pragma omp parallel for schedule(static)
    for (i = 0; i < n; ++i)
        for (int j = 0; j <= m; ++j) {
            orc_side L, R;
            if (j) {
                size_t a = AT(j - 1, i);
                L.drho = c->s[0][a]; L.du = c->s[1][a]; L.dv = c->s[2][a]; L.dp = c->s[3][a];
                L.rho = cur[0][a] + 0.5 * c->hx * c->s[0][a];
                L.u = cur[1][a] + 0.5 * c->hx * c->s[1][a];
                L.v = cur[2][a] + 0.5 * c->hx * c->s[2][a];
                L.p = cur[3][a] + 0.5 * c->hx * c->s[3][a];
            } else {
                const orc_ghost *g = &c->gL[i];
                L.drho = g->srho; L.du = g->su; L.dv = g->sv; L.dp = g->sp;
                L.rho = g->rho + 0.5 * c->hx * g->srho;
                L.u = g->u + 0.5 * c->hx * g->su;
                L.v = g->v + 0.5 * c->hx * g->sv;
                L.p = g->p + 0.5 * c->hx * g->sp;
            }
            if (j < m) {
                size_t a = AT(j, i);
                R.drho = c->s[0][a]; R.du = c->s[1][a]; R.dv = c->s[2][a]; R.dp = c->s[3][a];
                R.rho = cur[0][a] - 0.5 * c->hx * c->s[0][a];
                R.u = cur[1][a] - 0.5 * c->hx * c->s[1][a];
                R.v = cur[2][a] - 0.5 * c->hx * c->s[2][a];
                R.p = cur[3][a] - 0.5 * c->hx * c->s[3][a];
            } else {
                const orc_ghost *g = &c->gR[i];
                R.drho = g->srho; R.du = g->su; R.dv = g->sv; R.dp = g->sp;
                R.rho = g->rho - 0.5 * c->hx * g->srho;
                R.u = g->u - 0.5 * c->hx * g->su;
                R.v = g->v - 0.5 * c->hx * g->sv;
                R.p = g->p - 0.5 * c->hx * g->sp;
            }
            if (transversal) {
                if (j) {
                    size_t a = AT(j - 1, i);
                    L.trho = c->t[0][a]; L.tu = c->t[1][a]; L.tv = c->t[2][a]; L.tp = c->t[3][a];
                } else {
                    const orc_ghost *g = &c->gL[i];
                    L.trho = g->trho; L.tu = g->tu; L.tv = g->tv; L.tp = g->tp;
                }
                if (j < m) {
                    size_t a = AT(j, i);
                    R.trho = c->t[0][a]; R.tu = c->t[1][a]; R.tv = c->t[2][a]; R.tp = c->t[3][a];
                } else {
                    const orc_ghost *g = &c->gR[i];
                    R.trho = g->trho; R.tu = g->tu; R.tv = g->tv; R.tp = g->tp;
                }
            } else {
                L.trho = L.tu = L.tv = L.tp = 0.0;
                R.trho = R.tu = R.tv = R.tp = 0.0;
            }
            int code = orc_ifvar_check2(&L, &R, c->eps) ? 1 : 0;
            double out[8];
            if (orc_grp2d_flux_one(1.0, 0.0, c->gamma, L, R, tau, c->eps, out, NULL, c->g2d))
                code = 2;
            size_t f = AT(j, i);
            for (int k = 0; k < 4; ++k) {
                c->F[k][f] = out[k];
                c->Ix[k][f] = out[4 + k];
            }
            c->cx[(size_t)i * (m + 1) + j] = (unsigned char)code;
        }
    return orc_last_code(c->cx, (size_t)n * (m + 1));
}

/* flux_generator_y, src/flux_calc/flux_generator_y.c:31-165 (tangential
 * derivatives of the y-faces are the negated x-slopes). */
static int orc_flux_y(orc2d *c, double *const cur[5], double tau, int transversal)
{
    const int m = c->m, n = c->n;
    int j;
#pragma omp parallel for schedule(static)
    for (j = 0; j < m; ++j)
        for (int i = 0; i <= n; ++i) {
            orc_side D, U;
            if (i) {
                size_t a = AT(j, i - 1);
                D.drho = c->t[0][a]; D.du = c->t[1][a]; D.dv = c->t[2][a]; D.dp = c->t[3][a];
                D.rho = cur[0][a] + 0.5 * c->hy * c->t[0][a];
                D.u = cur[1][a] + 0.5 * c->hy * c->t[1][a];
                D.v = cur[2][a] + 0.5 * c->hy * c->t[2][a];
                D.p = cur[3][a] + 0.5 * c->hy * c->t[3][a];
            } else {
                const orc_ghost *g = &c->gD[j];
                D.drho = g->trho; D.du = g->tu; D.dv = g->tv; D.dp = g->tp;
                D.rho = g->rho + 0.5 * c->hy * g->trho;
                D.u = g->u + 0.5 * c->hy * g->tu;
                D.v = g->v + 0.5 * c->hy * g->tv;
                D.p = g->p + 0.5 * c->hy * g->tp;
            }
            if (i < n) {
                size_t a = AT(j, i);
                U.drho = c->t[0][a]; U.du = c->t[1][a]; U.dv = c->t[2][a]; U.dp = c->t[3][a];
                U.rho = cur[0][a] - 0.5 * c->hy * c->t[0][a];
                U.u = cur[1][a] - 0.5 * c->hy * c->t[1][a];
                U.v = cur[2][a] - 0.5 * c->hy * c->t[2][a];
                U.p = cur[3][a] - 0.5 * c->hy * c->t[3][a];
            } else {
                const orc_ghost *g = &c->gU[j];
                U.drho = g->trho; U.du = g->tu; U.dv = g->tv; U.dp = g->tp;
                U.rho = g->rho - 0.5 * c->hy * g->trho;
                U.u = g->u - 0.5 * c->hy * g->tu;
                U.v = g->v - 0.5 * c->hy * g->tv;
                U.p = g->p - 0.5 * c->hy * g->tp;
            }
            if (transversal) {
                if (i) {
                    size_t a = AT(j, i - 1);
                    D.trho = -c->s[0][a]; D.tu = -c->s[1][a]; D.tv = -c->s[2][a]; D.tp = -c->s[3][a];
                } else {
                    const orc_ghost *g = &c->gD[j];
                    D.trho = -g->srho; D.tu = -g->su; D.tv = -g->sv; D.tp = -g->sp;
                }
                if (i < n) {
                    size_t a = AT(j, i);
                    U.trho = -c->s[0][a]; U.tu = -c->s[1][a]; U.tv = -c->s[2][a]; U.tp = -c->s[3][a];
                } else {
                    const orc_ghost *g = &c->gU[j];
                    U.trho = -g->srho; U.tu = -g->su; U.tv = -g->sv; U.tp = -g->sp;
                }
            } else {
                D.trho = D.tu = D.tv = D.tp = -0.0;
                U.trho = U.tu = U.tv = U.tp = -0.0;
            }
            int code = orc_ifvar_check2(&D, &U, c->eps) ? 1 : 0;
            double out[8];
            if (orc_grp2d_flux_one(0.0, 1.0, c->gamma, D, U, tau, c->eps, out, NULL, c->g2d))
                code = 2;
            size_t f = ATY(j, i);
            for (int k = 0; k < 4; ++k) {
                c->G[k][f] = out[k];
                c->Iy[k][f] = out[4 + k];
            }
            c->cy[f] = (unsigned char)code;
        }
    return orc_last_code(c->cy, (size_t)m * (n + 1));
}

static void orc_free2d(orc2d *c)
{
    for (int k = 0; k < 4; ++k) {
        free(c->s[k]); free(c->t[k]);
        free(c->F[k]); free(c->Ix[k]);
        free(c->G[k]); free(c->Iy[k]);
    }
    free(c->cx); free(c->cy);
    free(c->gL); free(c->gR); free(c->gD); free(c->gU);
}

/*
 * The 2D time loops: GRP_solver_2D_EUL_source
 * (src/finite_volume/grp_solver_2D_EUL_source.c:75-338) and
 * GRP_solver_2D_split_EUL_source (grp_solver_2D_split_EUL_source.c:75-379),
 * including plot snapshots (:155-174), the CFL time step taken from CV[0]
 * (:180-205), the error reactions (stop after the step vs. abort) and the
 * values written back on exit (:292-300).
 */
int orc_run_2d(int m, int n, double *rho, double *u, double *v, double *p, double *E,
               const double *cfg_in, int ncfg, int split, int threads,
               const double *plot_times, int nplot_in, double *snaps, int *nsnap_out,
               double *info)
{
    double cfg[ORC_NCONF];
    int k, q;
    for (q = 0; q < ORC_NCONF; ++q)
        cfg[q] = q < ncfg ? cfg_in[q] : INFINITY;
#ifdef _OPENMP
    if (threads > 0)
        omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const double t_all = cfg[1], eps = cfg[4], gamma = cfg[6], CFL = cfg[7];
    const int N = (int)cfg[5];
    const double h_x = cfg[10], h_y = cfg[11];
    double tau = cfg[16];

    int N_plot = (plot_times && nplot_in > 0) ? nplot_in + 2 : 2;
    double *time_plot = (double *)malloc(N_plot * sizeof(double));
    time_plot[0] = 0.0;
    time_plot[N_plot - 1] = t_all;
    for (q = 0; q < N_plot - 2; ++q)
        time_plot[q + 1] = plot_times[q];
    const int N_T = N_plot < 5 ? N_plot : 5;

    orc2d c;
    memset(&c, 0, sizeof(c));
    c.m = m; c.n = n; c.gamma = gamma; c.eps = eps; c.hx = h_x; c.hy = h_y; c.alpha = cfg[41];
    c.bx = (int)cfg[17]; c.by = (int)cfg[18];
    /* config[301] (unused by the reference) selects the genuinely-2D GRP solver
       that flux_solver.c:189 has as its commented-out alternative */
    c.g2d = cfg[301] == 1.0;
    const size_t mn = (size_t)m * n;
    for (k = 0; k < N_T; ++k)
        for (q = 0; q < 5; ++q)
            c.snap[k][q] = (double *)malloc(mn * sizeof(double));
    for (q = 0; q < 4; ++q) {
        c.s[q] = (double *)calloc(mn, sizeof(double));
        c.t[q] = (double *)calloc(mn, sizeof(double));
        c.F[q] = (double *)malloc((size_t)(m + 1) * n * sizeof(double));
        c.Ix[q] = (double *)malloc((size_t)(m + 1) * n * sizeof(double));
        c.G[q] = (double *)malloc((size_t)m * (n + 1) * sizeof(double));
        c.Iy[q] = (double *)malloc((size_t)m * (n + 1) * sizeof(double));
    }
    c.cx = (unsigned char *)calloc((size_t)(m + 1) * n, 1);
    c.cy = (unsigned char *)calloc((size_t)m * (n + 1), 1);
    c.gL = (orc_ghost *)calloc(n, sizeof(orc_ghost));
    c.gR = (orc_ghost *)calloc(n, sizeof(orc_ghost));
    c.gD = (orc_ghost *)calloc(m, sizeof(orc_ghost));
    c.gU = (orc_ghost *)calloc(m, sizeof(orc_ghost));

    /* initial data and E exactly as the 2D driver builds them (hydrocode.c:245-254) */
    for (size_t a = 0; a < mn; ++a) {
        c.snap[0][0][a] = rho[a];
        c.snap[0][1][a] = u[a];
        c.snap[0][2][a] = v[a];
        c.snap[0][3][a] = p[a];
        double e = 0.5 * u[a] * u[a] + p[a] / (gamma - 1.0) / rho[a];
        e += 0.5 * v[a] * v[a];
        c.snap[0][4][a] = e;
    }

    int nt = 0, nt_plot = 0, stop_t = 0, find_x = 0, find_y = 0, DS = 1;
    double time_c = 0.0, cpu_sum = 0.0, half_tau = 0.0, nu = 0.0, mu = 0.0, half_nu = 0.0;
    double *cpu_time = (double *)calloc(N_T, sizeof(double));
    double t_start = wall_clock();

    for (k = 1; k <= N; split ? (DS ? k : ++k) : ++k) {
        double tic = wall_clock();
        if (time_c >= time_plot[nt_plot] && nt_plot < (N_plot - 1)) {
            nt_plot++;
            if (nt < (N_T - 1)) {
                for (q = 0; q < 5; ++q)
                    memcpy(c.snap[nt + 1][q], c.snap[nt][q], mn * sizeof(double));
                nt++;
            }
        }
        double *cur[5] = {c.snap[nt][0], c.snap[nt][1], c.snap[nt][2], c.snap[nt][3], c.snap[nt][4]};
        double *ini[5] = {c.snap[0][0], c.snap[0][1], c.snap[0][2], c.snap[0][3], c.snap[0][4]};

        if (!split || DS) {
            double h_S_max = INFINITY;
            for (size_t a = 0; a < mn; ++a) {
                double cc = sqrt(gamma * ini[3][a] / ini[0][a]);
                double sigma = fabs(cc) + fabs(ini[1][a]) + fabs(ini[2][a]);
                h_S_max = fmin(h_S_max, fmin(h_x, h_y) / sigma);
            }
            if (isfinite(t_all) || !isfinite(cfg[16]) || cfg[16] <= 0.0) {
                tau = CFL * h_S_max;
                if (tau < eps)
                    stop_t = 1;
                else if ((time_c + tau) > (t_all - eps))
                    tau = t_all - time_c;
                else if (!isfinite(tau))
                    goto done;
            }
            if (split) {
                half_tau = tau * 0.5;
                half_nu = half_tau / h_x;
                mu = tau / h_y;
            } else {
                nu = tau / h_x;
                mu = tau / h_y;
            }
        }

        if (!split) {
            if (!orc_bc_values_x(&c, cur, ini, find_x))
                goto done;
            orc_limit_x(&c, cur, find_x);
            find_x = 1;
            if (!orc_bc_values_y(&c, cur, ini, find_y))
                goto done;
            orc_limit_y(&c, cur, find_y);
            find_y = 1;
            int fe = orc_flux_x(&c, cur, tau, 1);
            if (fe == 1)
                goto done;
            else if (fe == 2)
                stop_t = 1;
            fe = orc_flux_y(&c, cur, tau, 1);
            if (fe == 1)
                goto done;
            else if (fe == 2)
                stop_t = 1;
            int j, i;
            int upd_bad = 0;
#pragma omp parallel for private(i) reduction(| : upd_bad) schedule(static)
            for (j = 0; j < m; ++j)
                for (i = 0; i < n; ++i) {
                    size_t a = AT(j, i), fx0 = AT(j, i), fx1 = AT(j + 1, i), fy0 = ATY(j, i), fy1 = ATY(j, i + 1);
                    double r = cur[0][a];
                    double mom_x = r * cur[1][a] - nu * (c.F[1][fx1] - c.F[1][fx0]) - mu * (c.G[1][fy1] - c.G[1][fy0]);
                    double mom_y = r * cur[2][a] - nu * (c.F[2][fx1] - c.F[2][fx0]) - mu * (c.G[2][fy1] - c.G[2][fy0]);
                    double ene = r * cur[4][a] - nu * (c.F[3][fx1] - c.F[3][fx0]) - mu * (c.G[3][fy1] - c.G[3][fy0]);
                    r += -nu * (c.F[0][fx1] - c.F[0][fx0]) - mu * (c.G[0][fy1] - c.G[0][fy0]);
                    cur[0][a] = r;
                    cur[1][a] = mom_x / r;
                    cur[2][a] = mom_y / r;
                    cur[4][a] = ene / r;
                    cur[3][a] = (ene - 0.5 * mom_x * cur[1][a] - 0.5 * mom_y * cur[2][a]) * (gamma - 1.0);
                    if (cur[3][a] < eps || r < eps)
                        upd_bad = 1;
                    for (q = 0; q < 4; ++q) {
                        c.s[q][a] = (c.Ix[q][fx1] - c.Ix[q][fx0]) / h_x;
                        c.t[q][a] = (c.Iy[q][fy1] - c.Iy[q][fy0]) / h_y;
                    }
                }
            if (upd_bad)
                stop_t = 1;
            time_c += tau;
            if (stop_t || time_c > (t_all - eps) || !isfinite(time_c))
                break;
        } else {
            if (!orc_bc_values_x(&c, cur, ini, find_x))
                goto done;
            orc_limit_x(&c, cur, find_x);
            find_x = 1;
            int fe = orc_flux_x(&c, cur, half_tau, 0);
            if (fe == 1)
                goto done;
            else if (fe == 2)
                stop_t = 1;
            int j, i;
            int upd_bad = 0;
#pragma omp parallel for private(i) reduction(| : upd_bad) schedule(static)
            for (j = 0; j < m; ++j)
                for (i = 0; i < n; ++i) {
                    size_t a = AT(j, i), fx0 = AT(j, i), fx1 = AT(j + 1, i);
                    double r = cur[0][a];
                    double mom_x = r * cur[1][a] - half_nu * (c.F[1][fx1] - c.F[1][fx0]);
                    double mom_y = r * cur[2][a] - half_nu * (c.F[2][fx1] - c.F[2][fx0]);
                    double ene = r * cur[4][a] - half_nu * (c.F[3][fx1] - c.F[3][fx0]);
                    r += -half_nu * (c.F[0][fx1] - c.F[0][fx0]);
                    cur[0][a] = r;
                    cur[1][a] = mom_x / r;
                    cur[2][a] = mom_y / r;
                    cur[4][a] = ene / r;
                    cur[3][a] = (ene - 0.5 * mom_x * cur[1][a] - 0.5 * mom_y * cur[2][a]) * (gamma - 1.0);
                    if (cur[3][a] < eps || r < eps)
                        upd_bad = 1;
                    for (q = 0; q < 4; ++q)
                        c.s[q][a] = (c.Ix[q][fx1] - c.Ix[q][fx0]) / h_x;
                }
            if (upd_bad)
                stop_t = 1;
            if (stop_t)
                break;
            if (DS) {
                if (!orc_bc_values_y(&c, cur, ini, find_y))
                    goto done;
                orc_limit_y(&c, cur, find_y);
                find_y = 1;
                fe = orc_flux_y(&c, cur, tau, 0);
                if (fe == 1)
                    goto done;
                else if (fe == 2)
                    stop_t = 1;
                upd_bad = 0;
#pragma omp parallel for private(i) reduction(| : upd_bad) schedule(static)
                for (j = 0; j < m; ++j)
                    for (i = 0; i < n; ++i) {
                        size_t a = AT(j, i), fy0 = ATY(j, i), fy1 = ATY(j, i + 1);
                        double r = cur[0][a];
                        double mom_x = r * cur[1][a] - mu * (c.G[1][fy1] - c.G[1][fy0]);
                        double mom_y = r * cur[2][a] - mu * (c.G[2][fy1] - c.G[2][fy0]);
                        double ene = r * cur[4][a] - mu * (c.G[3][fy1] - c.G[3][fy0]);
                        r += -mu * (c.G[0][fy1] - c.G[0][fy0]);
                        cur[0][a] = r;
                        cur[1][a] = mom_x / r;
                        cur[2][a] = mom_y / r;
                        cur[4][a] = ene / r;
                        cur[3][a] = (ene - 0.5 * mom_x * cur[1][a] - 0.5 * mom_y * cur[2][a]) * (gamma - 1.0);
                        if (cur[3][a] < eps || r < eps)
                            upd_bad = 1;
                        for (q = 0; q < 4; ++q)
                            c.t[q][a] = (c.Iy[q][fy1] - c.Iy[q][fy0]) / h_y;
                    }
                if (upd_bad)
                    stop_t = 1;
                time_c += tau;
            }
            if (stop_t || time_c > (t_all - eps) || !isfinite(time_c))
                break;
            DS = DS ? 0 : 1;
        }
        double toc = wall_clock();
        cpu_sum += toc - tic;
        cpu_time[nt] = cpu_sum;
    }
done:;
    double t_end = wall_clock();
    double k_out = (double)k;
    N_plot = nt + 1;
    if (isfinite(time_c))
        time_plot[nt] = time_c;
    else if (isfinite(t_all))
        time_plot[nt] = t_all;
    else if (isfinite(tau))
        time_plot[nt] = k * tau;

    for (size_t a = 0; a < mn; ++a) {
        rho[a] = c.snap[nt][0][a];
        u[a] = c.snap[nt][1][a];
        v[a] = c.snap[nt][2][a];
        p[a] = c.snap[nt][3][a];
        if (E)
            E[a] = c.snap[nt][4][a];
    }
    if (snaps)
        for (k = 0; k < N_plot; ++k)
            for (q = 0; q < 5; ++q)
                memcpy(snaps + ((size_t)k * 5 + q) * mn, c.snap[k][q], mn * sizeof(double));
    if (nsnap_out)
        *nsnap_out = N_plot;
    if (info) {
        info[0] = k_out;
        info[1] = time_plot[nt];
        info[2] = cpu_time[nt];
        info[3] = t_end - t_start;
    }
    for (k = 0; k < N_T; ++k)
        for (q = 0; q < 5; ++q)
            free(c.snap[k][q]);
    orc_free2d(&c);
    free(cpu_time);
    free(time_plot);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* 1D time loops                                                              */
/* ------------------------------------------------------------------------- */

/*
 * Godunov_solver_EUL_source (src/finite_volume/godunov_solver_EUL_source.c:27-230)
 * and GRP_solver_EUL_source (src/finite_volume/grp_solver_EUL_source.c:27-334),
 * with bound_cond_slope_limiter (src/inter_process/bound_cond_slope_limiter.c:30-136)
 * and minmod_limiter (slope_limiter.c:31-83).
 */
int orc_run_1d(int m, double *rho, double *u, double *p, double *E_out,
               const double *cfg_in, int ncfg, int order, double *info)
{
    double cfg[ORC_NCONF];
    int j, k, q;
    for (q = 0; q < ORC_NCONF; ++q)
        cfg[q] = q < ncfg ? cfg_in[q] : INFINITY;
    const double t_all = cfg[1], eps = cfg[4], gamma = cfg[6], CFL = cfg[7], h = cfg[10];
    const int N = (int)cfg[5];
    const int bound = (int)cfg[17];
    const double alpha = cfg[41];
    double tau = cfg[16];
    const int N_plot_in = 2;
    double time_plot[2] = {0.0, t_all};

    double *R[2], *Uv[2], *P[2], *Ev[2];
    for (k = 0; k < 2; ++k) {
        R[k] = (double *)malloc(m * sizeof(double));
        Uv[k] = (double *)malloc(m * sizeof(double));
        P[k] = (double *)malloc(m * sizeof(double));
        Ev[k] = (double *)malloc(m * sizeof(double));
    }
    for (j = 0; j < m; ++j) {
        R[0][j] = rho[j];
        Uv[0][j] = u[j];
        P[0][j] = p[j];
        Ev[0][j] = 0.5 * u[j] * u[j] + p[j] / (gamma - 1.0) / rho[j];
    }
    double *s_rho = (double *)calloc(m, sizeof(double)), *s_u = (double *)calloc(m, sizeof(double)),
           *s_p = (double *)calloc(m, sizeof(double));
    double *mid[3], *dire[3], *F[3];
    for (q = 0; q < 3; ++q) {
        mid[q] = (double *)malloc((m + 1) * sizeof(double));
        dire[q] = (double *)malloc((m + 1) * sizeof(double));
        F[q] = (double *)malloc((m + 1) * sizeof(double));
    }
    double gL[6] = {0, 0, 0, 0, 0, 0}, gR[6] = {0, 0, 0, 0, 0, 0}; /* rho,u,p, srho,su,sp */
    int nt = 0, stop_t = 0, found = 0;
    double time_c = 0.0, cpu_sum = 0.0, cpu_time[2] = {0.0, 0.0};
    double t_start = wall_clock();

    for (k = 1; k <= N; ++k) {
        double tic = wall_clock();
        if (time_c >= time_plot[nt] && nt < (N_plot_in - 1)) {
            for (j = 0; j < m; ++j) {
                R[nt + 1][j] = R[nt][j];
                Uv[nt + 1][j] = Uv[nt][j];
                Ev[nt + 1][j] = Ev[nt][j];
                P[nt + 1][j] = P[nt][j];
            }
            nt++;
        }
        double *r = R[nt], *uu = Uv[nt], *pp = P[nt], *ee = Ev[nt];
        double h_S_max = INFINITY;

        /* boundary values, bound_cond_slope_limiter.c:41-82 */
        switch (bound) {
        case -1:
            if (!found) {
                gL[1] = Uv[0][0]; gR[1] = Uv[0][m - 1];
                gL[2] = P[0][0]; gR[2] = P[0][m - 1];
                gL[0] = R[0][0]; gR[0] = R[0][m - 1];
            }
            break;
        case -2:
            gL[1] = -uu[0]; gR[1] = -uu[m - 1];
            gL[2] = pp[0]; gR[2] = pp[m - 1];
            gL[0] = r[0]; gR[0] = r[m - 1];
            break;
        case -4:
            gL[1] = uu[0]; gR[1] = uu[m - 1];
            gL[2] = pp[0]; gR[2] = pp[m - 1];
            gL[0] = r[0]; gR[0] = r[m - 1];
            break;
        case -7:
            gL[1] = uu[m - 1]; gR[1] = uu[0];
            gL[2] = pp[m - 1]; gR[2] = pp[0];
            gL[0] = r[m - 1]; gR[0] = r[0];
            break;
        case -24:
            gL[1] = -uu[0]; gR[1] = uu[m - 1];
            gL[2] = pp[0]; gR[2] = pp[m - 1];
            gL[0] = r[0]; gR[0] = r[m - 1];
            break;
        default:
            goto done1;
        }
        if (order == 2) {
            /* minmod_limiter on u, p, rho (slope_limiter.c:47-81) */
            double *sv[3] = {s_u, s_p, s_rho};
            double *Uq[3] = {uu, pp, r};
            double ULq[3] = {gL[1], gL[2], gL[0]}, URq[3] = {gR[1], gR[2], gR[0]};
            for (q = 0; q < 3; ++q)
                for (j = 0; j < m; ++j) {
                    double sL, sR;
                    if (j)
                        sL = (Uq[q][j] - Uq[q][j - 1]) / h;
                    else
                        sL = (Uq[q][j] - ULq[q]) / h;
                    if (j < m - 1)
                        sR = (Uq[q][j + 1] - Uq[q][j]) / h;
                    else
                        sR = (URq[q] - Uq[q][j]) / h;
                    if (found)
                        sv[q][j] = orc_minmod3(alpha * sL, alpha * sR, sv[q][j]);
                    else
                        sv[q][j] = orc_minmod2(sL, sR);
                }
            switch (bound) {
            case -2:
                gL[4] = s_u[0]; gR[4] = s_u[m - 1];
                break;
            case -7:
                gL[4] = s_u[m - 1]; gR[4] = s_u[0];
                gL[5] = s_p[m - 1]; gR[5] = s_p[0];
                gL[3] = s_rho[m - 1]; gR[3] = s_rho[0];
                break;
            case -24:
                gL[4] = s_u[0];
                break;
            }
        }
        found = 1;

        for (j = 0; j <= m; ++j) {
            double Ls[6], Rs[6];
            if (order == 1) {
                if (j) { Ls[0] = r[j - 1]; Ls[1] = uu[j - 1]; Ls[2] = pp[j - 1]; }
                else { Ls[0] = gL[0]; Ls[1] = gL[1]; Ls[2] = gL[2]; }
                if (j < m) { Rs[0] = r[j]; Rs[1] = uu[j]; Rs[2] = pp[j]; }
                else { Rs[0] = gR[0]; Rs[1] = gR[1]; Rs[2] = gR[2]; }
                /* the reference's interface structs start zero-filled and keep
                 * zero derivatives in the first-order scheme */
                Ls[3] = Ls[4] = Ls[5] = 0.0;
                Rs[3] = Rs[4] = Rs[5] = 0.0;
            } else {
                if (j) {
                    Ls[0] = r[j - 1] + 0.5 * h * s_rho[j - 1];
                    Ls[1] = uu[j - 1] + 0.5 * h * s_u[j - 1];
                    Ls[2] = pp[j - 1] + 0.5 * h * s_p[j - 1];
                } else {
                    Ls[0] = gL[0] + 0.5 * h * gL[3];
                    Ls[1] = gL[1] + 0.5 * h * gL[4];
                    Ls[2] = gL[2] + 0.5 * h * gL[5];
                }
                if (j < m) {
                    Rs[0] = r[j] - 0.5 * h * s_rho[j];
                    Rs[1] = uu[j] - 0.5 * h * s_u[j];
                    Rs[2] = pp[j] - 0.5 * h * s_p[j];
                } else {
                    /* the right ghost is reconstructed with a '+' in the reference
                     * (grp_solver_EUL_source.c:158-162) */
                    Rs[0] = gR[0] + 0.5 * h * gR[3];
                    Rs[1] = gR[1] + 0.5 * h * gR[4];
                    Rs[2] = gR[2] + 0.5 * h * gR[5];
                }
            }
            double cL = sqrt(gamma * Ls[2] / Ls[0]);
            double cR = sqrt(gamma * Rs[2] / Rs[0]);
            h_S_max = fmin(h_S_max, h / (fabs(Ls[1]) + fabs(cL)));
            h_S_max = fmin(h_S_max, h / (fabs(Rs[1]) + fabs(cR)));
            if (order == 2) {
                if (j) { Ls[4] = s_u[j - 1]; Ls[5] = s_p[j - 1]; Ls[3] = s_rho[j - 1]; }
                else { Ls[3] = gL[3]; Ls[4] = gL[4]; Ls[5] = gL[5]; }
                if (j < m) { Rs[4] = s_u[j]; Rs[5] = s_p[j]; Rs[3] = s_rho[j]; }
                else { Rs[3] = gR[3]; Rs[4] = gR[4]; Rs[5] = gR[5]; }
                /* ifvar_check dim 1 (fluid_var_check.c:21-36) aborts the run */
                if (Ls[2] < eps || Rs[2] < eps || Ls[0] < eps || Rs[0] < eps ||
                    !isfinite(Ls[5]) || !isfinite(Rs[5]) || !isfinite(Ls[4]) || !isfinite(Rs[4]) ||
                    !isfinite(Ls[3]) || !isfinite(Rs[3]))
                    goto done1;
            }
            double D[3], U[3];
            orc_grp1d_solve(gamma, Ls, Rs, eps, order == 1 ? INFINITY : eps, D, U);
            if (orc_star_dire_check1(U, D, eps))
                stop_t = 1;
            for (q = 0; q < 3; ++q) {
                mid[q][j] = U[q];
                dire[q][j] = D[q];
            }
            if (order == 1) {
                F[0][j] = U[0] * U[1];
                F[1][j] = F[0][j] * U[1] + U[2];
                F[2][j] = (gamma / (gamma - 1.0)) * U[2] + 0.5 * F[0][j] * U[1];
                F[2][j] = F[2][j] * U[1];
            }
        }

        if (isfinite(t_all) || !isfinite(cfg[16]) || cfg[16] <= 0.0) {
            tau = CFL * h_S_max;
            if (tau < eps)
                stop_t = 1;
            else if ((time_c + tau) > (t_all - eps))
                tau = t_all - time_c;
            else if (!isfinite(tau))
                goto done1;
        }
        double nu = tau / h;

        if (order == 2)
            for (j = 0; j <= m; ++j) {
                mid[0][j] += 0.5 * tau * dire[0][j];
                mid[1][j] += 0.5 * tau * dire[1][j];
                mid[2][j] += 0.5 * tau * dire[2][j];
                F[0][j] = mid[0][j] * mid[1][j];
                F[1][j] = F[0][j] * mid[1][j] + mid[2][j];
                F[2][j] = (gamma / (gamma - 1.0)) * mid[2][j] + 0.5 * F[0][j] * mid[1][j];
                F[2][j] = F[2][j] * mid[1][j];
                mid[0][j] += 0.5 * tau * dire[0][j];
                mid[1][j] += 0.5 * tau * dire[1][j];
                mid[2][j] += 0.5 * tau * dire[2][j];
            }

        for (j = 0; j < m; ++j) {
            double Mom = r[j] * uu[j] - nu * (F[1][j + 1] - F[1][j]);
            double Ene = r[j] * ee[j] - nu * (F[2][j + 1] - F[2][j]);
            r[j] = r[j] - nu * (F[0][j + 1] - F[0][j]);
            uu[j] = Mom / r[j];
            ee[j] = Ene / r[j];
            pp[j] = (Ene - 0.5 * Mom * uu[j]) * (gamma - 1.0);
            if (pp[j] < eps || r[j] < eps)
                stop_t = 1;
            if (order == 2) {
                s_u[j] = (mid[1][j + 1] - mid[1][j]) / h;
                s_p[j] = (mid[2][j + 1] - mid[2][j]) / h;
                s_rho[j] = (mid[0][j + 1] - mid[0][j]) / h;
            }
        }
        time_c += tau;
        if (stop_t || time_c > (t_all - eps) || !isfinite(time_c))
            break;
        double toc = wall_clock();
        cpu_sum += toc - tic;
        cpu_time[nt] = cpu_sum;
    }
done1:;
    double t_end = wall_clock();
    if (isfinite(time_c))
        time_plot[nt] = time_c;
    else if (isfinite(t_all))
        time_plot[nt] = t_all;
    else if (isfinite(tau))
        time_plot[nt] = k * tau;
    for (j = 0; j < m; ++j) {
        rho[j] = R[nt][j];
        u[j] = Uv[nt][j];
        p[j] = P[nt][j];
        if (E_out)
            E_out[j] = Ev[nt][j];
    }
    if (info) {
        info[0] = (double)k;
        info[1] = time_plot[nt];
        info[2] = cpu_time[nt];
        info[3] = t_end - t_start;
    }
    for (k = 0; k < 2; ++k) {
        free(R[k]); free(Uv[k]); free(P[k]); free(Ev[k]);
    }
    free(s_rho); free(s_u); free(s_p);
    for (q = 0; q < 3; ++q) {
        free(mid[q]); free(dire[q]); free(F[q]);
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* point-solver entry points (golden vectors)                                 */
/* ------------------------------------------------------------------------- */

/* ------------------------------------------------------------------------- */
/* 1D Lagrangian schemes                                                      */
/* ------------------------------------------------------------------------- */

/*
 * linear_GRP_solver_LAG, src/riemann_solver/linear_grp_solver_LAG.c:32-154
 * (Ben-Artzi & Falcovitz's Lagrangian GRP): Ls/Rs = rho, u, p and the
 * material derivatives t_rho, t_u, t_p.  D = (rho*_L, u, p, rho*_R)_t,
 * U = (rho*_L, u*, p*, rho*_R).  The 3-rarefaction branch uses the left
 * state's c_L, s_rho_L, s_p_L in its correction term (:128), as the
 * reference does.
 */
static void orc_lag_solve(double gL, double gR, const double Ls[6], const double Rs[6], double eps, double atc,
                          double D[4], double U[4])
{
    const double rho_L = Ls[0], u_L = Ls[1], p_L = Ls[2], s_rho_L = Ls[3], s_u_L = Ls[4], s_p_L = Ls[5];
    const double rho_R = Rs[0], u_R = Rs[1], p_R = Rs[2], s_rho_R = Rs[3], s_u_R = Rs[4], s_p_R = Rs[5];
    const double zetaL = (gL - 1.0) / (gL + 1.0);
    const double zetaR = (gR - 1.0) / (gR + 1.0);
    int CRW[2];
    double c_L = sqrt(gL * p_L / rho_L), c_R = sqrt(gR * p_R / rho_R);
    double g_L = rho_L * c_L, g_R = rho_R * c_R;
    double u_star, p_star, rho_star_L, rho_star_R, c_star_L, c_star_R, g_star_L, g_star_R, beta_star;
    double a_L, b_L, d_L, a_R, b_R, d_R, L_rho, L_u, L_p, A, B, W_L, W_R;

    orc_exact(gL, gR, u_L, u_R, p_L, p_R, c_L, c_R, eps, eps, 500, &u_star, &p_star, CRW, NULL);
    if (CRW[0]) {
        rho_star_L = rho_L * pow(p_star / p_L, 1.0 / gL);
        c_star_L = c_L * pow(p_star / p_L, 0.5 * (gL - 1.0) / gL);
    } else {
        rho_star_L = rho_L * (p_star + zetaL * p_L) / (p_L + zetaL * p_star);
        c_star_L = sqrt(gL * p_star / rho_star_L);
    }
    if (CRW[1]) {
        rho_star_R = rho_R * pow(p_star / p_R, 1.0 / gR);
        c_star_R = c_R * pow(p_star / p_R, 0.5 * (gR - 1.0) / gR);
    } else {
        rho_star_R = rho_R * (p_star + zetaR * p_R) / (p_R + zetaR * p_star);
        c_star_R = sqrt(gR * p_star / rho_star_R);
    }
    g_star_R = rho_star_R * c_star_R;
    g_star_L = rho_star_L * c_star_L;

    double dist = sqrt((u_L - u_R) * (u_L - u_R) + (p_L - p_R) * (p_L - p_R));
    if (dist < atc) { /* acoustic case (:83-91) */
        a_L = 1.0;
        b_L = 1.0 / g_star_L;
        d_L = -g_L * s_u_L - s_p_L;
        a_R = -1.0;
        b_R = 1.0 / g_star_R;
        d_R = -g_R * s_u_R + s_p_R;
    } else {
        if (CRW[0]) { /* 1-rarefaction (:95-102) */
            beta_star = g_star_L / g_L;
            a_L = 1.0;
            b_L = 1.0 / g_star_L;
            d_L = (s_u_L + s_p_L / g_L) + 1.0 / g_L / (3.0 * gL - 1.0) * (c_L * c_L * s_rho_L - s_p_L) *
                                              (pow(beta_star, (3.0 * gL - 1.0) / 2.0 / (gL + 1.0)) - 1.0);
            d_L = -1.0 * sqrt(g_L * g_star_L) * d_L;
        } else { /* 1-shock (:103-114) */
            W_L = (p_star - p_L) / (u_star - u_L);
            A = -0.5 / (p_star + zetaL * p_L);
            a_L = 2.0 + A * (p_star - p_L);
            b_L = -W_L / g_star_L / g_star_L - (a_L - 1.0) / W_L;
            L_rho = (p_star - p_L) / 2.0 / rho_L;
            B = 1.0 / (p_star - p_L) - zetaL * A;
            L_u = rho_L * (u_star - u_L) * (gL * p_L * B + 0.5) + W_L;
            L_p = 1.0 + B * (p_star - p_L);
            d_L = L_u * s_u_L - L_p * s_p_L - L_rho * s_rho_L;
        }
        if (CRW[1]) { /* 3-rarefaction (:116-123) */
            beta_star = g_star_R / g_R;
            a_R = -1.0;
            b_R = 1.0 / g_star_R;
            d_R = (s_u_R - s_p_R / g_R) + 1.0 / g_R / (3.0 * gR - 1.0) * (-c_L * c_L * s_rho_L + s_p_L) *
                                              (pow(beta_star, (3.0 * gR - 1.0) / 2.0 / (gR + 1.0)) - 1.0);
            d_R = -1.0 * sqrt(g_R * g_star_R) * d_R;
        } else { /* 3-shock (:124-135) */
            W_R = (p_star - p_R) / (u_star - u_R);
            A = -0.5 / (p_star + zetaR * p_R);
            a_R = -2.0 - A * (p_star - p_R);
            b_R = W_R / g_star_R / g_star_R - (a_R + 1.0) / W_R;
            L_rho = (p_star - p_R) / 2.0 / rho_R;
            B = 1.0 / (p_star - p_R) - zetaR * A;
            L_u = rho_R * (u_R - u_star) * (gR * p_R * B + 0.5) - W_R;
            L_p = 1.0 + B * (p_star - p_R);
            d_R = L_u * s_u_R + L_p * s_p_R + L_rho * s_rho_R;
        }
    }
    U[1] = u_star;
    U[2] = p_star;
    U[0] = rho_star_L;
    U[3] = rho_star_R;
    D[1] = (d_L * b_R - d_R * b_L) / (a_L * b_R - a_R * b_L);
    D[2] = (d_L * a_R - d_R * a_L) / (b_L * a_R - b_R * a_L);
    D[0] = D[2] / c_star_L / c_star_L;
    D[3] = D[2] / c_star_R / c_star_R;
}

/* minmod_limiter on a moving grid (src/inter_process/slope_limiter.c:31-83,
 * NO_h true): the differences are over half the distance of the neighbours'
 * centres, the ghost cells having lengths HL, HR. */
static void orc_minmod_moving(int m, int found, double alpha, double *s, const double *U, double UL, double UR,
                              double HL, double HR, const double *X)
{
    for (int j = 0; j < m; ++j) {
        double h, sL, sR;
        if (j) {
            h = 0.5 * (X[j + 1] - X[j - 1]);
            sL = (U[j] - U[j - 1]) / h;
        } else {
            h = 0.5 * (X[j + 1] - X[j] + HL);
            sL = (U[j] - UL) / h;
        }
        if (j < m - 1) {
            h = 0.5 * (X[j + 2] - X[j]);
            sR = (U[j + 1] - U[j]) / h;
        } else {
            h = 0.5 * (X[j + 1] - X[j] + HR);
            sR = (UR - U[j]) / h;
        }
        s[j] = found ? orc_minmod3(alpha * sL, alpha * sR, s[j]) : orc_minmod2(sL, sR);
    }
}

/*
 * Godunov_solver_LAG_source (src/finite_volume/godunov_solver_LAG_source.c:28-243,
 * order 1) and GRP_solver_LAG_source (src/finite_volume/grp_solver_LAG_source.c:28-355,
 * order 2): cells carry fixed masses, the interfaces move with the star
 * velocity, the time step is min(CFL h/c, 1.01 tau_prev).  Boundary values,
 * ghost-cell lengths and slopes as bound_cond_slope_limiter with moving
 * coordinates (src/inter_process/bound_cond_slope_limiter.c:30-136); the
 * GRP checks run with config[8] = 1 as the 1D driver sets it for LAG
 * (src/hydrocode_1D/hydrocode.c:238).  Two stored states (no plot times).
 * X_out: the final m+1 node coordinates (may be NULL).
 */
int orc_run_1d_lag(int m, double *rho, double *u, double *p, double *E_out, double *X_out,
                   const double *cfg_in, int ncfg, int order, double *info)
{
    double cfg[ORC_NCONF];
    int j, k, q;
    for (q = 0; q < ORC_NCONF; ++q)
        cfg[q] = q < ncfg ? cfg_in[q] : INFINITY;
    const double t_all = cfg[1], eps = cfg[4], gamma = cfg[6], CFL = cfg[7], h = cfg[10];
    const int N = (int)cfg[5];
    const int bound = (int)cfg[17];
    const double alpha = cfg[41];
    const double C_m = 1.01;
    double tau = cfg[16];
    double time_plot[2] = {0.0, t_all};

    double *R[2], *Uv[2], *P[2], *Ev[2], *X[2];
    for (k = 0; k < 2; ++k) {
        R[k] = (double *)malloc(m * sizeof(double));
        Uv[k] = (double *)malloc(m * sizeof(double));
        P[k] = (double *)malloc(m * sizeof(double));
        Ev[k] = (double *)malloc(m * sizeof(double));
        X[k] = (double *)malloc((m + 1) * sizeof(double));
    }
    for (j = 0; j <= m; ++j)
        X[0][j] = h * j;
    for (j = 0; j < m; ++j) {
        R[0][j] = rho[j];
        Uv[0][j] = u[j];
        P[0][j] = p[j];
        Ev[0][j] = 0.5 * u[j] * u[j] + p[j] / (gamma - 1.0) / rho[j];
    }
    double *MASS = (double *)malloc(m * sizeof(double));
    for (j = 0; j < m; ++j)
        MASS[j] = h * R[0][j];
    double *s_rho = (double *)calloc(m, sizeof(double)), *s_u = (double *)calloc(m, sizeof(double)),
           *s_p = (double *)calloc(m, sizeof(double));
    double *U_F = (double *)malloc((m + 1) * sizeof(double)), *P_F = (double *)malloc((m + 1) * sizeof(double));
    double *U_next = (double *)malloc((m + 1) * sizeof(double)), *P_next = (double *)malloc((m + 1) * sizeof(double));
    double *RL_next = (double *)malloc((m + 1) * sizeof(double)), *RR_next = (double *)malloc((m + 1) * sizeof(double));
    double *U_t = (double *)malloc((m + 1) * sizeof(double)), *P_t = (double *)malloc((m + 1) * sizeof(double));
    double *RL_t = (double *)malloc((m + 1) * sizeof(double)), *RR_t = (double *)malloc((m + 1) * sizeof(double));
    /* ghost cells: rho, u, p, srho, su, sp, H (the reference's b_f_var starts with zero slopes, H = h) */
    double gL[7] = {0, 0, 0, 0, 0, 0, h}, gR[7] = {0, 0, 0, 0, 0, 0, h};
    int nt = 0, stop_t = 0, found = 0;
    double time_c = 0.0, cpu_sum = 0.0, cpu_time[2] = {0.0, 0.0};
    double t_start = wall_clock();

    for (k = 1; k <= N; ++k) {
        double tic = wall_clock();
        if (time_c >= time_plot[nt] && nt < 1) {
            for (j = 0; j < m; ++j) {
                R[nt + 1][j] = R[nt][j];
                Uv[nt + 1][j] = Uv[nt][j];
                Ev[nt + 1][j] = Ev[nt][j];
                P[nt + 1][j] = P[nt][j];
                X[nt + 1][j] = X[nt][j];
            }
            X[nt + 1][m] = X[nt][m];
            nt++;
        }
        double *r = R[nt], *uu = Uv[nt], *pp = P[nt], *ee = Ev[nt], *x = X[nt];
        double h_S_max = INFINITY;

        /* boundary values and ghost lengths (bound_cond_slope_limiter.c:41-106) */
        switch (bound) {
        case -1:
            if (!found) {
                gL[1] = Uv[0][0]; gR[1] = Uv[0][m - 1];
                gL[2] = P[0][0]; gR[2] = P[0][m - 1];
                gL[0] = R[0][0]; gR[0] = R[0][m - 1];
            }
            gL[6] = h; gR[6] = h;
            break;
        case -2:
            gL[1] = -uu[0]; gR[1] = -uu[m - 1];
            gL[2] = pp[0]; gR[2] = pp[m - 1];
            gL[0] = r[0]; gR[0] = r[m - 1];
            gL[6] = x[1] - x[0]; gR[6] = x[m] - x[m - 1];
            break;
        case -4:
            gL[1] = uu[0]; gR[1] = uu[m - 1];
            gL[2] = pp[0]; gR[2] = pp[m - 1];
            gL[0] = r[0]; gR[0] = r[m - 1];
            gL[6] = x[1] - x[0]; gR[6] = x[m] - x[m - 1];
            break;
        case -7:
            gL[1] = uu[m - 1]; gR[1] = uu[0];
            gL[2] = pp[m - 1]; gR[2] = pp[0];
            gL[0] = r[m - 1]; gR[0] = r[0];
            gL[6] = x[m] - x[m - 1]; gR[6] = x[1] - x[0];
            break;
        case -24:
            gL[1] = -uu[0]; gR[1] = uu[m - 1];
            gL[2] = pp[0]; gR[2] = pp[m - 1];
            gL[0] = r[0]; gR[0] = r[m - 1];
            gL[6] = x[1] - x[0]; gR[6] = x[m] - x[m - 1];
            break;
        default:
            goto done_lag;
        }
        if (order == 2) {
            orc_minmod_moving(m, found, alpha, s_u, uu, gL[1], gR[1], gL[6], gR[6], x);
            orc_minmod_moving(m, found, alpha, s_p, pp, gL[2], gR[2], gL[6], gR[6], x);
            orc_minmod_moving(m, found, alpha, s_rho, r, gL[0], gR[0], gL[6], gR[6], x);
            switch (bound) {
            case -2:
                gL[4] = s_u[0]; gR[4] = s_u[m - 1];
                break;
            case -7:
                gL[4] = s_u[m - 1]; gR[4] = s_u[0];
                gL[5] = s_p[m - 1]; gR[5] = s_p[0];
                gL[3] = s_rho[m - 1]; gR[3] = s_rho[0];
                break;
            case -24:
                gL[4] = s_u[0];
                break;
            }
        }
        found = 1;

        for (j = 0; j <= m; ++j) {
            double Ls[6], Rs[6], h_L, h_R;
            const double *cL_ = j ? NULL : gL, *cR_ = j < m ? NULL : gR;  /* ghost or cell */
            h_L = j ? x[j] - x[j - 1] : gL[6];
            h_R = j < m ? x[j + 1] - x[j] : gR[6];
            if (order == 1) { /* cell values (godunov_solver_LAG_source.c:103-128) */
                Ls[0] = cL_ ? cL_[0] : r[j - 1];
                Ls[1] = cL_ ? cL_[1] : uu[j - 1];
                Ls[2] = cL_ ? cL_[2] : pp[j - 1];
                Rs[0] = cR_ ? cR_[0] : r[j];
                Rs[1] = cR_ ? cR_[1] : uu[j];
                Rs[2] = cR_ ? cR_[2] : pp[j];
            } else { /* grp_solver_LAG_source.c:137-162; the right ghost with '+' as there */
                if (j) {
                    Ls[0] = r[j - 1] + 0.5 * h_L * s_rho[j - 1];
                    Ls[1] = uu[j - 1] + 0.5 * h_L * s_u[j - 1];
                    Ls[2] = pp[j - 1] + 0.5 * h_L * s_p[j - 1];
                } else {
                    Ls[0] = gL[0] + 0.5 * h_L * gL[3];
                    Ls[1] = gL[1] + 0.5 * h_L * gL[4];
                    Ls[2] = gL[2] + 0.5 * h_L * gL[5];
                }
                if (j < m) {
                    Rs[0] = r[j] - 0.5 * h_R * s_rho[j];
                    Rs[1] = uu[j] - 0.5 * h_R * s_u[j];
                    Rs[2] = pp[j] - 0.5 * h_R * s_p[j];
                } else {
                    Rs[0] = gR[0] + 0.5 * h_R * gR[3];
                    Rs[1] = gR[1] + 0.5 * h_R * gR[4];
                    Rs[2] = gR[2] + 0.5 * h_R * gR[5];
                }
            }
            double c_L = sqrt(gamma * Ls[2] / Ls[0]);
            double c_R = sqrt(gamma * Rs[2] / Rs[0]);
            h_S_max = fmin(h_S_max, h_L / c_L);
            h_S_max = fmin(h_S_max, h_R / c_R);
            if ((bound == -2 || bound == -24) && j == 0)
                h_S_max = fmin(h_S_max, h_L / (fabs(Ls[1]) + c_L));
            if (bound == -2 && j == m)
                h_S_max = fmin(h_S_max, h_R / (fabs(Rs[1]) + c_R));

            if (order == 1) { /* godunov_solver_LAG_source.c:137-152 */
                double us, ps;
                int crw[2];
                orc_exact(gamma, gamma, Ls[1], Rs[1], Ls[2], Rs[2], c_L, c_R, eps, eps, 500, &us, &ps, crw, NULL);
                if (ps < eps)
                    stop_t = 1;
                if (!isfinite(ps) || !isfinite(us))
                    stop_t = 1;
                U_F[j] = us;
                P_F[j] = ps;
                continue;
            }
            /* material derivatives (grp_solver_LAG_source.c:173-198) */
            double dL[3], dR[3]; /* rho, u, p */
            if (j) { dL[1] = s_u[j - 1]; dL[2] = s_p[j - 1]; dL[0] = s_rho[j - 1]; }
            else { dL[0] = gL[3]; dL[1] = gL[4]; dL[2] = gL[5]; }
            if (j < m) { dR[1] = s_u[j]; dR[2] = s_p[j]; dR[0] = s_rho[j]; }
            else { dR[0] = gR[3]; dR[1] = gR[4]; dR[2] = gR[5]; }
            /* ifvar_check dim 1 aborts the run (:199-203) */
            if (Ls[2] < eps || Rs[2] < eps || Ls[0] < eps || Rs[0] < eps || !isfinite(dL[2]) || !isfinite(dR[2]) ||
                !isfinite(dL[1]) || !isfinite(dR[1]) || !isfinite(dL[0]) || !isfinite(dR[0]))
                goto done_lag;
            Ls[4] = dL[1] / Ls[0];
            Ls[5] = dL[2] / Ls[0];
            Ls[3] = dL[0] / Ls[0];
            Rs[4] = dR[1] / Rs[0];
            Rs[5] = dR[2] / Rs[0];
            Rs[3] = dR[0] / Rs[0];
            double D[4], Ust[4];
            orc_lag_solve(gamma, gamma, Ls, Rs, eps, eps, D, Ust);
            /* star_dire_check dim 1 with config[8] = 1 (fluid_var_check.c:72-90) */
            if (Ust[2] < eps || Ust[0] < eps || Ust[3] < eps || !isfinite(Ust[1]) || !isfinite(Ust[2]) ||
                !isfinite(Ust[0]) || !isfinite(Ust[3]) || !isfinite(D[1]) || !isfinite(D[2]) || !isfinite(D[0]) ||
                !isfinite(D[3]))
                stop_t = 1;
            RL_next[j] = Ust[0];
            RR_next[j] = Ust[3];
            U_next[j] = Ust[1];
            P_next[j] = Ust[2];
            RL_t[j] = D[0];
            RR_t[j] = D[3];
            U_t[j] = D[1];
            P_t[j] = D[2];
        }

        if (isfinite(t_all) || !isfinite(cfg[16]) || cfg[16] <= 0.0) {
            tau = fmin(CFL * h_S_max, C_m * tau);
            if (tau < eps)
                stop_t = 1;
            else if ((time_c + tau) > (t_all - eps))
                tau = t_all - time_c;
            else if (!isfinite(tau))
                goto done_lag;
        }
        for (j = 0; j <= m; ++j) {
            if (order == 2) {
                U_F[j] = U_next[j] + 0.5 * tau * U_t[j];
                P_F[j] = P_next[j] + 0.5 * tau * P_t[j];
                RL_next[j] += tau * RL_t[j];
                RR_next[j] += tau * RR_t[j];
                U_next[j] += tau * U_t[j];
                P_next[j] += tau * P_t[j];
            }
            x[j] += tau * U_F[j];
        }
        for (j = 0; j < m; ++j) {
            r[j] = 1.0 / (1.0 / r[j] + tau / MASS[j] * (U_F[j + 1] - U_F[j]));
            uu[j] = uu[j] - tau / MASS[j] * (P_F[j + 1] - P_F[j]);
            ee[j] = ee[j] - tau / MASS[j] * (P_F[j + 1] * U_F[j + 1] - P_F[j] * U_F[j]);
            pp[j] = (ee[j] - 0.5 * uu[j] * uu[j]) * (gamma - 1.0) * r[j];
            if (pp[j] < eps || r[j] < eps)
                stop_t = 1;
            if (order == 2) {
                s_u[j] = (U_next[j + 1] - U_next[j]) / (x[j + 1] - x[j]);
                s_p[j] = (P_next[j + 1] - P_next[j]) / (x[j + 1] - x[j]);
                s_rho[j] = (RL_next[j + 1] - RR_next[j]) / (x[j + 1] - x[j]);
            }
        }
        time_c += tau;
        if (stop_t || time_c > (t_all - eps) || !isfinite(time_c))
            break;
        double toc = wall_clock();
        cpu_sum += toc - tic;
        cpu_time[nt] = cpu_sum;
    }
done_lag:;
    double t_end = wall_clock();
    if (isfinite(time_c))
        time_plot[nt] = time_c;
    else if (isfinite(t_all))
        time_plot[nt] = t_all;
    else if (isfinite(tau))
        time_plot[nt] = k * tau;
    for (j = 0; j < m; ++j) {
        rho[j] = R[nt][j];
        u[j] = Uv[nt][j];
        p[j] = P[nt][j];
        if (E_out)
            E_out[j] = Ev[nt][j];
    }
    if (X_out)
        for (j = 0; j <= m; ++j)
            X_out[j] = X[nt][j];
    if (info) {
        info[0] = (double)k;
        info[1] = time_plot[nt];
        info[2] = cpu_time[nt];
        info[3] = t_end - t_start;
    }
    for (k = 0; k < 2; ++k) {
        free(R[k]); free(Uv[k]); free(P[k]); free(Ev[k]); free(X[k]);
    }
    free(MASS); free(s_rho); free(s_u); free(s_p); free(U_F); free(P_F);
    free(U_next); free(P_next); free(RL_next); free(RR_next); free(U_t); free(P_t); free(RL_t); free(RR_t);
    return 0;
}

/* linear_GRP_solver_LAG on cnt interfaces; layout as ref_lag in ref_harness.c. */
void orc_lag(int cnt, const double *in, double eps, double atc, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 13 * q;
        double D[4], U[4];
        orc_lag_solve(a[0], a[0], a + 1, a + 7, eps, atc, D, U);
        double *o = out + 8 * q;
        for (int k2 = 0; k2 < 4; ++k2) {
            o[k2] = D[k2];
            o[4 + k2] = U[k2];
        }
    }
}

void orc_riemann_exact(int cnt, const double *in, double eps, double tol, int N, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 8 * q;
        double us, ps;
        int crw[2];
        double gap = orc_exact(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], eps, tol, N, &us, &ps, crw, NULL);
        double *o = out + 5 * q;
        o[0] = us; o[1] = ps; o[2] = crw[0]; o[3] = crw[1]; o[4] = gap;
    }
}

void orc_riemann_exact_iters(int cnt, const double *in, double eps, double tol, int N, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 8 * q;
        double us, ps;
        int crw[2], it;
        double gap = orc_exact(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], eps, tol, N, &us, &ps, crw, &it);
        double *o = out + 6 * q;
        o[0] = us; o[1] = ps; o[2] = crw[0]; o[3] = crw[1]; o[4] = gap; o[5] = it;
    }
}

void orc_riemann_exact_ben(int cnt, const double *in, double eps, double tol, int N, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 7 * q;
        double us, ps;
        int crw[2];
        double gap = orc_exact(a[0], a[0], a[1], a[2], a[3], a[4], a[5], a[6], eps, tol, N, &us, &ps, crw, NULL);
        double *o = out + 5 * q;
        o[0] = us; o[1] = ps; o[2] = crw[0]; o[3] = crw[1]; o[4] = gap;
    }
}

static void side_from(orc_side *s, const double *a)
{
    s->rho = a[0]; s->u = a[1]; s->v = a[2]; s->p = a[3];
    s->drho = a[4]; s->du = a[5]; s->dv = a[6]; s->dp = a[7];
    s->trho = a[8]; s->tu = a[9]; s->tv = a[10]; s->tp = a[11];
}

void orc_grp2d_flux(int cnt, const double *in, double tau, double eps, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 27 * q;
        orc_side L, R;
        side_from(&L, a + 3);
        side_from(&R, a + 15);
        double o8[8];
        int rv = orc_grp2d_flux_one(a[0], a[1], a[2], L, R, tau, eps, o8, NULL, 0);
        double *o = out + 9 * q;
        for (int k = 0; k < 8; ++k)
            o[k] = o8[k];
        o[8] = rv;
    }
}

/*
 * GRP_2D_flux of the two-component build (flux_solver.c:158-237 with
 * MULTIFLUID_BASICS): per-side gamma, passive volume fraction z and mass
 * fraction phi through linear_GRP_solver_Edir_Q1D, the mixture gamma of the
 * mid-time z (:203-208) in the energy flux, and the component fluxes and
 * interface values of :221-235.
 * in: cnt x 40 = n_x, n_y, then per side (left, right) gamma, rho,u,v,p,
 *     d_rho,d_u,d_v,d_p, t_rho,t_u,t_v,t_p, z,d_z,t_z, phi,d_phi,t_phi.
 * out: cnt x 19 = F_rho,F_u,F_v,F_e, RHO_int,U_int,V_int,P_int, F_phi,F_gamma,
 *     F_e_a, PHI, Z_a, U_qt_add_c,V_qt_add_c, U_qt_star,V_qt_star, P_star,
 *     return code.  gamma_a / gamma_b: config[6] / config[106]; store_gamma:
 *     config[60] (F_gamma is written only when it is set, else 0).
 */
static void scal_from(orc_scal *x, const double *a)
{
    x->z = a[0]; x->dz = a[1]; x->tz = a[2];
    x->phi = a[3]; x->dphi = a[4]; x->tphi = a[5];
}

void orc_grp2d_flux_mf(int cnt, const double *in, double tau, double eps, double gamma_a, double gamma_b,
                       int store_gamma, double *out)
{
    /* independent faces: split over the OpenMP threads (the reference's
       unstructured solver loops over its faces the same way) */
#pragma omp parallel for schedule(dynamic, 256)
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 40 * q;
        const double n_x = a[0], n_y = a[1];
        const double gL = a[2], gR = a[21];
        orc_side L, R;
        orc_scal XL, XR;
        side_from(&L, a + 3);
        scal_from(&XL, a + 15);
        side_from(&R, a + 22);
        scal_from(&XR, a + 34);
        /* rotation into the face frame, :172-189 (z and phi are scalars) */
        double u = L.u * n_x + L.v * n_y;
        double u_R = R.u * n_x + R.v * n_y;
        double d_u = L.du * n_x + L.dv * n_y;
        double d_u_R = R.du * n_x + R.dv * n_y;
        double t_u = L.tu * n_x + L.tv * n_y;
        double t_u_R = R.tu * n_x + R.tv * n_y;
        L.v = -L.u * n_y + L.v * n_x;
        R.v = -R.u * n_y + R.v * n_x;
        L.dv = -L.du * n_y + L.dv * n_x;
        R.dv = -R.du * n_y + R.dv * n_x;
        L.tv = -L.tu * n_y + L.tv * n_x;
        R.tv = -R.tu * n_y + R.tv * n_x;
        L.u = u;
        R.u = u_R;
        L.du = d_u;
        R.du = d_u_R;
        L.tu = t_u;
        R.tu = t_u_R;

        double ws[2], dire[4], mid[4], star[4], DX[2], UX[2];
        orc_q1d_solve_x(gL, gR, &L, &R, &XL, &XR, eps, eps, ws, dire, mid, star, DX, UX, NULL, 0);
        int rv = 0;
        if (mid[3] < eps || mid[0] < eps)
            rv = 1;
        else if (!orc_isfinite4(mid))
            rv = 2;
        else if (!orc_isfinite4(dire))
            rv = 3;

        double rho_mid = mid[0] + 0.5 * tau * dire[0];
        double u_mid = (mid[1] + 0.5 * tau * dire[1]) * n_x - (mid[2] + 0.5 * tau * dire[2]) * n_y;
        double v_mid = (mid[1] + 0.5 * tau * dire[1]) * n_y + (mid[2] + 0.5 * tau * dire[2]) * n_x;
        double p_mid = mid[3] + 0.5 * tau * dire[3];
        double phi_mid = UX[1] + 0.5 * tau * DX[1];
        double z_a_mid = UX[0] + 0.5 * tau * DX[0];
        double gamma_mid = 1.0 / (z_a_mid / (gamma_a - 1.0) + (1.0 - z_a_mid) / (gamma_b - 1.0)) + 1.0;

        double *o = out + 19 * q;
        double F_rho = rho_mid * (u_mid * n_x + v_mid * n_y);
        o[0] = F_rho;
        o[1] = F_rho * u_mid + p_mid * n_x;
        o[2] = F_rho * v_mid + p_mid * n_y;
        double F_e = (gamma_mid / (gamma_mid - 1.0)) * p_mid / rho_mid + 0.5 * (u_mid * u_mid + v_mid * v_mid);
        o[3] = F_rho * F_e;
        o[5] = (mid[1] + tau * dire[1]) * n_x - (mid[2] + tau * dire[2]) * n_y;
        o[6] = (mid[1] + tau * dire[1]) * n_y + (mid[2] + tau * dire[2]) * n_x;
        o[4] = mid[0] + tau * dire[0];
        o[7] = mid[3] + tau * dire[3];
        o[8] = F_rho * phi_mid;
        o[9] = store_gamma ? F_rho * gamma_mid : 0.0;
        double F_e_a = z_a_mid / (gamma_a - 1.0) * p_mid / rho_mid + 0.5 * phi_mid * (u_mid * u_mid + v_mid * v_mid);
        o[10] = F_rho * F_e_a;
        o[11] = UX[1] + tau * DX[1];
        o[12] = UX[0] + tau * DX[0];
        o[13] = F_rho * u_mid * phi_mid;
        o[14] = F_rho * v_mid * phi_mid;
        o[15] = p_mid * n_x;
        o[16] = p_mid * n_y;
        o[17] = p_mid / rho_mid * F_rho;
        o[18] = rv;
    }
}

void orc_q1d(int cnt, const double *in, double eps, double atc, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 25 * q;
        orc_side L, R;
        side_from(&L, a + 1);
        side_from(&R, a + 13);
        double ws[2], D[4], U[4], S[4];
        orc_q1d_solve(a[0], a[0], &L, &R, eps, atc, ws, D, U, S, NULL, 0);
        double *o = out + 14 * q;
        o[0] = ws[0]; o[1] = ws[1];
        for (int k = 0; k < 4; ++k) {
            o[2 + k] = D[k];
            o[6 + k] = U[k];
            o[10 + k] = S[k];
        }
    }
}

/* linear_GRP_solver_Edir_G2D on cnt interfaces; layout as orc_q1d. */
void orc_g2d(int cnt, const double *in, double eps, double atc, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 25 * q;
        orc_side L, R;
        side_from(&L, a + 1);
        side_from(&R, a + 13);
        double ws[2], D[4], U[4], S[4];
        orc_q1d_solve(a[0], a[0], &L, &R, eps, atc, ws, D, U, S, NULL, 1);
        double *o = out + 14 * q;
        o[0] = ws[0]; o[1] = ws[1];
        for (int k = 0; k < 4; ++k) {
            o[2 + k] = D[k];
            o[6 + k] = U[k];
            o[10 + k] = S[k];
        }
    }
}

void orc_grp1d(int cnt, const double *in, double eps, double atc, double *out)
{
    for (int q = 0; q < cnt; ++q) {
        const double *a = in + 13 * q;
        double D[3], U[3];
        orc_grp1d_solve(a[0], a + 1, a + 7, eps, atc, D, U);
        double *o = out + 6 * q;
        for (int k = 0; k < 3; ++k) {
            o[k] = D[k];
            o[3 + k] = U[k];
        }
    }
}
