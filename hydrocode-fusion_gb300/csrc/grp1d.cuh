// grp1d.cuh -- device direct Eulerian GRP solver of the 1D scheme,
// src/riemann_solver/linear_grp_solver_Edir.c:33-337 (FP64, operand order
// kept; the exact Riemann solver is riemann_solver_exact_Ben.c:230-408, the
// same arithmetic as the two-gamma variant with equal gammas, at most 50
// Newton iterations).  atc = INFINITY gives the first-order Godunov flux
// (acoustic branch after the exact solver), atc = eps the second-order GRP.
#pragma once

#include "hydro_device.cuh"

namespace hydro {

template <typename R>
struct Side1 {
    R rho, u, p, srho, su, sp;
};

template <typename R>
__device__ __forceinline__ void grp1d_solve(const Side1<R>& Ls, const Side1<R>& Rs, const Gas<R>& G, R atc, R D[3],
                                            R U[3], int& iters)
{
    const R gamma = G.g;
    const R rho_L = Ls.rho, u_L = Ls.u, p_L = Ls.p, s_rho_L = Ls.srho, s_u_L = Ls.su, s_p_L = Ls.sp;
    const R rho_R = Rs.rho, u_R = Rs.u, p_R = Rs.p, s_rho_R = Rs.srho, s_u_R = Rs.su, s_p_R = Rs.sp;
    const R zeta = G.zeta, zts = zeta * zeta;
    R u_star, p_star, rho_star_L, rho_star_R, c_star_L, c_star_R;
    StarInfo st;
    st.crw0 = st.crw1 = 0;
    st.iters = -1;
    R c_L = M<R>::sqrt_(gamma * p_L / rho_L);
    R c_R = M<R>::sqrt_(gamma * p_R / rho_R);
    R dist = M<R>::sqrt_((u_L - u_R) * (u_L - u_R) + (p_L - p_R) * (p_L - p_R));
    if (dist < atc && atc < R(2) * G.eps) {
        rho_star_L = rho_L;
        rho_star_R = rho_R;
        c_star_L = c_L;
        c_star_R = c_R;
        u_star = R(0.5) * (u_R + u_L);
        p_star = R(0.5) * (p_R + p_L);
    } else {
        exact_riemann(u_L, u_R, p_L, p_R, c_L, c_R, G.eps, 50, G, u_star, p_star, st);
        if (p_star > p_L)
            rho_star_L = rho_L * (p_star + zeta * p_L) / (p_L + zeta * p_star);
        else
            rho_star_L = rho_L * M<R>::pow_(p_star / p_L, G.inv_g);
        if (p_star > p_R)
            rho_star_R = rho_R * (p_star + zeta * p_R) / (p_R + zeta * p_star);
        else
            rho_star_R = rho_R * M<R>::pow_(p_star / p_R, G.inv_g);
        c_star_L = M<R>::sqrt_(gamma * p_star / rho_star_L);
        c_star_R = M<R>::sqrt_(gamma * p_star / rho_star_R);
    }
    iters = st.iters;
    const int CRW0 = st.crw0, CRW1 = st.crw1;

    if (dist < atc) {  // acoustic case (:86-144)
        if (u_L - c_L > R(0)) {
            D[0] = -s_rho_L * u_L - rho_L * s_u_L;
            D[1] = (D[0] * u_L + s_rho_L * u_L * u_L + R(2) * rho_L * u_L * s_u_L + s_p_L) / -rho_L;
            D[2] = -G.gm1 * (R(0.5) * D[0] * u_L * u_L + rho_L * u_L * D[1]);
            D[2] = D[2] - s_u_L * (gamma * p_L + R(0.5) * G.gm1 * rho_L * u_L * u_L);
            D[2] = D[2] - u_L * (gamma * s_p_L + G.gm1 * (R(0.5) * s_rho_L * u_L * u_L + rho_L * u_L * s_u_L));
            U[0] = rho_L; U[1] = u_L; U[2] = p_L;
        } else if (u_R + c_R < R(0)) {
            D[0] = -s_rho_R * u_R - rho_R * s_u_R;
            D[1] = (D[0] * u_R + s_rho_R * u_R * u_R + R(2) * rho_R * u_R * s_u_R + s_p_R) / -rho_R;
            D[2] = -G.gm1 * (R(0.5) * D[0] * u_R * u_R + rho_R * u_R * D[1]);
            D[2] = D[2] - s_u_R * (gamma * p_R + R(0.5) * G.gm1 * rho_R * u_R * u_R);
            D[2] = D[2] - u_R * (gamma * s_p_R + G.gm1 * (R(0.5) * s_rho_R * u_R * u_R + rho_R * u_R * s_u_R));
            U[0] = rho_R; U[1] = u_R; U[2] = p_R;
        } else {
            R PI = (u_star + c_star_R) * rho_star_L * c_star_L * c_star_L / (u_star - c_star_L) / rho_star_R / c_star_R / c_star_R;
            D[1] = (s_p_L / rho_L + c_L * s_u_L) * PI / (R(1) - PI) + (s_p_R / rho_R - c_R * s_u_R) / (PI - R(1));
            D[2] = ((u_star + c_star_R) / rho_star_R / c_star_R / c_star_R) - ((u_star - c_star_L) / rho_star_L / c_star_L / c_star_L);
            D[2] = (s_p_R / rho_R - c_R * s_u_R - s_p_L / rho_L - c_L * s_u_L) / D[2];
            if (u_star > R(0)) {
                U[0] = rho_star_L; U[1] = u_star; U[2] = p_star;
                D[2] = D[2] * (R(1) - (u_star * u_star / c_star_L / c_star_L)) + rho_star_L * u_star * D[1];
                D[0] = (u_star * (s_p_L - s_rho_L * c_star_L * c_star_L) + D[2]) / c_star_L / c_star_L;
            } else {
                U[0] = rho_star_R; U[1] = u_star; U[2] = p_star;
                D[2] = D[2] * (R(1) - (u_star * u_star / c_star_R / c_star_R)) + rho_star_R * u_star * D[1];
                D[0] = (u_star * (s_p_R - s_rho_R * c_star_R * c_star_R) + D[2]) / c_star_R / c_star_R;
            }
        }
        return;
    }

    // non-acoustic case (:146-336)
    R speed_L, speed_R;
    if (CRW0)
        speed_L = u_L - c_L;
    else
        speed_L = (rho_star_L * u_star - rho_L * u_L) / (rho_star_L - rho_L);
    if (CRW1)
        speed_R = u_R + c_R;
    else
        speed_R = (rho_star_R * u_star - rho_R * u_R) / (rho_star_R - rho_R);

    if (speed_L > R(0)) {
        D[0] = -s_rho_L * u_L - rho_L * s_u_L;
        D[1] = (D[0] * u_L + s_rho_L * u_L * u_L + R(2) * rho_L * u_L * s_u_L + s_p_L) / -rho_L;
        D[2] = (s_u_L * p_L + u_L * s_p_L) * gamma / (R(1) - gamma) - R(0.5) * s_rho_L * u_L * u_L * u_L -
               R(1.5) * rho_L * u_L * u_L * s_u_L;
        D[2] = D[2] - R(0.5) * D[0] * u_L * u_L - rho_L * u_L * D[1];
        D[2] = D[2] * G.gm1;
        U[0] = rho_L; U[1] = u_L; U[2] = p_L;
    } else if (speed_R < R(0)) {
        D[0] = -s_rho_R * u_R - rho_R * s_u_R;
        D[1] = (D[0] * u_R + s_rho_R * u_R * u_R + R(2) * rho_R * u_R * s_u_R + s_p_R) / -rho_R;
        D[2] = -G.gm1 * (R(0.5) * D[0] * u_R * u_R + rho_R * u_R * D[1]);
        D[2] = D[2] - s_u_R * (gamma * p_R + R(0.5) * G.gm1 * rho_R * u_R * u_R);
        D[2] = D[2] - u_R * (gamma * s_p_R + G.gm1 * (R(0.5) * s_rho_R * u_R * u_R + rho_R * u_R * s_u_R));
        U[0] = rho_R; U[1] = u_R; U[2] = p_R;
    } else if (CRW0 && ((u_star - c_star_L) > R(0))) {  // t-axis in the 1-rarefaction
        U[1] = zeta * (u_L + R(2) * c_L / G.gm1);
        U[2] = U[1] * U[1] * rho_L / gamma / M<R>::pow_(p_L, G.inv_g);
        U[2] = M<R>::pow_(U[2], G.g_g1);
        U[0] = gamma * U[2] / U[1] / U[1];
        R pe1 = M<R>::pow_(U[1] / c_L, G.e1), pe2 = M<R>::pow_(U[1] / c_L, G.e2);
        D[1] = R(0.5) * (pe1 * G.opz + pe2 * zeta) / (R(0.5) + zeta);
        D[1] = D[1] * (s_p_L - s_rho_L * c_L * c_L) / G.gm1 / rho_L;
        D[1] = D[1] - c_L * pe1 * (s_u_L + (gamma * s_p_L / c_L - c_L * s_rho_L) / G.gm1 / rho_L);
        D[2] = U[0] * U[1] * D[1];
        D[0] = U[0] * U[1] * pe2 * (s_p_L - s_rho_L * c_L * c_L) / rho_L;
        D[0] = (D[0] + D[2]) / U[1] / U[1];
    } else if (CRW1 && ((u_star + c_star_R) < R(0))) {  // t-axis in the 3-rarefaction
        U[1] = zeta * (u_R - R(2) * c_R / G.gm1);
        U[2] = U[1] * U[1] * rho_R / gamma / M<R>::pow_(p_R, G.inv_g);
        U[2] = M<R>::pow_(U[2], G.g_g1);
        U[0] = gamma * U[2] / U[1] / U[1];
        R pe1 = M<R>::pow_(-U[1] / c_R, G.e1), pe2 = M<R>::pow_(-U[1] / c_R, G.e2);
        D[1] = R(0.5) * (pe1 * G.opz + pe2 * zeta) / (R(0.5) + zeta);
        D[1] = D[1] * (s_p_R - s_rho_R * c_R * c_R) / G.gm1 / rho_R;
        D[1] = D[1] + c_R * pe1 * (s_u_R - (gamma * s_p_R / c_R - c_R * s_rho_R) / G.gm1 / rho_R);
        D[2] = U[0] * U[1] * D[1];
        D[0] = U[0] * U[1] * pe2 * (s_p_R - s_rho_R * c_R * c_R) / rho_R;
        D[0] = (D[0] + D[2]) / U[1] / U[1];
    } else {  // non-sonic
        R a_L, b_L, d_L, a_R, b_R, d_R;
        if (CRW0) {
            a_L = R(1);
            b_L = R(1) / rho_star_L / c_star_L;
            R pe1 = M<R>::pow_(c_star_L / c_L, G.e1), pe2 = M<R>::pow_(c_star_L / c_L, G.e2);
            d_L = R(0.5) * (pe1 * G.opz + pe2 * zeta) / (R(0.5) + zeta);
            d_L = d_L * (s_p_L - s_rho_L * c_L * c_L) / G.gm1 / rho_L;
            d_L = d_L - c_L * pe1 * (s_u_L + (gamma * s_p_L / c_L - c_L * s_rho_L) / G.gm1 / rho_L);
        } else {
            R sq = M<R>::sqrt_((R(1) - zeta) / (rho_L * (p_star + zeta * p_L)));
            R H1 = R(0.5) * sq * (p_star + (R(1) + R(2) * zeta) * p_L) / (p_star + zeta * p_L);
            R H2 = R(-0.5) * sq * ((R(2) + zeta) * p_star + zeta * p_L) / (p_star + zeta * p_L);
            R H3 = R(-0.5) * sq * (p_star - p_L) / rho_L;
            R shk_spd = (rho_star_L * u_star - rho_L * u_L) / (rho_star_L - rho_L);
            a_L = R(1) - rho_star_L * (shk_spd - u_star) * H1;
            b_L = (u_star - shk_spd) / rho_star_L / c_star_L / c_star_L + H1;
            R L_rho = (u_L - shk_spd) * H3;
            R L_u = shk_spd - u_L + rho_L * c_L * c_L * H2 + rho_L * H3;
            R L_p = (u_L - shk_spd) * H2 - R(1) / rho_L;
            d_L = L_rho * s_rho_L + L_u * s_u_L + L_p * s_p_L;
        }
        if (CRW1) {
            a_R = R(1);
            b_R = R(-1) / rho_star_R / c_star_R;
            R pe1 = M<R>::pow_(c_star_R / c_R, G.e1), pe2 = M<R>::pow_(c_star_R / c_R, G.e2);
            d_R = R(0.5) * (pe1 * G.opz + pe2 * zeta) / (R(0.5) + zeta);
            d_R = d_R * (s_p_R - s_rho_R * c_R * c_R) / G.gm1 / rho_R;
            d_R = d_R + c_R * pe1 * (s_u_R - (gamma * s_p_R / c_R - c_R * s_rho_R) / G.gm1 / rho_R);
        } else {
            R sq = M<R>::sqrt_((R(1) - zeta) / (rho_R * (p_star + zeta * p_R)));
            R H1 = R(0.5) * sq * (p_star + (R(1) + R(2) * zeta) * p_R) / (p_star + zeta * p_R);
            R H2 = R(-0.5) * sq * ((R(2) + zeta) * p_star + zeta * p_R) / (p_star + zeta * p_R);
            R H3 = R(-0.5) * sq * (p_star - p_R) / rho_R;
            R shk_spd = (rho_star_R * u_star - rho_R * u_R) / (rho_star_R - rho_R);
            a_R = R(1) + rho_star_R * (shk_spd - u_star) * H1;
            b_R = (u_star - shk_spd) / rho_star_R / c_star_R / c_star_R - H1;
            R L_rho = (shk_spd - u_R) * H3;
            R L_u = shk_spd - u_R - rho_R * c_R * c_R * H2 - rho_R * H3;
            R L_p = (shk_spd - u_R) * H2 - R(1) / rho_R;
            d_R = L_rho * s_rho_R + L_u * s_u_R + L_p * s_p_R;
        }
        R p_t_mat = (d_L * a_R / a_L - d_R) / (b_L * a_R / a_L - b_R);
        R u_t_mat = (d_L - b_L * p_t_mat) / a_L;
        if (u_star < R(0)) {
            U[0] = rho_star_R; U[1] = u_star; U[2] = p_star;
            D[1] = u_t_mat + u_star * p_t_mat / rho_star_R / c_star_R / c_star_R;
            D[2] = p_t_mat + rho_star_R * u_star * u_t_mat;
            if (CRW1) {
                D[0] = rho_star_R * u_star * M<R>::pow_(c_star_R / c_R, G.e2) * (s_p_R - s_rho_R * c_R * c_R) / rho_R;
                D[0] = (D[0] + D[2]) / c_star_R / c_star_R;
            } else {
                R shk_spd = (rho_star_R * u_star - rho_R * u_R) / (rho_star_R - rho_R);
                R H1 = rho_R * p_R * (R(1) - zts) / (p_R + zeta * p_star) / (p_R + zeta * p_star);
                R H2 = rho_R * p_star * (zts - R(1)) / (p_R + zeta * p_star) / (p_R + zeta * p_star);
                R H3 = (p_star + zeta * p_R) / (p_R + zeta * p_star);
                R g_rho = u_star - shk_spd;
                R g_u = u_star * rho_star_R * (shk_spd - u_star) * H1;
                R g_p = shk_spd / c_star_R / c_star_R - u_star * H1;
                R f = (shk_spd - u_R) * (H2 * s_p_R + H3 * s_rho_R) - rho_R * (H2 * c_R * c_R + H3) * s_u_R;
                D[0] = (f * u_star - g_p * p_t_mat - g_u * u_t_mat) / g_rho;
            }
        } else {
            U[0] = rho_star_L; U[1] = u_star; U[2] = p_star;
            D[1] = u_t_mat + u_star * p_t_mat / rho_star_L / c_star_L / c_star_L;
            D[2] = p_t_mat + rho_star_L * u_star * u_t_mat;
            if (CRW0) {
                D[0] = rho_star_L * u_star * M<R>::pow_(c_star_L / c_L, G.e2) * (s_p_L - s_rho_L * c_L * c_L) / rho_L;
                D[0] = (D[0] + D[2]) / c_star_L / c_star_L;
            } else {
                R shk_spd = (rho_star_L * u_star - rho_L * u_L) / (rho_star_L - rho_L);
                R H1 = rho_L * p_L * (R(1) - zts) / (p_L + zeta * p_star) / (p_L + zeta * p_star);
                R H2 = rho_L * p_star * (zts - R(1)) / (p_L + zeta * p_star) / (p_L + zeta * p_star);
                R H3 = (p_star + zeta * p_L) / (p_L + zeta * p_star);
                R g_rho = u_star - shk_spd;
                R g_u = u_star * rho_star_L * (shk_spd - u_star) * H1;
                R g_p = shk_spd / c_star_L / c_star_L - u_star * H1;
                R f = (shk_spd - u_L) * (H2 * s_p_L + H3 * s_rho_L) - rho_L * (H2 * c_L * c_L + H3) * s_u_L;
                D[0] = (f * u_star - g_p * p_t_mat - g_u * u_t_mat) / g_rho;
            }
        }
    }
}

}  // namespace hydro
