// g2d.cuh -- non-acoustic case of the genuinely-2D direct Eulerian GRP solver.
//
// linear_GRP_solver_Edir_G2D (src/riemann_solver/linear_grp_solver_Edir_G2D.c:48-637)
// is the alternative interface solver that GRP_2D_flux keeps commented out at
// src/flux_calc/flux_solver.c:189 (called with atc = eps there); the library
// selects it with config[301] = 1.  Up to the acoustic case it is the quasi-1D
// solver with one change, its uniform-pair distance also counts the
// tangential velocity jump (:112; face_uniform<R, 1>), so q1d_star and the
// acoustic branch of q1d_derivs serve both.  Its non-acoustic case (:273-629)
// differs: the tangential derivatives enter the characteristic relations of
// both waves (the L_v coefficient of a shock, the Q term of a rarefaction, the
// v T_u and v T_p corrections of d_L and d_R), and the result is already the
// total time derivative along the t-axis, so no transversal terms follow.
//
// Single-fluid, EXACT_TANGENT_DERIVATIVE off (the reference defines it only for
// its documentation build, :16-18), frame velocities lambda_u = lambda_v = 0 as
// GRP_2D_flux and flux_generator_x/_y leave them (flux_solver.c:163,
// flux_generator_x.c:35-36): a subtracted zero is dropped (exact), a term
// 0 * x is kept where x can be non-finite, so NaN propagates as in the
// reference.  FP64 statements keep the reference's association (the FP64
// form is compiled without contraction), so results differ from it only by
// the rounding of pow.
#pragma once

namespace hydro {

// Q of a rarefaction's transversal correction (:367-370); the closed form has a
// removable singularity at gamma = 3.
template <typename R>
__device__ __forceinline__ R g2d_q(R c_frac, const Gas<R>& G)
{
    const R zeta = G.zeta;
    if (G.g < R(3) - G.eps || G.g > R(3) + G.eps)
        return (c_frac * (zeta - R(1)) + M<R>::pow_(c_frac, G.e1) * zeta) / (R(2) * zeta - R(1));
    return R(0.5) * c_frac + M<R>::pow_(c_frac, G.e1) * (R(0.5) - R(0.25) / zeta * M<R>::log_(c_frac));
}

template <typename R>
__device__ __noinline__ void g2d_derivs_exact(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G,
                                              const Star<R>& S, R D[4], R U[4])
{
    const R rho_L = L.rho, rho_R = Rr.rho;
    const R d_rho_L = L.drho, d_rho_R = Rr.drho, t_rho_L = L.trho, t_rho_R = Rr.trho;
    const R u_L = L.u, u_R = Rr.u, d_u_L = L.du, d_u_R = Rr.du, t_u_L = L.tu, t_u_R = Rr.tu;
    const R v_L = L.v, v_R = Rr.v, d_v_L = L.dv, d_v_R = Rr.dv, t_v_L = L.tv, t_v_R = Rr.tv;
    const R p_L = L.p, p_R = Rr.p, d_p_L = L.dp, d_p_R = Rr.dp, t_p_L = L.tp, t_p_R = Rr.tp;
    const R c_L = S.c_L, c_R = S.c_R;
    const R u_star = S.u_star, p_star = S.p_star;
    const R rho_star_L = S.rho_star_L, rho_star_R = S.rho_star_R, c_star_L = S.c_star_L, c_star_R = S.c_star_R;
    const R zetaL = G.zeta, zetaR = G.zeta, gL = G.g, gR = G.g;
    const R e3 = R(2) / G.zeta - R(1);  // exponent of the rarefaction's tangential-pressure term

    // trivial cases: the t-axis lies outside the wave fan (:274-304)
    if (S.speed_L > R(0)) {
        U[0] = rho_L; U[1] = u_L; U[2] = v_L; U[3] = p_L;
        D[0] = -u_L * d_rho_L - v_L * t_rho_L - rho_L * (d_u_L + t_v_L);
        D[1] = -u_L * d_u_L - v_L * t_u_L - d_p_L / rho_L;
        D[2] = -u_L * d_v_L - v_L * t_v_L - t_p_L / rho_L;
        D[3] = -u_L * d_p_L - v_L * t_p_L - rho_L * c_L * c_L * (d_u_L + t_v_L);
        return;
    }
    if (S.speed_R < R(0)) {
        U[0] = rho_R; U[1] = u_R; U[2] = v_R; U[3] = p_R;
        D[0] = -u_R * d_rho_R - v_R * t_rho_R - rho_R * (d_u_R + t_v_R);
        D[1] = -u_R * d_u_R - v_R * t_u_R - d_p_R / rho_R;
        D[2] = -u_R * d_v_R - v_R * t_v_R - t_p_R / rho_R;
        D[3] = -u_R * d_p_R - v_R * t_p_R - rho_R * c_R * c_R * (d_u_R + t_v_R);
        return;
    }

    // tangential derivatives from the acoustic relations on the star side that
    // holds the t-axis (:337-349)
    R T_rho, T_u, T_p;
    if (u_star < R(0)) {
        T_p = R(0.5) * ((t_u_L - t_u_R) * rho_star_R * c_star_R + t_p_L + t_p_R);
        T_u = R(0.5) * (t_u_L + t_u_R + (t_p_L - t_p_R) / rho_star_R / c_star_R);
        T_rho = t_rho_R - t_p_R / (c_star_R * c_star_R) + T_p / (c_star_R * c_star_R);
    } else {
        T_p = R(0.5) * ((t_u_L - t_u_R) * rho_star_L * c_star_L + t_p_L + t_p_R);
        T_u = R(0.5) * (t_u_L + t_u_R + (t_p_L - t_p_R) / rho_star_L / c_star_L);
        T_rho = t_rho_L - t_p_L / (c_star_L * c_star_L) + T_p / (c_star_L * c_star_L);
    }

    R C;
    if (S.crw0 && (u_star - c_star_L) > R(0)) {  // t-axis inside the 1-rarefaction (:351-384)
        U[1] = zetaL * (u_L + R(2) * c_L / G.gm1);
        C = U[1];
        U[3] = M<R>::pow_(C / c_L, G.sexp) * p_L;
        U[0] = gL * U[3] / C / C;
        U[2] = v_L;
        const R c_frac = C / c_L;
        const R TdS = (d_p_L - d_rho_L * c_L * c_L) / G.gm1 / rho_L;
        const R d_Psi = d_u_L + (gL * d_p_L / c_L - c_L * d_rho_L) / G.gm1 / rho_L;
        const R pe1 = M<R>::pow_(c_frac, G.e1);
        D[1] = (G.opz * pe1 + zetaL * M<R>::pow_(c_frac, G.e2));
        D[1] = D[1] / G.op2z * TdS;
        D[1] = D[1] - c_L * pe1 * d_Psi;
        D[1] = D[1] - c_L * t_v_L * g2d_q(c_frac, G);
        D[3] = U[0] * U[1] * D[1];
        D[0] = U[0] * U[1] * M<R>::pow_(c_frac, G.e2) * TdS * G.gm1;
        D[0] = (D[0] + D[3]) / C / C - U[2] * T_rho;
        D[2] = -U[1] * d_v_L * U[0] / rho_L - U[2] * t_v_L - T_p / U[0];
        D[2] = D[2] - (zetaL - R(1)) * (M<R>::pow_(c_frac, e3) - R(1)) / (zetaL - R(2)) / U[0] * t_p_L;
        D[3] = D[3] - U[2] * T_p;
        D[1] = D[1] - U[2] * T_u + U[1] * t_v_L;
        return;
    }
    if (S.crw1 && (u_star + c_star_R) < R(0)) {  // t-axis inside the 3-rarefaction (:385-418)
        U[1] = zetaR * (u_R - R(2) * c_R / G.gm1);
        C = R(0) - U[1];
        U[3] = M<R>::pow_(C / c_R, G.sexp) * p_R;
        U[0] = gR * U[3] / C / C;
        U[2] = v_R;
        const R c_frac = C / c_R;
        const R TdS = (d_p_R - d_rho_R * c_R * c_R) / G.gm1 / rho_R;
        const R d_Phi = d_u_R - (gR * d_p_R / c_R - c_R * d_rho_R) / G.gm1 / rho_R;
        const R pe1 = M<R>::pow_(c_frac, G.e1);
        D[1] = (G.opz * pe1 + zetaR * M<R>::pow_(c_frac, G.e2));
        D[1] = D[1] / G.op2z * TdS;
        D[1] = D[1] + c_R * pe1 * d_Phi;
        D[1] = D[1] + c_R * t_v_R * g2d_q(c_frac, G);
        D[3] = U[0] * U[1] * D[1];
        D[0] = U[0] * U[1] * M<R>::pow_(c_frac, G.e2) * TdS * G.gm1;
        D[0] = (D[0] + D[3]) / C / C - U[2] * T_rho;
        D[2] = -U[1] * d_v_R * U[0] / rho_R - U[2] * t_v_R - T_p / U[0];
        D[2] = D[2] - (zetaR - R(1)) * (M<R>::pow_(c_frac, e3) - R(1)) / (zetaR - R(2)) / U[0] * t_p_R;
        D[3] = D[3] - U[2] * T_p;
        D[1] = D[1] - U[2] * T_u + U[1] * t_v_R;
        return;
    }

    // non-sonic case: the t-axis is in the star region (:419-627)
    R T_v;
    if (u_star < R(0)) {
        U[0] = rho_star_R; U[1] = u_star; U[2] = v_R; U[3] = p_star;
        C = c_star_R;
        T_v = t_v_R;
    } else {
        U[0] = rho_star_L; U[1] = u_star; U[2] = v_L; U[3] = p_star;
        C = c_star_L;
        T_v = t_v_L;
    }
    // One c_frac across the branches, as in the reference: with two
    // rarefactions the 3-wave's value is the one the 1-side D[2] uses (:588).
    R c_frac = R(1);
    R a_L, b_L, d_L, a_R, b_R, d_R;
    // characteristic relation across the 1-wave: a_L u_t + b_L p_t = d_L (:444-481)
    if (S.crw0) {
        a_L = R(1);
        b_L = R(1) / rho_star_L / c_star_L;
        c_frac = c_star_L / c_L;
        const R TdS = (d_p_L - d_rho_L * c_L * c_L) / G.gm1 / rho_L;
        const R d_Psi = d_u_L + (gL * d_p_L / c_L - c_L * d_rho_L) / G.gm1 / rho_L;
        const R pe1 = M<R>::pow_(c_frac, G.e1);
        d_L = (G.opz * pe1 + zetaL * M<R>::pow_(c_frac, G.e2));
        d_L = d_L / G.op2z * TdS;
        d_L = d_L - c_L * pe1 * d_Psi;
        d_L = d_L - c_L * t_v_L * g2d_q(c_frac, G);
    } else {
        const R SmUs = -M<R>::sqrt_(R(0.5) * ((gL + R(1)) * p_L + G.gm1 * p_star) / rho_star_L);
        const R SmUL = -M<R>::sqrt_(R(0.5) * ((gL + R(1)) * p_star + G.gm1 * p_L) / rho_L);
        const R VAR = M<R>::sqrt_((R(1) - zetaL) / (rho_L * (p_star + zetaL * p_L)));
        const R H1 = R(0.5) * VAR * (p_star + G.op2z * p_L) / (p_star + zetaL * p_L);
        const R H2 = R(-0.5) * VAR * ((R(2) + zetaL) * p_star + zetaL * p_L) / (p_star + zetaL * p_L);
        const R H3 = R(-0.5) * VAR * (p_star - p_L) / rho_L;
        const R L_p = R(-1) / rho_L - SmUL * H2;
        const R L_u = SmUL + rho_L * (c_L * c_L * H2 + H3);
        const R L_rho = -SmUL * H3;
        const R L_v = SmUs + rho_L * (c_L * c_L * H2 + H3);
        a_L = R(1) - rho_star_L * SmUs * H1;
        b_L = -SmUs / (rho_star_L * c_star_L * c_star_L) + H1;
        d_L = L_rho * d_rho_L + L_u * d_u_L + L_p * d_p_L + L_v * t_v_L;
    }
    d_L = d_L - a_L * v_L * T_u - b_L * v_L * T_p;
    // and across the 3-wave (:482-519)
    if (S.crw1) {
        a_R = R(1);
        b_R = R(-1) / rho_star_R / c_star_R;
        c_frac = c_star_R / c_R;
        const R TdS = (d_p_R - d_rho_R * c_R * c_R) / G.gm1 / rho_R;
        const R d_Phi = d_u_R - (gR * d_p_R / c_R - c_R * d_rho_R) / G.gm1 / rho_R;
        const R pe1 = M<R>::pow_(c_frac, G.e1);
        d_R = (G.opz * pe1 + zetaR * M<R>::pow_(c_frac, G.e2));
        d_R = d_R / G.op2z * TdS;
        d_R = d_R + c_R * pe1 * d_Phi;
        d_R = d_R + c_R * t_v_R * g2d_q(c_frac, G);
    } else {
        const R SmUs = M<R>::sqrt_(R(0.5) * ((gR + R(1)) * p_R + G.gm1 * p_star) / rho_star_R);
        const R SmUR = M<R>::sqrt_(R(0.5) * ((gR + R(1)) * p_star + G.gm1 * p_R) / rho_R);
        const R VAR = M<R>::sqrt_((R(1) - zetaR) / (rho_R * (p_star + zetaR * p_R)));
        const R H1 = R(0.5) * VAR * (p_star + G.op2z * p_R) / (p_star + zetaR * p_R);
        const R H2 = R(-0.5) * VAR * ((R(2) + zetaR) * p_star + zetaR * p_R) / (p_star + zetaR * p_R);
        const R H3 = R(-0.5) * VAR * (p_star - p_R) / rho_R;
        const R L_p = R(-1) / rho_R + SmUR * H2;
        const R L_u = SmUR - rho_R * (c_R * c_R * H2 + H3);
        const R L_rho = SmUR * H3;
        const R L_v = SmUs - rho_R * (c_R * c_R * H2 + H3);
        a_R = R(1) + rho_star_R * SmUs * H1;
        b_R = -(SmUs / (rho_star_R * c_star_R * c_star_R) + H1);
        d_R = L_rho * d_rho_R + L_u * d_u_R + L_p * d_p_R + L_v * t_v_R;
    }
    d_R = d_R - a_R * v_R * T_u - b_R * v_R * T_p;
    const R detA = a_L * b_R - b_L * a_R;
    const R u_t_mat = (b_R * d_L - b_L * d_R) / detA;
    const R p_t_mat = (a_L * d_R - a_R * d_L) / detA;
    const R D0_p_tau = p_t_mat + U[2] * T_p;
    const R D0_u_tau = u_t_mat + U[2] * T_u;
    // total derivatives along the t-axis (:521-530)
    D[1] = u_t_mat + u_star / U[0] / C / C * D0_p_tau + u_star * T_v;
    D[3] = p_t_mat + u_star * U[0] * D0_u_tau;
    if (u_star < R(0)) {
        if (S.crw1) {  // :533-546
            D[0] = rho_star_R * u_star * M<R>::pow_(c_star_R / c_R, G.e2) * (d_p_R - d_rho_R * c_R * c_R) / rho_R;
            D[0] = (D[0] + D[3] + U[2] * T_p) / c_star_R / c_star_R - U[2] * T_rho;
            D[2] = -U[1] * d_v_R * U[0] / rho_R - U[2] * t_v_R - T_p / U[0];
            D[2] = D[2] + R(0) * d_v_R;
            D[2] = D[2] + u_star / c_star_R * (zetaR - R(1)) * (M<R>::pow_(c_frac, e3) - R(1)) / (zetaR - R(2)) / U[0] *
                              t_p_R;
        } else {  // :547-577
            const R SmUs = M<R>::sqrt_(R(0.5) * ((gR + R(1)) * p_R + G.gm1 * p_star) / rho_star_R);
            const R SmUR = M<R>::sqrt_(R(0.5) * ((gR + R(1)) * p_star + G.gm1 * p_R) / rho_R);
            const R VAR = p_R + zetaR * p_star;
            const R H1 = rho_R * p_R * (R(1) - zetaR * zetaR) / VAR / VAR;
            const R H2 = rho_R * p_star * (zetaR * zetaR - R(1)) / VAR / VAR;
            const R H3 = (p_star + zetaR * p_R) / VAR;
            const R L_rho = SmUR * H3 * d_rho_R;
            const R L_u = -rho_R * (H2 * c_R * c_R + H3) * d_u_R;
            const R L_p = H2 * SmUR * d_p_R;
            const R L_v = -rho_R * (H2 * c_R * c_R + H3) * t_v_R;
            D[0] = ((u_star + SmUs) / c_star_R / c_star_R - u_star * H1) * D0_p_tau +
                   rho_star_R * u_star * SmUs * H1 * D0_u_tau;
            D[0] = (D[0] - u_star * (L_p + L_rho + L_u + L_v)) / SmUs;
            D[0] = D[0] - U[2] * T_rho;
            const R f = SmUR * (H2 * d_p_R + H3 * d_rho_R) - rho_R * (H2 * c_R * c_R + H3) * d_u_R;
            const R rho_x = (f + H1 * (p_t_mat - rho_star_R * SmUs * u_t_mat) - D[0]) / (SmUR + u_R);
            D[0] = D[0] + R(0) * rho_x;
            D[2] = -(U[1] * (SmUR * d_v_R - t_p_R / rho_R) + (u_star + SmUs) * T_p / U[0]) / SmUs;
            D[2] = D[2] + R(0) * d_v_R - U[2] * t_v_R;
        }
    } else {
        if (S.crw0) {  // :580-593
            D[0] = rho_star_L * u_star * M<R>::pow_(c_star_L / c_L, G.e2) * (d_p_L - d_rho_L * c_L * c_L) / rho_L;
            D[0] = (D[0] + D[3] + U[2] * T_p) / c_star_L / c_star_L - U[2] * T_rho;
            D[2] = -U[1] * d_v_L * U[0] / rho_L - U[2] * t_v_L - T_p / U[0];
            D[2] = D[2] + R(0) * d_v_L;
            D[2] = D[2] - u_star / c_star_L * (zetaL - R(1)) * (M<R>::pow_(c_frac, e3) - R(1)) / (zetaL - R(2)) / U[0] *
                              t_p_L;
        } else {  // :594-624
            const R SmUs = -M<R>::sqrt_(R(0.5) * ((gL + R(1)) * p_L + G.gm1 * p_star) / rho_star_L);
            const R SmUL = -M<R>::sqrt_(R(0.5) * ((gL + R(1)) * p_star + G.gm1 * p_L) / rho_L);
            const R VAR = p_L + zetaL * p_star;
            const R H1 = rho_L * p_L * (R(1) - zetaL * zetaL) / VAR / VAR;
            const R H2 = rho_L * p_star * (zetaL * zetaL - R(1)) / VAR / VAR;
            const R H3 = (p_star + zetaL * p_L) / VAR;
            const R L_rho = SmUL * H3 * d_rho_L;
            const R L_u = -rho_L * (H2 * c_L * c_L + H3) * d_u_L;
            const R L_p = H2 * SmUL * d_p_L;
            const R L_v = -rho_L * (H2 * c_L * c_L + H3) * t_v_L;
            D[0] = ((u_star + SmUs) / c_star_L / c_star_L - u_star * H1) * D0_p_tau +
                   rho_star_L * u_star * SmUs * H1 * D0_u_tau;
            D[0] = (D[0] - u_star * (L_p + L_rho + L_u + L_v)) / SmUs;
            D[0] = D[0] - U[2] * T_rho;
            const R f = SmUL * (H2 * d_p_L + H3 * d_rho_L) - rho_L * (H2 * c_L * c_L + H3) * d_u_L;
            const R rho_x = (f + H1 * (p_t_mat - rho_star_L * SmUs * u_t_mat) - D[0]) / (SmUL + u_L);
            D[0] = D[0] + R(0) * rho_x;
            D[2] = -(U[1] * (SmUL * d_v_L - t_p_L / rho_L) + (u_star + SmUs) * T_p / U[0]) / SmUs;
            D[2] = D[2] + R(0) * d_v_L - U[2] * t_v_L;
        }
    }
    D[1] = D[1] + R(0) * T_u;
    D[3] = D[3] + R(0) * T_p;
}

}  // namespace hydro
