// Two-component interface solver (FP64): the quasi-1D direct Eulerian GRP
// solver and GRP_2D_flux as the reference compiles them with MULTIFLUID_BASICS.
//
//  * linear_GRP_solver_Edir_Q1D (src/riemann_solver/linear_grp_solver_Edir_Q1D.c:38-554)
//    with a gamma per side (ifv_L->gamma, ifv_R->gamma) and the volume fraction
//    z and mass fraction phi as passive scalars (:55-62): they take the t-axis
//    side's value, and their time derivatives follow the tangential velocity's
//    without its pressure terms (:147-154, :180-245, :264-286, :297-338,
//    :444-519, :533-544);
//  * Riemann_solver_exact (src/riemann_solver/riemann_solver_exact_Ben.c:30-211),
//    the two-gamma exact solver;
//  * GRP_2D_flux (src/flux_calc/flux_solver.c:158-237): rotation into the face
//    frame, the mid-time state, the mixture gamma of the mid-time volume
//    fraction (:203-208) in the energy flux, and the component fluxes and
//    t+tau interface values (:221-235).
//
// Only the unstructured two-fluid code of the reference calls this variant, so
// it is exposed as a batch of independent faces (hydro_grp2d_flux_mf), not
// inside the structured step kernels: those stay single-gamma.  Every
// expression keeps the reference's operand order (files that include this are
// compiled without FMA contraction); the frame velocity is 0 as GRP_2D_flux
// sets it, and its products with derivatives are kept where a non-finite
// derivative would make them NaN.
#pragma once

#include "hydro_device.cuh"

namespace hydro {

// One side's passive scalars: z, phi with normal (d) and tangential (t) derivatives.
struct MfScal {
    double z, dz, tz, phi, dphi, tphi;
};

// Newton progress of a face whose exact solve was stopped at a pass's
// iteration cap: the current pressure and the iterations done.  The iteration
// is a function of these two alone (the velocities and the gap are recomputed
// from the pressure, the slopes at the start of the next iteration), so a later
// pass resumes it and takes exactly the steps one uninterrupted loop would.
struct MfNewton {
    double p;
    int it;
    int crw;  // wave pattern, once known: 4 | crw0 << 1 | crw1 (0: not yet computed)
};

// Exact two-gamma Riemann solver: GL on the 1-wave side, GR on the 3-wave side
// (riemann_solver_exact_Ben.c:30-211).  tol and eps are both config[4].
// At most `cap` iterations are taken in this call (cap >= 500: the reference's
// limit alone); when the cap stops an unfinished iteration, NW holds its state
// and the function returns true.  cap == 0 only classifies: the wave pattern and
// the starting pressure go to NW (true is returned unless the trivial case
// settles the face).  resume: continue from NW instead of the reference's
// starting pressure.
__device__ __noinline__ bool mf_exact(double uL, double uR, double pL, double pR, double cL, double cR, double eps,
                                      const Gas<double>& GL, const Gas<double>& GR, double& u_star, double& p_star,
                                      int& crw0, int& crw1, int cap, bool resume, MfNewton& NW)
{
    if (resume && NW.crw) {
        crw0 = (NW.crw >> 1) & 1;
        crw1 = NW.crw & 1;
    } else {
        const double uLR = curve_left(pR, uL, pL, cL, GL);
        const double uRL = curve_right(pL, uR, pR, cR, GR);
        crw1 = (uLR > uR + eps) ? 0 : 1;
        crw0 = (uRL > uL - eps) ? 1 : 0;
    }

    double k1 = -cL / pL / GL.g;
    double k3 = cR / pR / GR.g;
    double p_int;
    int it = 0;
    if (resume) {
        p_int = NW.p;
        it = NW.it;
    } else {
        p_int = (k1 * pL - k3 * pR - uL + uR) / (k1 - k3);
        if (p_int < 0.0)
            p_int = (pL < pR) ? pL : pR;
        p_int = 0.5 * p_int;
    }
    if (fabs(uL - uR) < eps && fabs(pL - pR) < eps) {
        p_star = 0.5 * (pL + pR);
        u_star = 0.5 * (uL + uR);
        return false;
    }
    if (cap == 0) {
        NW.p = p_int;
        NW.it = 0;
        NW.crw = 4 | crw0 << 1 | crw1;
        return true;
    }
    double vL, vR, k1n, k3n;   // curves and slopes at p_int (the slopes: the next iteration's k1, k3)
    const SideConst<double> KL = side_const(pL, cL, GL), KR = side_const(pR, cR, GR);
    curve_slope_at<double, true>(p_int, uL, pL, cL, GL, KL, vL, k1n);
    curve_slope_at<double, false>(p_int, uR, pR, cR, GR, KR, vR, k3n);
    double gap = fabs(vL - vR);
    const int stop = it + cap;
    while ((gap > eps) && (it != 500)) {
        if (it >= stop) {
            NW.p = p_int;
            NW.it = it;
            NW.crw = 4 | crw0 << 1 | crw1;
            return true;
        }
        k1 = k1n;
        k3 = k3n;
        const double p_new = p_int + (vR - vL) / (k1 - k3);
        p_int = (p_new < 0.0) ? 0.5 * p_int : p_new;
        ++it;
        curve_slope_at<double, true>(p_int, uL, pL, cL, GL, KL, vL, k1n);
        curve_slope_at<double, false>(p_int, uR, pR, cR, GR, KR, vR, k3n);
        gap = fabs(vL - vR);
    }
    u_star = k1 * (vR - vL) / (k1 - k3) + vL;
    p_star = p_int;
    return false;
}

// Scalars taken from one side's state as it stands (left/right of all waves).
__device__ __forceinline__ void mf_scal_side(const MfScal& X, double u, double v, double DX[2], double UX[2])
{
    UX[0] = X.z;
    UX[1] = X.phi;
    DX[0] = -u * X.dz - v * X.tz;
    DX[1] = -u * X.dphi - v * X.tphi;
}

// A state left or right of all waves: t-axis values and derivatives of that side.
__device__ __forceinline__ void mf_upwind_side(const Side<double>& S, const MfScal& X, double c, double D[4],
                                               double U[4], double DX[2], double UX[2])
{
    U[0] = S.rho; U[1] = S.u; U[2] = S.v; U[3] = S.p;
    D[0] = -S.u * S.drho - S.v * S.trho - S.rho * (S.du + S.tv);
    D[1] = -S.u * S.du - S.v * S.tu - S.dp / S.rho;
    D[2] = -S.u * S.dv - S.v * S.tv - S.tp / S.rho;
    D[3] = -S.u * S.dp - S.v * S.tp - S.rho * c * c * (S.du + S.tv);
    mf_scal_side(X, S.u, S.v, DX, UX);
}

// Sonic point inside a rarefaction (:290-339).  LEFT: the 1-rarefaction
// (d_Psi, minus sign), else the 3-rarefaction (d_Phi, plus sign); the caller
// has set U[0..3] and C.
template <bool LEFT>
__device__ __forceinline__ void mf_sonic(const Side<double>& S, const MfScal& X, const Gas<double>& G, double c,
                                         double C, double D[4], double U[4], double DX[2], double UX[2])
{
    const double c_frac = C / c;
    const double TdS = (S.dp - S.drho * c * c) / G.gm1 / S.rho;
    const double pe1 = M<double>::pow_(c_frac, G.e1), pe2 = M<double>::pow_(c_frac, G.e2);
    D[1] = (G.opz * pe1 + G.zeta * pe2);
    D[1] = D[1] / G.op2z * TdS;
    if (LEFT) {
        const double d_Psi = S.du + (G.g * S.dp / c - c * S.drho) / G.gm1 / S.rho;
        D[1] = D[1] - c * pe1 * d_Psi;
    } else {
        const double d_Phi = S.du - (G.g * S.dp / c - c * S.drho) / G.gm1 / S.rho;
        D[1] = D[1] + c * pe1 * d_Phi;
    }
    D[3] = U[0] * U[1] * D[1];
    D[0] = U[0] * U[1] * pe2 * TdS * G.gm1;
    D[0] = (D[0] + D[3]) / C / C;
    D[2] = -U[1] * S.dv * U[0] / S.rho;
    UX[0] = X.z;
    UX[1] = X.phi;
    DX[0] = -U[1] * X.dz * U[0] / S.rho;
    DX[1] = -U[1] * X.dphi * U[0] / S.rho;
}

// a, b, d of the characteristic relation across the 1-wave (LEFT) or 3-wave
// (:365-424): rarefaction or shock.
template <bool LEFT>
__device__ __forceinline__ void mf_wave_abd(const Side<double>& S, const Gas<double>& G, double c, double p_star,
                                            double rho_star, double c_star, bool crw, double& a, double& b, double& d)
{
    if (crw) {
        a = 1.0;
        b = LEFT ? 1.0 / rho_star / c_star : -1.0 / rho_star / c_star;
        const double c_frac = c_star / c;
        const double TdS = (S.dp - S.drho * c * c) / G.gm1 / S.rho;
        const double pe1 = M<double>::pow_(c_frac, G.e1), pe2 = M<double>::pow_(c_frac, G.e2);
        d = (G.opz * pe1 + G.zeta * pe2);
        d = d / G.op2z * TdS;
        if (LEFT) {
            const double d_Psi = S.du + (G.g * S.dp / c - c * S.drho) / G.gm1 / S.rho;
            d = d - c * pe1 * d_Psi;
        } else {
            const double d_Phi = S.du - (G.g * S.dp / c - c * S.drho) / G.gm1 / S.rho;
            d = d + c * pe1 * d_Phi;
        }
        return;
    }
    const double zeta = G.zeta, g = G.g, p = S.p, rho = S.rho;
    double SmUs = sqrt(0.5 * ((g + 1.0) * p + G.gm1 * p_star) / rho_star);
    double SmU = sqrt(0.5 * ((g + 1.0) * p_star + G.gm1 * p) / rho);
    if (LEFT) {
        SmUs = -SmUs;
        SmU = -SmU;
    }
    const double VAR = sqrt((1.0 - zeta) / (rho * (p_star + zeta * p)));
    const double H1 = 0.5 * VAR * (p_star + G.op2z * p) / (p_star + zeta * p);
    const double H2 = -0.5 * VAR * ((2.0 + zeta) * p_star + zeta * p) / (p_star + zeta * p);
    const double H3 = -0.5 * VAR * (p_star - p) / rho;
    double L_p, L_u, L_rho;
    if (LEFT) {
        L_p = -1.0 / rho - SmU * H2;
        L_u = SmU + rho * (c * c * H2 + H3);
        L_rho = -SmU * H3;
        a = 1.0 - rho_star * SmUs * H1;
        b = -SmUs / (rho_star * c_star * c_star) + H1;
    } else {
        L_p = -1.0 / rho + SmU * H2;
        L_u = SmU - rho * (c * c * H2 + H3);
        L_rho = SmU * H3;
        a = 1.0 + rho_star * SmUs * H1;
        b = -(SmUs / (rho_star * c_star * c_star) + H1);
    }
    d = L_rho * S.drho + L_u * S.du + L_p * S.dp;
}

// Density, tangential-velocity and scalar derivatives on the t-axis side of
// the contact (:433-520), given u_t and p_t (and D[3]).
template <bool LEFT>
__device__ __forceinline__ void mf_contact_side(const Side<double>& S, const MfScal& X, const Gas<double>& G, double c,
                                                double u_star, double p_star, double rho_star, double c_star,
                                                bool crw, double u_t_mat, double p_t_mat, double D[4], double U[4],
                                                double DX[2])
{
    if (crw) {
        D[0] = rho_star * u_star * M<double>::pow_(c_star / c, G.e2) * (S.dp - S.drho * c * c) / S.rho;
        D[0] = (D[0] + D[3]) / c_star / c_star;
        D[2] = -U[1] * S.dv * U[0] / S.rho;
        D[2] = D[2] + 0.0 * S.dv;
        DX[0] = -U[1] * X.dz * U[0] / S.rho;
        DX[0] = DX[0] + 0.0 * X.dz;
        DX[1] = -U[1] * X.dphi * U[0] / S.rho;
        DX[1] = DX[1] + 0.0 * X.dphi;
        return;
    }
    const double zeta = G.zeta, g = G.g, p = S.p, rho = S.rho;
    double SmUs = sqrt(0.5 * ((g + 1.0) * p + G.gm1 * p_star) / rho_star);
    double SmU = sqrt(0.5 * ((g + 1.0) * p_star + G.gm1 * p) / rho);
    if (LEFT) {
        SmUs = -SmUs;
        SmU = -SmU;
    }
    const double VAR = p + zeta * p_star;
    const double H1 = rho * p * (1.0 - zeta * zeta) / VAR / VAR;
    const double H2 = rho * p_star * (zeta * zeta - 1.0) / VAR / VAR;
    const double H3 = (p_star + zeta * p) / VAR;
    const double L_rho = SmU * H3 * S.drho;
    const double L_u = -rho * (H2 * c * c + H3) * S.du;
    const double L_p = H2 * SmU * S.dp;
    if (LEFT)
        D[0] = ((u_star + SmUs) / c_star / c_star - H1 * u_star) * p_t_mat + rho_star * u_star * SmUs * H1 * u_t_mat;
    else
        D[0] = ((u_star + SmUs) / c_star / c_star - u_star * H1) * p_t_mat + rho_star * u_star * SmUs * H1 * u_t_mat;
    D[0] = (D[0] - u_star * (L_p + L_rho + L_u)) / SmUs;
    const double f = SmU * (H2 * S.dp + H3 * S.drho) - rho * (H2 * c * c + H3) * S.du;
    const double rho_x = (f + H1 * (p_t_mat - rho_star * SmUs * u_t_mat) - D[0]) / (SmU + S.u);
    D[0] = D[0] + 0.0 * rho_x;
    D[2] = -U[1] * SmU * S.dv / SmUs;
    D[2] = D[2] + 0.0 * S.dv;
    DX[0] = -U[1] * SmU * X.dz / SmUs;
    DX[0] = DX[0] + 0.0 * X.dz;
    DX[1] = -U[1] * SmU * X.dphi / SmUs;
    DX[1] = DX[1] + 0.0 * X.dphi;
}

// The two-component quasi-1D GRP solver with atc = eps (as GRP_2D_flux calls
// it): t-axis values U (rho, u, v, p), UX (z, phi) and their time derivatives.
// cap / resume / NW as for mf_exact: returns true (and nothing else) when the
// exact solve was stopped at the cap.
__device__ __noinline__ bool mf_q1d(const Side<double>& L, const Side<double>& Rr, const MfScal& XL,
                                    const MfScal& XR, const Gas<double>& GL, const Gas<double>& GR, double eps,
                                    double D[4], double U[4], double DX[2], double UX[2], int cap, bool resume,
                                    MfNewton& NW)
{
    const double rho_L = L.rho, rho_R = Rr.rho, u_L = L.u, u_R = Rr.u, p_L = L.p, p_R = Rr.p;
    const double c_L = sqrt(GL.g * p_L / rho_L);
    const double c_R = sqrt(GR.g * p_R / rho_R);
    const double dist = sqrt((rho_L - rho_R) * (rho_L - rho_R) + (u_L - u_R) * (u_L - u_R) + (p_L - p_R) * (p_L - p_R));
    double u_star, p_star, rho_star_L, rho_star_R, c_star_L, c_star_R, speed_L, speed_R, C;
    int crw0 = 0, crw1 = 0;

    if (dist < eps) {  // :96-106, then the acoustic case (:139-254)
        u_star = 0.5 * (u_R + u_L);
        p_star = 0.5 * (p_R + p_L);
        rho_star_L = rho_L;
        c_star_L = c_L;
        speed_L = u_star - c_star_L;
        rho_star_R = rho_R;
        c_star_R = c_R;
        speed_R = u_star + c_star_R;
        if (speed_L > 0.0) {
            mf_upwind_side(L, XL, c_L, D, U, DX, UX);
            return false;
        }
        if (speed_R < 0.0) {
            mf_upwind_side(Rr, XR, c_R, D, U, DX, UX);
            return false;
        }
        // with the averaged star state c*_L = c_L, so the sonic branches
        // (u* - c*_L > 0 while speed_L <= 0) cannot be taken here
        const bool left = u_star > 0.0;
        if (left) {
            U[0] = rho_star_L; U[1] = u_star; U[2] = L.v; U[3] = p_star;
            C = c_star_L;
        } else {
            U[0] = rho_star_R; U[1] = u_star; U[2] = Rr.v; U[3] = p_star;
            C = c_star_R;
        }
        const Side<double>& S = left ? L : Rr;
        const MfScal& X = left ? XL : XR;
        UX[0] = X.z;
        UX[1] = X.phi;
        const double D_p = 0.5 * ((L.du * (U[0] * C) + L.dp) - (Rr.du * (U[0] * C) - Rr.dp));
        const double T_p = 0.5 * ((L.tu * (U[0] * C) + L.tp) - (Rr.tu * (U[0] * C) - Rr.tp));
        const double D_u = 0.5 * (L.du + L.dp / (U[0] * C) + Rr.du - Rr.dp / (U[0] * C));
        const double T_u = 0.5 * (L.tu + L.tp / (U[0] * C) + Rr.tu - Rr.tp / (U[0] * C));
        const double D_rho = S.drho - S.dp / (C * C) + D_p / (C * C);
        const double T_rho = S.trho - S.tp / (C * C) + T_p / (C * C);
        D[0] = -U[1] * D_rho - U[2] * T_rho - U[0] * (D_u + S.tv);
        D[1] = -U[1] * D_u - U[2] * T_u - D_p / U[0];
        D[2] = -U[1] * S.dv - U[2] * S.tv - T_p / U[0];
        D[3] = -U[1] * D_p - U[2] * T_p - U[0] * C * C * (D_u + S.tv);
        DX[0] = -U[1] * X.dz - U[2] * X.tz;
        DX[1] = -U[1] * X.dphi - U[2] * X.tphi;
        return false;
    }

    // star state and wave speeds (:107-134)
    if (mf_exact(u_L, u_R, p_L, p_R, c_L, c_R, eps, GL, GR, u_star, p_star, crw0, crw1, cap, resume, NW))
        return true;
    if (crw0) {
        rho_star_L = rho_L * M<double>::pow_(p_star / p_L, GL.inv_g);
        c_star_L = c_L * M<double>::pow_(p_star / p_L, GL.cexp);
        speed_L = u_L - c_L;
    } else {
        rho_star_L = rho_L * (p_star + GL.zeta * p_L) / (p_L + GL.zeta * p_star);
        c_star_L = sqrt(GL.g * p_star / rho_star_L);
        speed_L = u_L - c_L * sqrt(0.5 * ((GL.g + 1.0) * (p_star / p_L) + GL.gm1) / GL.g);
    }
    if (crw1) {
        rho_star_R = rho_R * M<double>::pow_(p_star / p_R, GR.inv_g);
        c_star_R = c_R * M<double>::pow_(p_star / p_R, GR.cexp);
        speed_R = u_R + c_R;
    } else {
        rho_star_R = rho_R * (p_star + GR.zeta * p_R) / (p_R + GR.zeta * p_star);
        c_star_R = sqrt(GR.g * p_star / rho_star_R);
        speed_R = u_R + c_R * sqrt(0.5 * ((GR.g + 1.0) * (p_star / p_R) + GR.gm1) / GR.g);
    }

    // non-acoustic case (:256-547)
    if (speed_L > 0.0) {
        mf_upwind_side(L, XL, c_L, D, U, DX, UX);
        return false;
    }
    if (speed_R < 0.0) {
        mf_upwind_side(Rr, XR, c_R, D, U, DX, UX);
        return false;
    }
    if (crw0 && ((u_star - c_star_L) > 0.0)) {  // sonic point in the 1-rarefaction
        U[1] = GL.zeta * (u_L + 2.0 * c_L / GL.gm1);
        C = U[1];
        U[3] = M<double>::pow_(C / c_L, GL.sexp) * p_L;
        U[0] = GL.g * U[3] / C / C;
        U[2] = L.v;
        mf_sonic<true>(L, XL, GL, c_L, C, D, U, DX, UX);
    } else if (crw1 && ((u_star + c_star_R) < 0.0)) {  // sonic point in the 3-rarefaction
        U[1] = GR.zeta * (u_R - 2.0 * c_R / GR.gm1);
        C = 0.0 - U[1];
        U[3] = M<double>::pow_(C / c_R, GR.sexp) * p_R;
        U[0] = GR.g * U[3] / C / C;
        U[2] = Rr.v;
        mf_sonic<false>(Rr, XR, GR, c_R, C, D, U, DX, UX);
    } else {  // non-sonic case
        if (u_star < 0.0) {
            U[0] = rho_star_R; U[1] = u_star; U[2] = Rr.v; U[3] = p_star;
            C = c_star_R;
            UX[0] = XR.z;
            UX[1] = XR.phi;
        } else {
            U[0] = rho_star_L; U[1] = u_star; U[2] = L.v; U[3] = p_star;
            C = c_star_L;
            UX[0] = XL.z;
            UX[1] = XL.phi;
        }
        double a_L, b_L, d_L, a_R, b_R, d_R;
        mf_wave_abd<true>(L, GL, c_L, p_star, rho_star_L, c_star_L, crw0, a_L, b_L, d_L);
        mf_wave_abd<false>(Rr, GR, c_R, p_star, rho_star_R, c_star_R, crw1, a_R, b_R, d_R);
        const double detA = a_L * b_R - b_L * a_R;
        const double u_t_mat = (b_R * d_L - b_L * d_R) / detA;
        const double p_t_mat = (a_L * d_R - a_R * d_L) / detA;
        D[1] = u_t_mat + u_star / U[0] / C / C * p_t_mat;
        D[3] = p_t_mat + u_star * U[0] * u_t_mat;
        if (u_star < 0.0)
            mf_contact_side<false>(Rr, XR, GR, c_R, u_star, p_star, rho_star_R, c_star_R, crw1, u_t_mat, p_t_mat, D, U,
                                   DX);
        else
            mf_contact_side<true>(L, XL, GL, c_L, u_star, p_star, rho_star_L, c_star_L, crw0, u_t_mat, p_t_mat, D, U,
                                  DX);
    }
    // transversal terms (:524-545)
    const double T_p = 0.5 * ((L.tu * (U[0] * C) + L.tp) - (Rr.tu * (U[0] * C) - Rr.tp));
    const double T_u = 0.5 * (L.tu + L.tp / (U[0] * C) + Rr.tu - Rr.tp / (U[0] * C));
    const bool left = u_star > 0.0;
    const Side<double>& S = left ? L : Rr;
    const MfScal& X = left ? XL : XR;
    const double T_rho = S.trho - S.tp / (C * C) + T_p / (C * C);
    D[0] = D[0] - U[2] * T_rho - U[0] * S.tv;
    D[1] = D[1] - U[2] * T_u;
    D[2] = D[2] - U[2] * S.tv - T_p / U[0];
    D[3] = D[3] - U[2] * T_p - U[0] * C * C * S.tv;
    DX[0] = DX[0] - U[2] * X.tz;
    DX[1] = DX[1] - U[2] * X.tphi;
    return false;
}

}  // namespace hydro
