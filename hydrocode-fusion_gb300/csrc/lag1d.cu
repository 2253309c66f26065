// lag1d.cu -- the 1D Lagrangian Godunov and GRP schemes on the GPU.
//
// Follows Godunov_solver_LAG_source (src/finite_volume/godunov_solver_LAG_source.c:28-243)
// and GRP_solver_LAG_source (src/finite_volume/grp_solver_LAG_source.c:28-355):
// each cell keeps its mass, the interfaces move with the star velocity, and
// the time step is min(CFL h/c, 1.01 tau_prev).  Boundary values, ghost-cell
// lengths and slopes follow bound_cond_slope_limiter with moving coordinates
// (src/inter_process/bound_cond_slope_limiter.c:30-136) and minmod_limiter
// (src/inter_process/slope_limiter.c:31-83); the interface solver is
// linear_GRP_solver_LAG (src/riemann_solver/linear_grp_solver_LAG.c:32-154).
//
// As for the Eulerian 1D schemes (solver1d.cu) the whole time loop is one
// launch on a thread-block cluster of up to 16 CTAs: each step's tau depends
// on every interface, and a tube of a few hundred cells cannot fill the GPU.
// Phases are separated by cluster barriers; the CFL minimum and the
// abort/stop flags are reduced per CTA and across the cluster through
// distributed shared memory.  Compiled with --fmad=false: FP64 operations
// round as the reference's C code (pow is the C library's method, libm_pow.cuh).
#include <atomic>
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "hydro_device.cuh"
#include "solver2d.h"

namespace hydro {

struct Run1DLagArgs {
    int m, order, N, bound, n_plot, el;
    double t_all, eps, cfl, h, cfg16, alpha;
    Gas<double> G;
    const double* init;   // [4][m] initial rho,u,p,E (boundary code -1)
    double* cur;          // [4][m] working state
    double* X;            // [m+1] node coordinates, moving
    double* snaps;        // [n_plot][4m + m+1] stored states and their nodes
    const double* time_plot;
    const double* mass;   // [m]
    double* s;            // [3][m] slopes of u, p, rho
    double* star;         // [4][m+1] rho*_L, u*, p*, rho*_R at t_n
    double* dire;         // [4][m+1] their time derivatives
    double* F;            // [2][m+1] interface velocity and pressure at t_n+1/2
    double* next;         // [4][m+1] rho_L, u, p, rho_R at t_n+1
    double* out;          // k, nt, time_c, tau, halted, exact solves, Newton iterations
};

// linear_GRP_solver_LAG (linear_grp_solver_LAG.c:32-154): L/R = rho, u, p and
// the material derivatives t_rho, t_u, t_p.  D = (rho*_L, u, p, rho*_R)_t,
// U = (rho*_L, u*, p*, rho*_R).  The 3-rarefaction term uses the left state's
// c, s_rho, s_p as in the reference (:128).
__device__ __forceinline__ void lag_solve(const double L[6], const double Rr[6], const Gas<double>& G, double atc,
                                          double D[4], double U[4], int& iters)
{
    const double rho_L = L[0], u_L = L[1], p_L = L[2], s_rho_L = L[3], s_u_L = L[4], s_p_L = L[5];
    const double rho_R = Rr[0], u_R = Rr[1], p_R = Rr[2], s_rho_R = Rr[3], s_u_R = Rr[4], s_p_R = Rr[5];
    const double g = G.g, zeta = G.zeta;
    const double c_L = sqrt(g * p_L / rho_L), c_R = sqrt(g * p_R / rho_R);
    const double g_L = rho_L * c_L, g_R = rho_R * c_R;
    double u_star, p_star;
    StarInfo st;
    exact_riemann<double>(u_L, u_R, p_L, p_R, c_L, c_R, G.eps, 500, G, u_star, p_star, st);
    iters = st.iters;
    double rho_star_L, rho_star_R, c_star_L, c_star_R;
    if (st.crw0) {
        rho_star_L = rho_L * M<double>::pow_(p_star / p_L, G.inv_g);
        c_star_L = c_L * M<double>::pow_(p_star / p_L, G.cexp);
    } else {
        rho_star_L = rho_L * (p_star + zeta * p_L) / (p_L + zeta * p_star);
        c_star_L = sqrt(g * p_star / rho_star_L);
    }
    if (st.crw1) {
        rho_star_R = rho_R * M<double>::pow_(p_star / p_R, G.inv_g);
        c_star_R = c_R * M<double>::pow_(p_star / p_R, G.cexp);
    } else {
        rho_star_R = rho_R * (p_star + zeta * p_R) / (p_R + zeta * p_star);
        c_star_R = sqrt(g * p_star / rho_star_R);
    }
    const double g_star_R = rho_star_R * c_star_R, g_star_L = rho_star_L * c_star_L;
    const double dist = sqrt((u_L - u_R) * (u_L - u_R) + (p_L - p_R) * (p_L - p_R));
    double a_L, b_L, d_L, a_R, b_R, d_R;
    if (dist < atc) {  // acoustic case (:83-91)
        a_L = 1.0;
        b_L = 1.0 / g_star_L;
        d_L = -g_L * s_u_L - s_p_L;
        a_R = -1.0;
        b_R = 1.0 / g_star_R;
        d_R = -g_R * s_u_R + s_p_R;
    } else {
        // exponent (3 gamma - 1) / 2 / (gamma + 1) of the rarefaction terms
        const double ebeta = (3.0 * g - 1.0) / 2.0 / (g + 1.0);
        if (st.crw0) {  // 1-rarefaction (:95-102)
            const double beta_star = g_star_L / g_L;
            a_L = 1.0;
            b_L = 1.0 / g_star_L;
            d_L = (s_u_L + s_p_L / g_L) +
                  1.0 / g_L / (3.0 * g - 1.0) * (c_L * c_L * s_rho_L - s_p_L) * (M<double>::pow_(beta_star, ebeta) - 1.0);
            d_L = -1.0 * sqrt(g_L * g_star_L) * d_L;
        } else {  // 1-shock (:103-114)
            const double W_L = (p_star - p_L) / (u_star - u_L);
            const double A = -0.5 / (p_star + zeta * p_L);
            a_L = 2.0 + A * (p_star - p_L);
            b_L = -W_L / g_star_L / g_star_L - (a_L - 1.0) / W_L;
            const double L_rho = (p_star - p_L) / 2.0 / rho_L;
            const double B = 1.0 / (p_star - p_L) - zeta * A;
            const double L_u = rho_L * (u_star - u_L) * (g * p_L * B + 0.5) + W_L;
            const double L_p = 1.0 + B * (p_star - p_L);
            d_L = L_u * s_u_L - L_p * s_p_L - L_rho * s_rho_L;
        }
        if (st.crw1) {  // 3-rarefaction (:116-123)
            const double beta_star = g_star_R / g_R;
            a_R = -1.0;
            b_R = 1.0 / g_star_R;
            d_R = (s_u_R - s_p_R / g_R) +
                  1.0 / g_R / (3.0 * g - 1.0) * (-c_L * c_L * s_rho_L + s_p_L) * (M<double>::pow_(beta_star, ebeta) - 1.0);
            d_R = -1.0 * sqrt(g_R * g_star_R) * d_R;
        } else {  // 3-shock (:124-135)
            const double W_R = (p_star - p_R) / (u_star - u_R);
            const double A = -0.5 / (p_star + zeta * p_R);
            a_R = -2.0 - A * (p_star - p_R);
            b_R = W_R / g_star_R / g_star_R - (a_R + 1.0) / W_R;
            const double L_rho = (p_star - p_R) / 2.0 / rho_R;
            const double B = 1.0 / (p_star - p_R) - zeta * A;
            const double L_u = rho_R * (u_R - u_star) * (g * p_R * B + 0.5) - W_R;
            const double L_p = 1.0 + B * (p_star - p_R);
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

namespace cg = cooperative_groups;

__global__ void __launch_bounds__(512) k_run1d_lag(const __grid_constant__ Run1DLagArgs a)
{
    cg::cluster_group cl = cg::this_cluster();
    const int m = a.m, tid = threadIdx.x;
    const int rank = (int)cl.block_rank(), CL = (int)cl.num_blocks();
    const int gtid = rank * (int)blockDim.x + tid, GNT = CL * (int)blockDim.x;
    const Gas<double>& G = a.G;
    const double gamma = G.g, eps = a.eps;
    double* rho = a.cur;
    double* uu = a.cur + m;
    double* pp = a.cur + 2 * m;
    double* ee = a.cur + 3 * m;
    double* X = a.X;
    double* s_u = a.s;
    double* s_p = a.s + m;
    double* s_rho = a.s + 2 * m;
    const int M1 = m + 1;
    __shared__ double part_hs[2];
    __shared__ int part_fl[2], part_bad[2];
    __shared__ double red[32];
    __shared__ int flg[32];
    // ghost cells: rho, u, p, srho, su, sp, H (zero slopes and H = h to start, as the reference's b_f_var)
    __shared__ double gL[7], gR[7];
    __shared__ double sh_hs;
    __shared__ int sh_abort, sh_stop;
    if (tid < 7) {
        gL[tid] = tid == 6 ? a.h : 0.0;
        gR[tid] = tid == 6 ? a.h : 0.0;
    }
    double time_c = 0.0, tau = a.cfg16;
    int nt = 0, found = 0, halted = 0, k;
    unsigned long long nfaces = 0, niters = 0;
    __syncthreads();
    for (k = 1; k <= a.N; ++k) {
        // plot snapshot: the reference copies CV.*[nt] and X[nt] to slot nt+1 and continues there
        if (time_c >= a.time_plot[nt] && nt < (a.n_plot - 1)) {
            double* sn = a.snaps + (size_t)nt * (5 * (size_t)m + 1);
            for (int q = gtid; q < 4 * m; q += GNT)
                sn[q] = a.cur[q];
            for (int q = gtid; q <= m; q += GNT)
                sn[4 * m + q] = X[q];
            nt++;
        }
        // boundary values and ghost lengths (bound_cond_slope_limiter.c:41-106)
        if (tid == 0) {
            const double* I = a.init;
            switch (a.bound) {
            case -1:
                if (!found) {
                    gL[1] = I[m]; gR[1] = I[m + m - 1];
                    gL[2] = I[2 * m]; gR[2] = I[2 * m + m - 1];
                    gL[0] = I[0]; gR[0] = I[m - 1];
                }
                gL[6] = a.h; gR[6] = a.h;
                break;
            case -2:
                gL[1] = -uu[0]; gR[1] = -uu[m - 1];
                gL[2] = pp[0]; gR[2] = pp[m - 1];
                gL[0] = rho[0]; gR[0] = rho[m - 1];
                gL[6] = X[1] - X[0]; gR[6] = X[m] - X[m - 1];
                break;
            case -4:
                gL[1] = uu[0]; gR[1] = uu[m - 1];
                gL[2] = pp[0]; gR[2] = pp[m - 1];
                gL[0] = rho[0]; gR[0] = rho[m - 1];
                gL[6] = X[1] - X[0]; gR[6] = X[m] - X[m - 1];
                break;
            case -7:
                gL[1] = uu[m - 1]; gR[1] = uu[0];
                gL[2] = pp[m - 1]; gR[2] = pp[0];
                gL[0] = rho[m - 1]; gR[0] = rho[0];
                gL[6] = X[m] - X[m - 1]; gR[6] = X[1] - X[0];
                break;
            case -24:
                gL[1] = -uu[0]; gR[1] = uu[m - 1];
                gL[2] = pp[0]; gR[2] = pp[m - 1];
                gL[0] = rho[0]; gR[0] = rho[m - 1];
                gL[6] = X[1] - X[0]; gR[6] = X[m] - X[m - 1];
                break;
            default:
                break;
            }
        }
        __syncthreads();
        if (a.order == 2) {
            // minmod_limiter on the moving grid (slope_limiter.c:47-81), u, p, rho
            for (int j = gtid; j < m; j += GNT) {
                const double* U3[3] = {uu, pp, rho};
                double* S3[3] = {s_u, s_p, s_rho};
                const double ULq[3] = {gL[1], gL[2], gL[0]}, URq[3] = {gR[1], gR[2], gR[0]};
                const double hl = j ? 0.5 * (X[j + 1] - X[j - 1]) : 0.5 * (X[j + 1] - X[j] + gL[6]);
                const double hr = (j < m - 1) ? 0.5 * (X[j + 2] - X[j]) : 0.5 * (X[j + 1] - X[j] + gR[6]);
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const double* U = U3[q];
                    const double sL = j ? (U[j] - U[j - 1]) / hl : (U[j] - ULq[q]) / hl;
                    const double sR = (j < m - 1) ? (U[j + 1] - U[j]) / hr : (URq[q] - U[j]) / hr;
                    S3[q][j] = found ? minmod3(a.alpha * sL, a.alpha * sR, S3[q][j]) : minmod2(sL, sR);
                }
            }
            cl.sync();  // the edge slopes below and the faces read slopes of other CTAs' cells
            if (tid == 0) {
                switch (a.bound) {
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
        }
        found = 1;
        __syncthreads();

        // interfaces at t_n
        double hs = INFINITY;
        int ab = 0, st = 0;
        for (int j = gtid; j <= m; j += GNT) {
            double Ls[6], Rs[6];
            const double h_L = j ? X[j] - X[j - 1] : gL[6];
            const double h_R = j < m ? X[j + 1] - X[j] : gR[6];
            if (a.order == 1) {
                Ls[0] = j ? rho[j - 1] : gL[0];
                Ls[1] = j ? uu[j - 1] : gL[1];
                Ls[2] = j ? pp[j - 1] : gL[2];
                Rs[0] = j < m ? rho[j] : gR[0];
                Rs[1] = j < m ? uu[j] : gR[1];
                Rs[2] = j < m ? pp[j] : gR[2];
            } else {
                if (j) {
                    Ls[0] = rho[j - 1] + 0.5 * h_L * s_rho[j - 1];
                    Ls[1] = uu[j - 1] + 0.5 * h_L * s_u[j - 1];
                    Ls[2] = pp[j - 1] + 0.5 * h_L * s_p[j - 1];
                } else {
                    Ls[0] = gL[0] + 0.5 * h_L * gL[3];
                    Ls[1] = gL[1] + 0.5 * h_L * gL[4];
                    Ls[2] = gL[2] + 0.5 * h_L * gL[5];
                }
                if (j < m) {
                    Rs[0] = rho[j] - 0.5 * h_R * s_rho[j];
                    Rs[1] = uu[j] - 0.5 * h_R * s_u[j];
                    Rs[2] = pp[j] - 0.5 * h_R * s_p[j];
                } else {  // the right ghost is reconstructed with '+' (grp_solver_LAG_source.c:158-162)
                    Rs[0] = gR[0] + 0.5 * h_R * gR[3];
                    Rs[1] = gR[1] + 0.5 * h_R * gR[4];
                    Rs[2] = gR[2] + 0.5 * h_R * gR[5];
                }
            }
            const double c_L = sqrt(gamma * Ls[2] / Ls[0]);
            const double c_R = sqrt(gamma * Rs[2] / Rs[0]);
            hs = fmin(hs, h_L / c_L);
            hs = fmin(hs, h_R / c_R);
            if ((a.bound == -2 || a.bound == -24) && j == 0)
                hs = fmin(hs, h_L / (fabs(Ls[1]) + c_L));
            if (a.bound == -2 && j == m)
                hs = fmin(hs, h_R / (fabs(Rs[1]) + c_R));
            if (a.order == 1) {  // godunov_solver_LAG_source.c:137-152
                double us, ps;
                StarInfo sti;
                exact_riemann<double>(Ls[1], Rs[1], Ls[2], Rs[2], c_L, c_R, G.eps, 500, G, us, ps, sti);
                nfaces++;
                niters += sti.iters;
                if (ps < eps || !M<double>::finite_(ps) || !M<double>::finite_(us))
                    st = 1;
                a.F[j] = us;
                a.F[M1 + j] = ps;
                continue;
            }
            // material derivatives (grp_solver_LAG_source.c:173-198)
            const double dL0 = j ? s_rho[j - 1] : gL[3], dL1 = j ? s_u[j - 1] : gL[4], dL2 = j ? s_p[j - 1] : gL[5];
            const double dR0 = j < m ? s_rho[j] : gR[3], dR1 = j < m ? s_u[j] : gR[4], dR2 = j < m ? s_p[j] : gR[5];
            // ifvar_check dim 1 aborts the run (:199-203)
            if (Ls[2] < eps || Rs[2] < eps || Ls[0] < eps || Rs[0] < eps || !M<double>::finite_(dL2) ||
                !M<double>::finite_(dR2) || !M<double>::finite_(dL1) || !M<double>::finite_(dR1) ||
                !M<double>::finite_(dL0) || !M<double>::finite_(dR0))
                ab = 1;
            Ls[4] = dL1 / Ls[0];
            Ls[5] = dL2 / Ls[0];
            Ls[3] = dL0 / Ls[0];
            Rs[4] = dR1 / Rs[0];
            Rs[5] = dR2 / Rs[0];
            Rs[3] = dR0 / Rs[0];
            double D[4], U[4];
            int it;
            lag_solve(Ls, Rs, G, eps, D, U, it);
            nfaces++;
            niters += it;
            // star_dire_check dim 1 (fluid_var_check.c:65-111): all four entries with config[8] = 1
            bool bad = U[2] < eps || U[0] < eps || !M<double>::finite_(U[1]) || !M<double>::finite_(U[2]) ||
                       !M<double>::finite_(U[0]) || !M<double>::finite_(D[1]) || !M<double>::finite_(D[2]) ||
                       !M<double>::finite_(D[0]);
            if (a.el == 1)
                bad = bad || U[3] < eps || !M<double>::finite_(U[3]) || !M<double>::finite_(D[3]);
            if (bad)
                st = 1;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a.star[q * M1 + j] = U[q];
                a.dire[q * M1 + j] = D[q];
            }
        }
        // block reductions: min of h/c, OR of the flags
        for (int off = 16; off; off >>= 1) {
            hs = fmin(hs, __shfl_xor_sync(0xffffffffu, hs, off));
            ab |= __shfl_xor_sync(0xffffffffu, ab, off);
            st |= __shfl_xor_sync(0xffffffffu, st, off);
        }
        if ((tid & 31) == 0) {
            red[tid >> 5] = hs;
            flg[tid >> 5] = ab | (st << 1);
        }
        __syncthreads();
        const int par = k & 1;
        if (tid == 0) {
            double v = INFINITY;
            int f = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                v = fmin(v, red[w]);
                f |= flg[w];
            }
            part_hs[par] = v;
            part_fl[par] = f;
        }
        cl.sync();  // every CTA's partials and interface results are visible
        if (tid == 0) {
            double v = INFINITY;
            int f = 0;
            for (int r = 0; r < CL; ++r) {  // fmin is exact: the order of the CTAs does not matter
                v = fmin(v, *cl.map_shared_rank(&part_hs[par], r));
                f |= *cl.map_shared_rank(&part_fl[par], r);
            }
            sh_hs = v;
            sh_abort = f & 1;
            sh_stop = (f >> 1) & 1;
        }
        __syncthreads();
        const double hsm = sh_hs;
        int stop_t = sh_stop;
        if (sh_abort) {
            halted = 1;
            break;
        }
        if (isfinite(a.t_all) || !isfinite(a.cfg16) || a.cfg16 <= 0.0) {
            tau = fmin(a.cfl * hsm, 1.01 * tau);
            if (tau < eps)
                stop_t = 1;
            else if ((time_c + tau) > (a.t_all - eps))
                tau = a.t_all - time_c;
            else if (!isfinite(tau)) {
                halted = 1;
                break;
            }
        }
        // interfaces at t_n+1/2 and t_n+1; the nodes move with them
        for (int j = gtid; j <= m; j += GNT) {
            if (a.order == 2) {
                const double rl = a.star[j], u = a.star[M1 + j], p = a.star[2 * M1 + j], rr = a.star[3 * M1 + j];
                const double drl = a.dire[j], du = a.dire[M1 + j], dp = a.dire[2 * M1 + j], drr = a.dire[3 * M1 + j];
                a.F[j] = u + 0.5 * tau * du;
                a.F[M1 + j] = p + 0.5 * tau * dp;
                a.next[j] = rl + tau * drl;
                a.next[M1 + j] = u + tau * du;
                a.next[2 * M1 + j] = p + tau * dp;
                a.next[3 * M1 + j] = rr + tau * drr;
            }
            X[j] += tau * a.F[j];
        }
        cl.sync();  // a cell reads both of its interfaces and nodes
        int bad = 0;
        for (int j = gtid; j < m; j += GNT) {
            const double* UF = a.F;
            const double* PF = a.F + M1;
            const double tm = tau / a.mass[j];
            rho[j] = 1.0 / (1.0 / rho[j] + tm * (UF[j + 1] - UF[j]));
            uu[j] = uu[j] - tm * (PF[j + 1] - PF[j]);
            ee[j] = ee[j] - tm * (PF[j + 1] * UF[j + 1] - PF[j] * UF[j]);
            pp[j] = (ee[j] - 0.5 * uu[j] * uu[j]) * (gamma - 1.0) * rho[j];
            if (pp[j] < eps || rho[j] < eps)
                bad = 1;
            if (a.order == 2) {
                const double dx = X[j + 1] - X[j];
                s_u[j] = (a.next[M1 + j + 1] - a.next[M1 + j]) / dx;
                s_p[j] = (a.next[2 * M1 + j + 1] - a.next[2 * M1 + j]) / dx;
                s_rho[j] = (a.next[j + 1] - a.next[3 * M1 + j]) / dx;
            }
        }
        bad = __syncthreads_or(bad);
        if (tid == 0)
            part_bad[par] = bad;
        cl.sync();  // also publishes this step's state and nodes to every CTA
        bad = 0;
        for (int r = 0; r < CL; ++r)
            bad |= *cl.map_shared_rank(&part_bad[par], r);
        if (bad)
            stop_t = 1;
        time_c += tau;
        if (stop_t || time_c > (a.t_all - eps) || !isfinite(time_c)) {
            halted = stop_t ? 2 : 0;
            break;
        }
    }
    // statistics
    for (int off = 16; off; off >>= 1) {
        nfaces += __shfl_xor_sync(0xffffffffu, nfaces, off);
        niters += __shfl_xor_sync(0xffffffffu, niters, off);
    }
    __shared__ unsigned long long sf[32], si[32];
    if ((tid & 31) == 0) {
        sf[tid >> 5] = nfaces;
        si[tid >> 5] = niters;
    }
    __shared__ unsigned long long cf, ci;
    __syncthreads();
    if (tid == 0) {
        unsigned long long Fs = 0, Is = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            Fs += sf[w];
            Is += si[w];
        }
        cf = Fs;
        ci = Is;
    }
    cl.sync();
    if (rank == 0 && tid == 0) {
        unsigned long long Fs = 0, Is = 0;
        for (int r = 0; r < CL; ++r) {
            Fs += *cl.map_shared_rank(&cf, r);
            Is += *cl.map_shared_rank(&ci, r);
        }
        a.out[0] = k;
        a.out[1] = nt;
        a.out[2] = time_c;
        a.out[3] = tau;
        a.out[4] = halted;
        a.out[5] = (double)Fs;
        a.out[6] = (double)Is;
    }
    cl.sync();  // no CTA leaves while rank 0 still reads its shared memory
}

// One cluster of up to 16 CTAs giving every interface its own thread (as
// launch_run1d in solver1d.cu); halves the cluster when it cannot be placed.
static cudaError_t launch_run1d_lag(const Run1DLagArgs& a, cudaStream_t st)
{
    // per-device kernel attribute, set on each device's first launch
    // (0 = not tried, 1 = set, 2 = refused)
    enum { MAX_DEVICES = 64 };
    static std::atomic<int> attr_state[MAX_DEVICES];
    int dev = 0;
    cudaGetDevice(&dev);
    int attr_set = 0;
    if (dev >= 0 && dev < MAX_DEVICES) {
        int st0 = attr_state[dev].load(std::memory_order_acquire);
        if (st0 == 0) {
            st0 = cudaFuncSetAttribute(k_run1d_lag, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess
                      ? 1 : 2;
            cudaGetLastError();
            attr_state[dev].store(st0, std::memory_order_release);
        }
        attr_set = st0 == 1;
    }
    const int faces = a.m + 1;
    int nt = 32 * ((faces + 32 * 16 - 1) / (32 * 16));
    if (nt > 512)
        nt = 512;
    int cl = (faces + nt - 1) / nt;
    if (cl > (attr_set ? 16 : 8))
        cl = attr_set ? 16 : 8;
    if (cl < 1)
        cl = 1;
    for (;;) {
        cudaLaunchConfig_t lc;
        memset(&lc, 0, sizeof(lc));
        lc.gridDim = dim3(cl);
        lc.blockDim = dim3(nt);
        lc.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cl;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        lc.attrs = at;
        lc.numAttrs = 1;
        cudaError_t e = cudaLaunchKernelEx(&lc, k_run1d_lag, a);
        if (e == cudaSuccess || cl == 1)
            return e;
        cudaGetLastError();
        cl = (cl + 1) / 2;
        nt = 32 * ((faces + 32 * cl - 1) / (32 * cl));
        if (nt > 512)
            nt = 512;
    }
}

// Runs one Lagrangian problem.  state: [4][m] rho,u,p,E in and the final state
// out; X: m+1 node coordinates in and out; snaps: [n_plot][4m + m+1] host
// snapshot slots (may be null when n_plot == 2).  -2 for an unknown boundary
// code.
static int run1d_lag(int m, int order, const double* cfg, int ncfg, double* state, double* X, const double* time_plot,
                     int n_plot, double* snaps_host, hydro_run_info* info, int* nt_out)
{
    memset(info, 0, sizeof(*info));
    auto at = [&](int k) { return k < ncfg ? cfg[k] : INFINITY; };
    Run1DLagArgs a;
    memset(&a, 0, sizeof(a));
    a.m = m;
    a.order = order;
    a.N = (int)at(5);
    a.bound = (int)at(17);
    a.n_plot = n_plot;
    a.el = isfinite(at(8)) ? (int)at(8) : 1;
    a.t_all = at(1);
    a.eps = at(4);
    a.cfl = at(7);
    a.h = at(10);
    a.cfg16 = at(16);
    a.alpha = at(41);
    if (a.bound != -1 && a.bound != -2 && a.bound != -4 && a.bound != -7 && a.bound != -24) {
        set_error("No suitable boundary conditions in x direction");
        return -2;
    }
    gas_fill(a.G, at(6), a.eps);
    std::vector<double> mass(m);
    for (int j = 0; j < m; ++j)  // MASS[k] = h * RHO[0][k] (godunov_solver_LAG_source.c:75-76)
        mass[j] = a.h * state[j];
    const size_t snap_sz = 5 * (size_t)m + 1;
    size_t need = 4 * (size_t)m * 2 + (size_t)(m + 1) + (size_t)n_plot * snap_sz + n_plot + (size_t)m + 3 * (size_t)m +
                  14 * (size_t)(m + 1) + 8;
    double* mem = nullptr;
    if (!cuda_ok(cudaMalloc(&mem, need * sizeof(double)), "1D Lagrangian buffers")) return -1;
    double* init = mem;
    double* cur = init + 4 * (size_t)m;
    double* dX = cur + 4 * (size_t)m;
    double* snaps = dX + (m + 1);
    double* tp = snaps + (size_t)n_plot * snap_sz;
    double* dmass = tp + n_plot;
    double* s = dmass + m;
    double* star = s + 3 * (size_t)m;
    double* dire = star + 4 * (size_t)(m + 1);
    double* F = dire + 4 * (size_t)(m + 1);
    double* next = F + 2 * (size_t)(m + 1);
    double* out = next + 4 * (size_t)(m + 1);
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = 0;
    if (!cuda_ok(cudaMemcpyAsync(init, state, 4 * m * sizeof(double), cudaMemcpyHostToDevice, st), "1D upload") ||
        !cuda_ok(cudaMemcpyAsync(cur, state, 4 * m * sizeof(double), cudaMemcpyHostToDevice, st), "1D upload") ||
        !cuda_ok(cudaMemcpyAsync(dX, X, (m + 1) * sizeof(double), cudaMemcpyHostToDevice, st), "1D upload") ||
        !cuda_ok(cudaMemcpyAsync(tp, time_plot, n_plot * sizeof(double), cudaMemcpyHostToDevice, st), "1D upload") ||
        !cuda_ok(cudaMemcpyAsync(dmass, mass.data(), m * sizeof(double), cudaMemcpyHostToDevice, st), "1D upload") ||
        !cuda_ok(cudaMemsetAsync(s, 0, 3 * m * sizeof(double), st), "1D clear"))
        rc = -1;
    if (!rc) {
        a.init = init; a.cur = cur; a.X = dX; a.snaps = snaps; a.time_plot = tp; a.mass = dmass; a.s = s;
        a.star = star; a.dire = dire; a.F = F; a.next = next; a.out = out;
        cudaEventRecord(e0, st);
        if (!cuda_ok(launch_run1d_lag(a, st), "1D Lagrangian launch")) rc = -1;
        count_launch();
        cudaEventRecord(e1, st);
    }
    double o[8] = {0};
    if (!rc && (!cuda_ok(cudaMemcpyAsync(o, out, 7 * sizeof(double), cudaMemcpyDeviceToHost, st), "1D result") ||
                !cuda_ok(cudaMemcpyAsync(state, cur, 4 * m * sizeof(double), cudaMemcpyDeviceToHost, st), "1D download") ||
                !cuda_ok(cudaMemcpyAsync(X, dX, (m + 1) * sizeof(double), cudaMemcpyDeviceToHost, st), "1D download") ||
                !cuda_ok(cudaStreamSynchronize(st), "1D Lagrangian run")))
        rc = -1;
    int nt = (int)o[1];
    if (!rc && snaps_host && nt > 0)
        if (!cuda_ok(cudaMemcpy(snaps_host, snaps, (size_t)nt * snap_sz * sizeof(double), cudaMemcpyDeviceToHost),
                     "1D snaps"))
            rc = -1;
    float ms = 0.f;
    if (!rc)
        cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    cudaFree(mem);
    if (rc)
        return rc;
    info->k_out = (int)o[0];
    info->time = o[2];
    info->tau = o[3];
    info->halted = (int)o[4];
    info->newton_faces = (unsigned long long)o[5];
    info->newton_iters = (unsigned long long)o[6];
    info->sweeps_launched = 1;
    info->gpu_ms = ms;
    *nt_out = nt;
    return 0;
}

// The scheme entry points' body: the reference's CV/X slots in and out.
static void entry_1d_lag(const int m, struct cell_var_stru CV, double* X[], double* cpu_time, int* N_plot,
                         double time_plot[], int order)
{
    std::vector<double> state(4 * (size_t)m), nodes(X[0], X[0] + m + 1);
    memcpy(&state[0], CV.RHO[0], m * sizeof(double));
    memcpy(&state[m], CV.U[0], m * sizeof(double));
    memcpy(&state[2 * m], CV.P[0], m * sizeof(double));
    memcpy(&state[3 * m], CV.E[0], m * sizeof(double));
    const int n_plot = *N_plot;
    std::vector<double> snaps((size_t)n_plot * (5 * (size_t)m + 1));
    hydro_run_info info;
    int nt = 0;
    int rc = run1d_lag(m, order, config, N_CONF, state.data(), nodes.data(), time_plot, n_plot, snaps.data(), &info,
                       &nt);
    if (rc == -2) {
        printf("No suitable boundary coditions in x direction!\n");
        config[5] = 1.0;
        *N_plot = 1;
        time_plot[0] = 0.0;
        return;
    }
    if (rc) {
        fprintf(stderr, "hydro_gb300: 1D Lagrangian run failed: %s\n", hydro_gb300_last_error());
        exit(5);
    }
    for (int k = 1; k < nt; ++k) {  // slot 0 is the caller's initial data
        const double* sp = &snaps[(size_t)k * (5 * (size_t)m + 1)];
        memcpy(CV.RHO[k], sp, m * sizeof(double));
        memcpy(CV.U[k], sp + m, m * sizeof(double));
        memcpy(CV.P[k], sp + 2 * m, m * sizeof(double));
        memcpy(CV.E[k], sp + 3 * m, m * sizeof(double));
        memcpy(X[k], sp + 4 * m, (m + 1) * sizeof(double));
    }
    memcpy(CV.RHO[nt], &state[0], m * sizeof(double));
    memcpy(CV.U[nt], &state[m], m * sizeof(double));
    memcpy(CV.P[nt], &state[2 * m], m * sizeof(double));
    memcpy(CV.E[nt], &state[3 * m], m * sizeof(double));
    memcpy(X[nt], nodes.data(), (m + 1) * sizeof(double));
    printf("\nTime is up at time step %d.\n", info.k_out);
    printf("The cost of GPU time for 1D-%s Lagrangian scheme for this problem is %g seconds.\n",
           order == 1 ? "Godunov" : "GRP", info.gpu_ms * 1e-3);
    config[5] = (double)info.k_out;
    *N_plot = nt + 1;
    const double t_all = config[1];
    if (isfinite(info.time))
        time_plot[nt] = info.time;
    else if (isfinite(t_all))
        time_plot[nt] = t_all;
    else if (isfinite(info.tau))
        time_plot[nt] = info.k_out * info.tau;
    cpu_time[nt] = info.gpu_ms * 1e-3;
}

}  // namespace hydro

using namespace hydro;

extern "C" {

void Godunov_solver_LAG_source(const int m, struct cell_var_stru CV, double* X[], double* cpu_time, int* N_plot,
                               double time_plot[])
{
    entry_1d_lag(m, CV, X, cpu_time, N_plot, time_plot, 1);
}

void GRP_solver_LAG_source(const int m, struct cell_var_stru CV, double* X[], double* cpu_time, int* N_plot,
                           double time_plot[])
{
    entry_1d_lag(m, CV, X, cpu_time, N_plot, time_plot, 2);
}

int hydro1d_run_lag(int m, double* rho, double* u, double* p, double* E, double* X, const double* cfg, int ncfg,
                    int order, hydro_run_info* info)
{
    std::vector<double> state(4 * (size_t)m), nodes(m + 1);
    const double g = ncfg > 6 ? cfg[6] : 1.4, h = ncfg > 10 ? cfg[10] : 1.0 / m;
    for (int j = 0; j < m; ++j) {
        state[j] = rho[j];
        state[m + j] = u[j];
        state[2 * m + j] = p[j];
        // the 1D driver's energy (src/hydrocode_1D/hydrocode.c:234-235)
        state[3 * m + j] = E ? E[j] : 0.5 * u[j] * u[j] + p[j] / (g - 1.0) / rho[j];
    }
    for (int j = 0; j <= m; ++j)  // X[0][j] = h j (src/hydrocode_1D/hydrocode.c:232-233)
        nodes[j] = h * j;
    double tp[2] = {0.0, ncfg > 1 ? cfg[1] : INFINITY};
    std::vector<double> c(cfg, cfg + ncfg);
    if (ncfg > 8 && !isfinite(c[8]))
        c[8] = 1.0;  // the driver sets config[8] = 1 for Lagrangian runs
    int nt = 0;
    int rc = run1d_lag(m, order, c.data(), ncfg, state.data(), nodes.data(), tp, 2, nullptr, info, &nt);
    if (rc)
        return rc;
    for (int j = 0; j < m; ++j) {
        rho[j] = state[j];
        u[j] = state[m + j];
        p[j] = state[2 * m + j];
        if (E)
            E[j] = state[3 * m + j];
    }
    if (X)
        for (int j = 0; j <= m; ++j)
            X[j] = nodes[j];
    return 0;
}

}  // extern "C"
