// solver1d.cu -- the 1D Eulerian Godunov and GRP schemes on the GPU.
//
// A 1D tube (the benchmark tube has 400 cells) is far too small to fill a
// GB300, and its time step depends on every interface's reconstructed state
// each step, so the whole time loop runs inside ONE kernel launch and nothing
// returns to the host until the run ends.  The work of a step is spread over
// a thread-block cluster of up to 16 CTAs on as many SMs (the exact Riemann
// solver's FP64 Newton iteration is the cost, and one SM's FP64 pipe would
// serialise it); phases are separated by cluster barriers, the CFL minimum
// and the stop/abort flags are reduced per CTA and then across the cluster
// through distributed shared memory, so every CTA takes the same decisions.
// State lives in global memory (L2-resident at this size).
//
// Follows Godunov_solver_EUL_source (src/finite_volume/godunov_solver_EUL_source.c:27-230)
// and GRP_solver_EUL_source (src/finite_volume/grp_solver_EUL_source.c:27-334)
// with bound_cond_slope_limiter (src/inter_process/bound_cond_slope_limiter.c:30-136)
// and minmod_limiter (src/inter_process/slope_limiter.c:31-83).  Compiled with
// --fmad=false: FP64 operations round as the reference's C code.
#include <atomic>
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "grp1d.cuh"
#include "solver2d.h"

namespace hydro {

struct Run1DArgs {
    int m, order, N, bound, n_plot;
    double t_all, eps, cfl, h, inv_h, cfg16, alpha;
    int pow2;
    Gas<double> G;
    const double* init;   // [4][m] initial rho,u,p,E (the reference's CV.*[0])
    double* cur;          // [4][m] working state
    double* snaps;        // [n_plot][4][m] plot snapshots
    const double* time_plot;
    double* s;            // [3][m] slopes rho,u,p
    double* mid;          // [3][m+1]
    double* dire;         // [3][m+1]
    double* F;            // [3][m+1]
    double* out;          // k, nt, time_c, tau, halted, newton faces, newton iterations
};

__device__ __forceinline__ double dh(double d, const Run1DArgs& a) { return a.pow2 ? d * a.inv_h : d / a.h; }

namespace cg = cooperative_groups;

__global__ void __launch_bounds__(512) k_run1d(const __grid_constant__ Run1DArgs a)
{
    cg::cluster_group cl = cg::this_cluster();
    const int m = a.m, tid = threadIdx.x;
    const int rank = (int)cl.block_rank(), CL = (int)cl.num_blocks();
    // cells and faces are spread over every thread of the cluster
    const int gtid = rank * (int)blockDim.x + tid, GNT = CL * (int)blockDim.x;
    // per-CTA partials of the reductions, double-buffered by step parity
    __shared__ double part_hs[2];
    __shared__ int part_fl[2], part_bad[2];
    const double gamma = a.G.g, eps = a.eps;
    double* rho = a.cur;
    double* uu = a.cur + m;
    double* pp = a.cur + 2 * m;
    double* ee = a.cur + 3 * m;
    double* s_rho = a.s;
    double* s_u = a.s + m;
    double* s_p = a.s + 2 * m;
    __shared__ double red[32];
    __shared__ int flg[32];
    __shared__ double gL[6], gR[6];  // rho,u,p, srho,su,sp
    __shared__ double sh_hs;
    __shared__ int sh_abort, sh_stop;
    if (tid < 6) {
        gL[tid] = 0.0;
        gR[tid] = 0.0;
    }
    double time_c = 0.0, tau = a.cfg16;
    int nt = 0, found = 0, halted = 0, k;
    unsigned long long nfaces = 0, niters = 0;
    __syncthreads();
    for (k = 1; k <= a.N; ++k) {
        // plot snapshot: the reference copies CV.*[nt] to CV.*[nt+1] and continues there
        if (time_c >= a.time_plot[nt] && nt < (a.n_plot - 1)) {
            for (int q = gtid; q < 4 * m; q += GNT)
                a.snaps[(size_t)nt * 4 * m + q] = a.cur[q];
            nt++;
        }
        if (tid == 0) {
            const double* I = a.init;
            switch (a.bound) {
            case -1:
                if (!found) {
                    gL[1] = I[m]; gR[1] = I[m + m - 1];
                    gL[2] = I[2 * m]; gR[2] = I[2 * m + m - 1];
                    gL[0] = I[0]; gR[0] = I[m - 1];
                }
                break;
            case -2:
                gL[1] = -uu[0]; gR[1] = -uu[m - 1];
                gL[2] = pp[0]; gR[2] = pp[m - 1];
                gL[0] = rho[0]; gR[0] = rho[m - 1];
                break;
            case -4:
                gL[1] = uu[0]; gR[1] = uu[m - 1];
                gL[2] = pp[0]; gR[2] = pp[m - 1];
                gL[0] = rho[0]; gR[0] = rho[m - 1];
                break;
            case -7:
                gL[1] = uu[m - 1]; gR[1] = uu[0];
                gL[2] = pp[m - 1]; gR[2] = pp[0];
                gL[0] = rho[m - 1]; gR[0] = rho[0];
                break;
            case -24:
                gL[1] = -uu[0]; gR[1] = uu[m - 1];
                gL[2] = pp[0]; gR[2] = pp[m - 1];
                gL[0] = rho[0]; gR[0] = rho[m - 1];
                break;
            default:
                break;
            }
        }
        __syncthreads();
        if (a.order == 2) {
            for (int j = gtid; j < m; j += GNT) {
                const double* U3[3] = {uu, pp, rho};
                double* S3[3] = {s_u, s_p, s_rho};
                const double ULq[3] = {gL[1], gL[2], gL[0]}, URq[3] = {gR[1], gR[2], gR[0]};
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const double* U = U3[q];
                    double sL = j ? dh(U[j] - U[j - 1], a) : dh(U[j] - ULq[q], a);
                    double sR = (j < m - 1) ? dh(U[j + 1] - U[j], a) : dh(URq[q] - U[j], a);
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

        // interfaces
        double hs = INFINITY;
        int ab = 0, st = 0;
        for (int j = gtid; j <= m; j += GNT) {
            Side1<double> L, R;
            if (a.order == 1) {
                if (j) { L.rho = rho[j - 1]; L.u = uu[j - 1]; L.p = pp[j - 1]; }
                else { L.rho = gL[0]; L.u = gL[1]; L.p = gL[2]; }
                if (j < m) { R.rho = rho[j]; R.u = uu[j]; R.p = pp[j]; }
                else { R.rho = gR[0]; R.u = gR[1]; R.p = gR[2]; }
                L.srho = L.su = L.sp = 0.0;
                R.srho = R.su = R.sp = 0.0;
            } else {
                if (j) {
                    L.rho = rho[j - 1] + 0.5 * a.h * s_rho[j - 1];
                    L.u = uu[j - 1] + 0.5 * a.h * s_u[j - 1];
                    L.p = pp[j - 1] + 0.5 * a.h * s_p[j - 1];
                    L.srho = s_rho[j - 1]; L.su = s_u[j - 1]; L.sp = s_p[j - 1];
                } else {
                    L.rho = gL[0] + 0.5 * a.h * gL[3];
                    L.u = gL[1] + 0.5 * a.h * gL[4];
                    L.p = gL[2] + 0.5 * a.h * gL[5];
                    L.srho = gL[3]; L.su = gL[4]; L.sp = gL[5];
                }
                if (j < m) {
                    R.rho = rho[j] - 0.5 * a.h * s_rho[j];
                    R.u = uu[j] - 0.5 * a.h * s_u[j];
                    R.p = pp[j] - 0.5 * a.h * s_p[j];
                    R.srho = s_rho[j]; R.su = s_u[j]; R.sp = s_p[j];
                } else {
                    // the right ghost is reconstructed with '+' (grp_solver_EUL_source.c:158-162)
                    R.rho = gR[0] + 0.5 * a.h * gR[3];
                    R.u = gR[1] + 0.5 * a.h * gR[4];
                    R.p = gR[2] + 0.5 * a.h * gR[5];
                    R.srho = gR[3]; R.su = gR[4]; R.sp = gR[5];
                }
            }
            double c_L = sqrt(gamma * L.p / L.rho);
            double c_R = sqrt(gamma * R.p / R.rho);
            hs = fmin(hs, a.h / (fabs(L.u) + fabs(c_L)));
            hs = fmin(hs, a.h / (fabs(R.u) + fabs(c_R)));
            if (a.order == 2) {
                // ifvar_check dim 1 aborts the run (grp_solver_EUL_source.c:193-197)
                bool bad = L.p < eps || R.p < eps || L.rho < eps || R.rho < eps || !M<double>::finite_(L.sp) ||
                           !M<double>::finite_(R.sp) || !M<double>::finite_(L.su) || !M<double>::finite_(R.su) ||
                           !M<double>::finite_(L.srho) || !M<double>::finite_(R.srho);
                if (bad)
                    ab = 1;
            }
            double D[3], U[3];
            int it;
            grp1d_solve(L, R, a.G, a.order == 1 ? (double)INFINITY : eps, D, U, it);
            if (it >= 0) {
                nfaces++;
                niters += it;
            }
            // star_dire_check dim 1, el = 0
            if (U[2] < eps || U[0] < eps || !M<double>::finite_(U[1]) || !M<double>::finite_(U[2]) ||
                !M<double>::finite_(U[0]) || !M<double>::finite_(D[1]) || !M<double>::finite_(D[2]) ||
                !M<double>::finite_(D[0]))
                st = 1;
            if (a.order == 1) {
                double Fr = U[0] * U[1];
                a.F[j] = Fr;
                a.F[(m + 1) + j] = Fr * U[1] + U[2];
                double Fe = a.G.g_g1 * U[2] + 0.5 * Fr * U[1];
                a.F[2 * (m + 1) + j] = Fe * U[1];
            } else {
                for (int q = 0; q < 3; ++q) {
                    a.mid[q * (m + 1) + j] = U[q];
                    a.dire[q * (m + 1) + j] = D[q];
                }
            }
        }
        // block reductions: min of h/S, OR of the flags
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
        cl.sync();  // partials of every CTA, and the faces' mid/dire/F, are now visible
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
            tau = a.cfl * hsm;
            if (tau < eps)
                stop_t = 1;
            else if ((time_c + tau) > (a.t_all - eps))
                tau = a.t_all - time_c;
            else if (!isfinite(tau)) {
                halted = 1;
                break;
            }
        }
        const double nu = tau / a.h;
        if (a.order == 2) {
            for (int j = gtid; j <= m; j += GNT) {
                double r = a.mid[j], u = a.mid[(m + 1) + j], p = a.mid[2 * (m + 1) + j];
                const double dr = a.dire[j], du = a.dire[(m + 1) + j], dp = a.dire[2 * (m + 1) + j];
                r += 0.5 * tau * dr;
                u += 0.5 * tau * du;
                p += 0.5 * tau * dp;
                double Fr = r * u;
                a.F[j] = Fr;
                a.F[(m + 1) + j] = Fr * u + p;
                double Fe = a.G.g_g1 * p + 0.5 * Fr * u;
                a.F[2 * (m + 1) + j] = Fe * u;
                r += 0.5 * tau * dr;
                u += 0.5 * tau * du;
                p += 0.5 * tau * dp;
                a.mid[j] = r;
                a.mid[(m + 1) + j] = u;
                a.mid[2 * (m + 1) + j] = p;
            }
            cl.sync();  // the update reads both faces of a cell, possibly computed by another CTA
        }
        int bad = 0;
        for (int j = gtid; j < m; j += GNT) {
            double Mom = rho[j] * uu[j] - nu * (a.F[(m + 1) + j + 1] - a.F[(m + 1) + j]);
            double Ene = rho[j] * ee[j] - nu * (a.F[2 * (m + 1) + j + 1] - a.F[2 * (m + 1) + j]);
            double r = rho[j] - nu * (a.F[j + 1] - a.F[j]);
            rho[j] = r;
            uu[j] = Mom / r;
            ee[j] = Ene / r;
            pp[j] = (Ene - 0.5 * Mom * uu[j]) * a.G.gm1;
            if (pp[j] < eps || r < eps)
                bad = 1;
            if (a.order == 2) {
                s_u[j] = dh(a.mid[(m + 1) + j + 1] - a.mid[(m + 1) + j], a);
                s_p[j] = dh(a.mid[2 * (m + 1) + j + 1] - a.mid[2 * (m + 1) + j], a);
                s_rho[j] = dh(a.mid[j + 1] - a.mid[j], a);
            }
        }
        bad = __syncthreads_or(bad);
        if (tid == 0)
            part_bad[par] = bad;
        cl.sync();  // also publishes this step's state to every CTA
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
        unsigned long long F = 0, I = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            F += sf[w];
            I += si[w];
        }
        cf = F;
        ci = I;
    }
    cl.sync();
    if (rank == 0 && tid == 0) {
        unsigned long long F = 0, I = 0;
        for (int r = 0; r < CL; ++r) {
            F += *cl.map_shared_rank(&cf, r);
            I += *cl.map_shared_rank(&ci, r);
        }
        a.out[0] = k;
        a.out[1] = nt;
        a.out[2] = time_c;
        a.out[3] = tau;
        a.out[4] = halted;
        a.out[5] = (double)F;
        a.out[6] = (double)I;
    }
    cl.sync();  // no CTA leaves while rank 0 still reads its shared memory
}

// Launch shape of the 1D loop: one warp-multiple of threads per CTA and as
// many CTAs (one cluster, at most 16) as give every interface its own thread,
// so the exact solves of a step spread over up to 16 SMs.
static cudaError_t launch_run1d(const Run1DArgs& a, cudaStream_t st)
{
    // the non-portable cluster size is a per-device attribute of the kernel:
    // set it on each device's first launch (0 = not tried, 1 = set, 2 = refused)
    enum { MAX_DEVICES = 64 };
    static std::atomic<int> attr_state[MAX_DEVICES];
    int dev = 0;
    cudaGetDevice(&dev);
    int attr_set = 0;
    if (dev >= 0 && dev < MAX_DEVICES) {
        int st0 = attr_state[dev].load(std::memory_order_acquire);
        if (st0 == 0) {
            st0 = cudaFuncSetAttribute(k_run1d, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess ? 1 : 2;
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
        cudaError_t e = cudaLaunchKernelEx(&lc, k_run1d, a);
        if (e == cudaSuccess || cl == 1)
            return e;
        cudaGetLastError();  // a cluster this size cannot be placed: halve it
        cl = (cl + 1) / 2;
        nt = 32 * ((faces + 32 * cl - 1) / (32 * cl));
        if (nt > 512)
            nt = 512;
    }
}

// Runs one 1D problem.  state: [4][m] rho,u,p,E in (CV.*[0]) and the final
// state out; snaps: [n_plot][4][m] host snapshot slots (may be null when n_plot == 2).
// Fills the kernel arguments from config[] semantics; -2 for an unknown boundary code.
static int prepare_args(Run1DArgs& a, int m, int order, const double* cfg, int ncfg, int n_plot)
{
    auto at = [&](int k) { return k < ncfg ? cfg[k] : INFINITY; };
    memset(&a, 0, sizeof(a));
    a.m = m;
    a.order = order;
    a.N = (int)at(5);
    a.bound = (int)at(17);
    a.n_plot = n_plot;
    a.t_all = at(1);
    a.eps = at(4);
    a.cfl = at(7);
    a.h = at(10);
    a.cfg16 = at(16);
    a.alpha = at(41);
    {
        int e;
        double f = frexp(a.h, &e);
        a.pow2 = (a.h > 0.0 && f == 0.5);
        a.inv_h = 1.0 / a.h;
    }
    if (a.bound != -1 && a.bound != -2 && a.bound != -4 && a.bound != -7 && a.bound != -24) {
        set_error("No suitable boundary conditions in x direction");
        return -2;
    }
    double g = at(6), zeta = (g - 1.0) / (g + 1.0);
    Gas<double>& G = a.G;
    G.g = g; G.gm1 = g - 1.0; G.zeta = zeta; G.mu = (g - 1.0) / (2.0 * g); G.nu = (g + 1.0) / (2.0 * g);
    G.g_g1 = g / (g - 1.0); G.inv_g = 1.0 / g; G.cexp = 0.5 * (g - 1.0) / g; G.sexp = 2.0 * g / (g - 1.0);
    G.e1 = 0.5 / zeta; G.e2 = (1.0 + zeta) / zeta; G.opz = 1.0 + zeta; G.op2z = 1.0 + 2.0 * zeta;
    G.eps = a.eps; G.g64 = g; G.eps64 = a.eps;
    return 0;
}

static void info_from(const double o[8], hydro_run_info* info)
{
    info->k_out = (int)o[0];
    info->time = o[2];
    info->tau = o[3];
    info->halted = (int)o[4];
    info->newton_faces = (unsigned long long)o[5];
    info->newton_iters = (unsigned long long)o[6];
    info->sweeps_launched = 1;
}

// Runs one 1D problem.  state: [4][m] rho,u,p,E in (CV.*[0]) and the final
// state out; snaps: [n_plot][4][m] host snapshot slots (may be null when n_plot == 2).
static int run1d(int m, int order, const double* cfg, int ncfg, double* state, const double* time_plot, int n_plot,
                 double* snaps_host, hydro_run_info* info, int* nt_out)
{
    memset(info, 0, sizeof(*info));
    Run1DArgs a;
    int prc = prepare_args(a, m, order, cfg, ncfg, n_plot);
    if (prc)
        return prc;
    size_t need = 4 * (size_t)m * 2 + (size_t)n_plot * 4 * m + n_plot + 3 * (size_t)m + 9 * (size_t)(m + 1) + 8;
    double* mem = nullptr;
    if (!cuda_ok(cudaMalloc(&mem, need * sizeof(double)), "1D buffers")) return -1;
    double* init = mem;
    double* cur = init + 4 * (size_t)m;
    double* snaps = cur + 4 * (size_t)m;
    double* tp = snaps + (size_t)n_plot * 4 * m;
    double* s = tp + n_plot;
    double* mid = s + 3 * (size_t)m;
    double* dire = mid + 3 * (size_t)(m + 1);
    double* F = dire + 3 * (size_t)(m + 1);
    double* out = F + 3 * (size_t)(m + 1);
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = 0;
    if (!cuda_ok(cudaMemcpyAsync(init, state, 4 * m * sizeof(double), cudaMemcpyHostToDevice, st), "1D upload") ||
        !cuda_ok(cudaMemcpyAsync(cur, state, 4 * m * sizeof(double), cudaMemcpyHostToDevice, st), "1D upload") ||
        !cuda_ok(cudaMemcpyAsync(tp, time_plot, n_plot * sizeof(double), cudaMemcpyHostToDevice, st), "1D upload") ||
        !cuda_ok(cudaMemsetAsync(s, 0, 3 * m * sizeof(double), st), "1D clear"))
        rc = -1;
    if (!rc) {
        a.init = init; a.cur = cur; a.snaps = snaps; a.time_plot = tp; a.s = s; a.mid = mid; a.dire = dire; a.F = F;
        a.out = out;
        cudaEventRecord(e0, st);
        if (!cuda_ok(launch_run1d(a, st), "1D launch")) rc = -1;
        count_launch();
        cudaEventRecord(e1, st);
    }
    double o[8] = {0};
    if (!rc && (!cuda_ok(cudaMemcpyAsync(o, out, 7 * sizeof(double), cudaMemcpyDeviceToHost, st), "1D result") ||
                !cuda_ok(cudaMemcpyAsync(state, cur, 4 * m * sizeof(double), cudaMemcpyDeviceToHost, st), "1D download") ||
                !cuda_ok(cudaStreamSynchronize(st), "1D run")))
        rc = -1;
    int nt = (int)o[1];
    if (!rc && snaps_host && nt > 0)
        if (!cuda_ok(cudaMemcpy(snaps_host, snaps, (size_t)nt * 4 * m * sizeof(double), cudaMemcpyDeviceToHost), "1D snaps"))
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
    info_from(o, info);
    info->gpu_ms = ms;
    *nt_out = nt;
    return 0;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the 1D run.
//
// Some callers cannot allocate device memory: frameworks that own the whole
// device pool through their own allocator (a cudaMalloc behind its back can
// fail or fragment the pool it has reserved), or embedded drivers whose memory
// budget is fixed at start-up.  For them the
// scratch of the 1D kernel (copy of the initial state, one snapshot slot,
// slopes, interface values, time derivatives, fluxes, result words) lives in
// the file-scope array below, sized for at most HYDRO1D_NOALLOC_MAX_CELLS
// cells: 20*m + 19 doubles, 2.6 MB at the limit, held by every GPU that loads
// the library until the process exits.
//
// Host code cannot use the array's name as a device address (it names a
// host-side stand-in), so the device address is looked up with
// cudaGetSymbolAddress once per device, on the first call made on that device
// with that device current, and cached per device.  Every call shares the one
// array and it keeps the previous call's contents: the slopes and result words
// are cleared on each call, and calls that overlap on the GPU (several
// streams, several host threads) race on it, so a caller must serialise them.
// The call copies its time-plot pair in from and its result words out to host
// memory and waits for its stream before it returns.
// ---------------------------------------------------------------------------
#define HYDRO1D_NOALLOC_MAX_CELLS 16384
#define HYDRO1D_NOALLOC_DOUBLES (20 * HYDRO1D_NOALLOC_MAX_CELLS + 19)

static __device__ __align__(256) double g_noalloc_scratch[HYDRO1D_NOALLOC_DOUBLES];

static double* noalloc_scratch_address(int* err)
{
    enum { MAX_DEVICES = 64 };
    static std::atomic<double*> addr[MAX_DEVICES];
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice") || dev < 0 || dev >= MAX_DEVICES) {
        *err = -1;
        return nullptr;
    }
    double* a = addr[dev].load(std::memory_order_acquire);
    if (!a) {
        // two host threads may both look it up; they store the same address
        void* p = nullptr;
        if (!cuda_ok(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress")) {
            *err = -1;
            return nullptr;
        }
        a = (double*)p;
        addr[dev].store(a, std::memory_order_release);
    }
    return a;
}

static int run1d_noalloc(int m, double* d_state, const double* cfg, int ncfg, int order, cudaStream_t st,
                         hydro_run_info* info)
{
    memset(info, 0, sizeof(*info));
    if (m < 2 || m > HYDRO1D_NOALLOC_MAX_CELLS) {
        set_error("hydro1d_run_noalloc: m must be in [2, 16384] (fixed device scratch)");
        return -3;
    }
    if (!d_state) {
        set_error("hydro1d_run_noalloc: null state");
        return -3;
    }
    Run1DArgs a;
    int prc = prepare_args(a, m, order, cfg, ncfg, 2);
    if (prc)
        return prc;
    int err = 0;
    double* base = noalloc_scratch_address(&err);
    if (!base)
        return err;
    double* init = base;
    double* snaps = init + 4 * (size_t)m;
    double* tp = snaps + 4 * (size_t)m;
    double* s = tp + 2;
    double* mid = s + 3 * (size_t)m;
    double* dire = mid + 3 * (size_t)(m + 1);
    double* F = dire + 3 * (size_t)(m + 1);
    double* out = F + 3 * (size_t)(m + 1);
    double tph[2] = {0.0, a.t_all};
    if (!cuda_ok(cudaMemcpyAsync(init, d_state, 4 * m * sizeof(double), cudaMemcpyDeviceToDevice, st), "noalloc copy") ||
        !cuda_ok(cudaMemcpyAsync(tp, tph, 2 * sizeof(double), cudaMemcpyHostToDevice, st), "noalloc copy") ||
        !cuda_ok(cudaMemsetAsync(s, 0, 3 * m * sizeof(double), st), "noalloc clear") ||
        !cuda_ok(cudaMemsetAsync(out, 0, 8 * sizeof(double), st), "noalloc clear"))
        return -1;
    a.init = init; a.cur = d_state; a.snaps = snaps; a.time_plot = tp; a.s = s; a.mid = mid; a.dire = dire; a.F = F;
    a.out = out;
    if (!cuda_ok(launch_run1d(a, st), "noalloc launch"))
        return -1;
    count_launch();
    double o[8];
    if (!cuda_ok(cudaMemcpyAsync(o, out, 8 * sizeof(double), cudaMemcpyDeviceToHost, st), "noalloc result") ||
        !cuda_ok(cudaStreamSynchronize(st), "noalloc run"))
        return -1;
    info_from(o, info);
    return 0;
}

static void entry_1d(const int m, struct cell_var_stru CV, double* cpu_time, int* N_plot, double time_plot[], int order)
{
    std::vector<double> state(4 * (size_t)m);
    memcpy(&state[0], CV.RHO[0], m * sizeof(double));
    memcpy(&state[m], CV.U[0], m * sizeof(double));
    memcpy(&state[2 * m], CV.P[0], m * sizeof(double));
    memcpy(&state[3 * m], CV.E[0], m * sizeof(double));
    const int n_plot = *N_plot;
    std::vector<double> snaps((size_t)n_plot * 4 * m);
    hydro_run_info info;
    int nt = 0;
    int rc = run1d(m, order, config, N_CONF, state.data(), time_plot, n_plot, snaps.data(), &info, &nt);
    if (rc == -2) {
        printf("No suitable boundary coditions in x direction!\n");
        config[5] = 1.0;
        *N_plot = 1;
        time_plot[0] = 0.0;
        return;
    }
    if (rc) {
        fprintf(stderr, "hydro_gb300: 1D run failed: %s\n", hydro_gb300_last_error());
        exit(5);
    }
    for (int k = 1; k < nt; ++k) {  // slot 0 is the caller's initial data
        const double* sp = &snaps[(size_t)k * 4 * m];
        memcpy(CV.RHO[k], sp, m * sizeof(double));
        memcpy(CV.U[k], sp + m, m * sizeof(double));
        memcpy(CV.P[k], sp + 2 * m, m * sizeof(double));
        memcpy(CV.E[k], sp + 3 * m, m * sizeof(double));
    }
    memcpy(CV.RHO[nt], &state[0], m * sizeof(double));
    memcpy(CV.U[nt], &state[m], m * sizeof(double));
    memcpy(CV.P[nt], &state[2 * m], m * sizeof(double));
    memcpy(CV.E[nt], &state[3 * m], m * sizeof(double));
    printf("\nTime is up at time step %d.\n", info.k_out);
    printf("The cost of GPU time for 1D-%s Eulerian scheme for this problem is %g seconds.\n",
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

void Godunov_solver_EUL_source(const int m, struct cell_var_stru CV, double* cpu_time, int* N_plot, double time_plot[])
{
    entry_1d(m, CV, cpu_time, N_plot, time_plot, 1);
}

void GRP_solver_EUL_source(const int m, struct cell_var_stru CV, double* cpu_time, int* N_plot, double time_plot[])
{
    entry_1d(m, CV, cpu_time, N_plot, time_plot, 2);
}

int hydro1d_run_noalloc(int m, double* d_state, const double* cfg, int ncfg, int order, void* stream,
                        hydro_run_info* info)
{
    return run1d_noalloc(m, d_state, cfg, ncfg, order, (cudaStream_t)stream, info);
}

int hydro1d_run(int m, double* rho, double* u, double* p, double* E, const double* cfg, int ncfg, int order,
                hydro_run_info* info)
{
    std::vector<double> state(4 * (size_t)m);
    double g = ncfg > 6 ? cfg[6] : 1.4;
    for (int j = 0; j < m; ++j) {
        state[j] = rho[j];
        state[m + j] = u[j];
        state[2 * m + j] = p[j];
        // the 1D driver's energy (src/hydrocode_1D/hydrocode.c:235)
        state[3 * m + j] = E ? E[j] : 0.5 * u[j] * u[j] + p[j] / (g - 1.0) / rho[j];
    }
    double tp[2] = {0.0, ncfg > 1 ? cfg[1] : INFINITY};
    int nt = 0;
    int rc = run1d(m, order, cfg, ncfg, state.data(), tp, 2, nullptr, info, &nt);
    if (rc)
        return rc;
    for (int j = 0; j < m; ++j) {
        rho[j] = state[j];
        u[j] = state[m + j];
        p[j] = state[2 * m + j];
        if (E)
            E[j] = state[3 * m + j];
    }
    return 0;
}

}  // extern "C"
