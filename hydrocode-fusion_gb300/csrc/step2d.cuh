// step2d.cuh -- fused 2D GRP time-step kernels (one launch per step/sweep).
//
// Device layout (every field a plane, x-major like the reference's CV.X[j][i]):
//   value of cell (x = j, y = i) at plane[j*ld + i], 0 <= j < m, 0 <= i < n,
//   so y is the contiguous axis.  A state is 13 planes: rho, u, v, p, E, the
//   four x-slopes s_* and the four y-slopes t_* (the slopes are genuine state:
//   the next step's minmod3 limiter uses them).
//
// One CTA owns a TJ x TI tile of cells and, in one launch:
//   1. stages rho,u,v,p of the tile plus a 2-cell halo in shared memory,
//      applying the boundary condition to ghost cells
//      (bound_cond_slope_limiter_x.c:34-82, _y.c:34-82);
//   2. limits the x- and y-slopes of the tile plus a 1-cell halo
//      (minmod_limiter_2D_x, slope_limiter_2D_x.c:32-84; minmod_limiter,
//      slope_limiter.c:31-83) and sets the ghost slopes by the boundary rules
//      (bound_cond_slope_limiter_x.c:94-126, _y.c:94-126);
//   3. solves every x- and y-face of the tile once (flux_generator_x.c:40-163,
//      flux_generator_y.c:40-163, GRP_2D_flux) into shared memory;
//   4. updates the cells and writes the new slopes from the t+tau interface
//      values (grp_solver_2D_EUL_source.c:228-263).
// Halo cells are recomputed by the neighbouring CTAs; nothing is written in
// place, the state ping-pongs between two buffers.
//
// Errors never trap: each face's code (ifvar_check -> 1, star/derivative
// check -> 2) is folded into a 64-bit key (serial index of the face in the
// reference's loop order, code) with atomicMax, so the host sees exactly the
// code the reference's serial loop would return (the last failing face
// wins).  The next launch reads the previous launch's keys and stops the run
// the way the reference does (abort = discard the step, stop = keep it).
#pragma once

#include <type_traits>

#include "hydro_device.cuh"
#include "learned.cuh"
#include "tma.cuh"

namespace hydro {

// Error/halt control block, one per solver, in device memory.
struct Ctl {
    unsigned long long key[3][2];  // [slot][0 = x-faces, 1 = y-faces]
    unsigned int upd_bad[3];       // positivity failure of the update
    int halted_seq;                // sequence number of the launch whose flags halted the run (0 = none)
    int halt_kind;                 // 1 = abort (that launch is discarded), 2 = stop (kept)
    unsigned long long newton_faces;  // faces that ran the exact solver
    unsigned long long newton_iters;  // Newton iterations summed over those faces
    unsigned long long newton_fallbacks;  // FP32 forms: faces finished by the FP64 Newton iteration
    unsigned int wait_err;                // a bounded wait in a kernel gave up (the launch is invalid)
    unsigned int pad32;
    unsigned long long pad[2];
};

template <typename R>
struct StepArgs {
    int m, n, ld;
    size_t plane;          // elements per plane
    const R* src_w;        // 5 planes: rho u v p E (input state)
    R* dst_w;              // 5 planes (output state)
    const R* src_s;        // 4 planes x-slopes (previous step's)
    R* dst_s;
    const R* src_t;        // 4 planes y-slopes
    R* dst_t;
    const R* ghost0;       // boundary code -1: initial edge values [4][n] left, [4][n] right, [4][m] down, [4][m] up
    Gas<R> G;
    R tau, htau;           // face time step and its half
    R hx, hy, hhx, hhy;    // grid sizes and their halves
    R inv_hx, inv_hy;      // exact reciprocals (used only when the size is a power of two)
    int pow2_x, pow2_y;
    R nu, mu;              // tau/h_x and tau/h_y of the update
    R alpha;               // minmod parameter
    int bx, by;            // boundary codes
    int find_x, find_y;    // 0 on the first limiting of that direction (minmod2), then 1 (minmod3)
    Ctl* ctl;
    int seq;               // launch sequence number (1, 2, ...) of this sweep
    int split_kind;        // 0 unsplit; for split sweeps the direction is the template parameter
    int stats;             // count Newton faces / iterations
    const uint32_t* mlp_frag;  // learned form: packed BF16 network
    const float* mlp_prm;      // learned form: FP32 parameters (biases)
    const void* mlp_img;       // learned form: the network's shared-memory image (MlpShared) in global memory
};

// ---------------------------------------------------------------------------
// halting protocol
// ---------------------------------------------------------------------------

// Decision from a finished launch's flags: 0 continue, 1 abort, 2 stop.
__device__ __host__ inline int halt_decision(unsigned long long kx, unsigned long long ky, unsigned int ub)
{
    int cx = (int)(kx & 3ull), cy = (int)(ky & 3ull);
    if (cx == 1 || cy == 1)
        return 1;
    if (cx == 2 || cy == 2 || ub)
        return 2;
    return 0;
}

// Returns true if this launch must not run.  Thread (0,0) of block (0,0) also
// records the halt and clears the slot the next launch will write.
__device__ __forceinline__ bool halt_prologue(Ctl* ctl, int seq)
{
    volatile Ctl* c = ctl;
    bool first = (threadIdx.x == 0 && threadIdx.y == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0);
    if (c->halted_seq)
        return true;
    if (seq > 1) {
        int ps = (seq - 1) % 3;
        int d = halt_decision(c->key[ps][0], c->key[ps][1], c->upd_bad[ps]);
        if (d) {
            if (first) {
                c->halt_kind = d;
                c->halted_seq = seq - 1;
            }
            return true;
        }
    }
    if (first) {
        int ns = (seq + 1) % 3;
        c->key[ns][0] = 0ull;
        c->key[ns][1] = 0ull;
        c->upd_bad[ns] = 0u;
    }
    return false;
}

// ---------------------------------------------------------------------------
// boundary-aware load of rho,u,v,p of cell (j, i), possibly a ghost
// ---------------------------------------------------------------------------
template <typename R, class A>
__device__ __forceinline__ void load_prims(const A& a, int j, int i, R w[4])
{
    const int m = a.m, n = a.n;
    // periodic directions first: a wrapped halo cell is a real cell whose own
    // ghosts in the other direction follow that direction's boundary rule
    if (a.bx == -7 && (j < 0 || j >= m))
        j = j < 0 ? j + m : j - m;
    if (a.by == -7 && (i < 0 || i >= n))
        i = i < 0 ? i + n : i - n;
    bool outx = (j < 0 || j >= m), outy = (i < 0 || i >= n);
    int jj = j, ii = i;
    R su = R(1), sv = R(1);
    int g0 = -1;  // index into the -1 (initial value) ghost table
    if (outx) {
        jj = j < 0 ? 0 : m - 1;
        if (a.bx == -2 || (a.bx == -24 && j < 0))
            su = R(-1);
        if (a.bx == -1 && !outy)
            g0 = (j < 0 ? 0 : 4 * n) + i;  // left table, right table
    }
    if (outy) {
        ii = i < 0 ? 0 : n - 1;
        if (a.by == -2 || (a.by == -24 && i < 0))
            sv = R(-1);
        if (a.by == -1 && !outx)
            g0 = 8 * n + (i < 0 ? 0 : 4 * m) + j;  // down table, up table
    }
    jj = jj < 0 ? 0 : (jj >= m ? m - 1 : jj);
    ii = ii < 0 ? 0 : (ii >= n ? n - 1 : ii);
    if (outx && outy) {  // corners of two non-periodic boundaries are never used
        su = R(1);
        sv = R(1);
        g0 = -1;
    }
    if (g0 >= 0) {
        const int stride = (g0 < 8 * n) ? n : m;
        w[0] = a.ghost0[g0];
        w[1] = a.ghost0[g0 + stride];
        w[2] = a.ghost0[g0 + 2 * stride];
        w[3] = a.ghost0[g0 + 3 * stride];
        return;
    }
    const size_t o = (size_t)jj * a.ld + ii;
    w[0] = a.src_w[o];
    w[1] = su * a.src_w[a.plane + o];
    w[2] = sv * a.src_w[2 * a.plane + o];
    w[3] = a.src_w[3 * a.plane + o];
}

// Index of a cell for reading its previous slopes (wrapped for periodic
// boundaries, clamped otherwise: non-periodic ghosts' slopes are overridden).
template <class A>
__device__ __forceinline__ size_t slope_index(const A& a, int j, int i)
{
    int jj = j, ii = i;
    if (jj < 0 || jj >= a.m)
        jj = (a.bx == -7) ? (jj < 0 ? jj + a.m : jj - a.m) : (jj < 0 ? 0 : a.m - 1);
    if (ii < 0 || ii >= a.n)
        ii = (a.by == -7) ? (ii < 0 ? ii + a.n : ii - a.n) : (ii < 0 ? 0 : a.n - 1);
    jj = jj < 0 ? 0 : (jj >= a.m ? a.m - 1 : jj);
    ii = ii < 0 ? 0 : (ii >= a.n ? a.n - 1 : ii);
    return (size_t)jj * a.ld + ii;
}

template <typename R>
__device__ __forceinline__ R div_h(R d, R h, R inv_h, int pow2)
{
    return pow2 ? d * inv_h : d / h;
}

// one slope: centred differences sL, sR over h, limited
template <typename R>
__device__ __forceinline__ R limit(R wl, R wc, R wr, R h, R inv_h, int pow2, R alpha, int find, R sprev)
{
    R sL = div_h(wc - wl, h, inv_h, pow2);
    R sR = div_h(wr - wc, h, inv_h, pow2);
    return find ? minmod3(alpha * sL, alpha * sR, sprev) : minmod2(sL, sR);
}

// Error key of a face: (serial + 1) << 2 | code, max-reduced.
__device__ __forceinline__ void report_face(Ctl* ctl, int slot, int dir, unsigned long long serial, int code)
{
    if (code)
        atomicMax(&ctl->key[slot][dir], ((serial + 1ull) << 2) | (unsigned long long)code);
}

// FP32 form: a face whose GRP star state fails the positivity / finiteness
// check in FP32 arithmetic is solved again in FP64 from the same
// (FP32-reconstructed) sides; returns the face's error code (0, 1 or 2) as
// the FP64 solve sees it.  Out of line and called from a separate pass after
// the face passes: it runs on a handful of faces per run.
template <int RS>
static __device__ __noinline__ int solve_face_fp64_retry(const Side<float>& L, const Side<float>& Rr, double g,
                                                         double eps, double dist2_max, double tau, bool ydir,
                                                         FaceOut<float>& o)
{
    Gas<double> G;
    gas_fill(G, g, eps);
    G.dist2_max = dist2_max;
    Side<double> Ld, Rd;
    Ld.rho = L.rho; Ld.u = L.u; Ld.v = L.v; Ld.p = L.p;
    Ld.drho = L.drho; Ld.du = L.du; Ld.dv = L.dv; Ld.dp = L.dp;
    Ld.trho = L.trho; Ld.tu = L.tu; Ld.tv = L.tv; Ld.tp = L.tp;
    Rd.rho = Rr.rho; Rd.u = Rr.u; Rd.v = Rr.v; Rd.p = Rr.p;
    Rd.drho = Rr.drho; Rd.du = Rr.du; Rd.dv = Rr.dv; Rd.dp = Rr.dp;
    Rd.trho = Rr.trho; Rd.tu = Rr.tu; Rd.tv = Rr.tv; Rd.tp = Rr.tp;
    Star<double> S;
    StarInfo st;
    st.fallback = 0;
    q1d_star<double, 0, RS, false>(Ld, Rd, G, S, st, -1.0);
    double D[4], U[4];
    q1d_derivs<double, 0, RS>(Ld, Rd, G, S, D, U);
    const int bad = star_dire_check2(U, D, eps) ? 2 : (ifvar_bad(Ld, Rd, eps) ? 1 : 0);
    FaceOut<double> od;
    face_flux<double>(D, U, tau, 0.5 * tau, G, od, ydir);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        o.F[k] = (float)od.F[k];
        o.I[k] = (float)od.I[k];
    }
    return bad;
}

// Solve one face given its two sides in the face's normal frame (KNOWN as in
// q1d_star: whether the uniform-pair decision has already been made; RS: the
// interface solver, 0 = quasi-1D, 1 = genuinely 2D).
template <typename R, int KNOWN = 0, int RS = 0>
__device__ __forceinline__ int solve_face(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G, R tau, R htau,
                                          FaceOut<R>& o, int& iters, int& fallback, bool ydir, R p_start = R(-1))
{
    int code = ifvar_bad(L, Rr, G.eps) ? 1 : 0;
    Star<R> S;
    StarInfo st;
    st.fallback = 0;
    q1d_star<R, KNOWN, RS>(L, Rr, G, S, st, p_start);
    R D[4], U[4];
    q1d_derivs<R, KNOWN, RS>(L, Rr, G, S, D, U);
    iters = st.iters;
    fallback = st.fallback;
    if (star_dire_check2(U, D, G.eps))
        code = 2;
    face_flux<R>(D, U, tau, htau, G, o, ydir);
    return code;
}

// The learned start runs only on faces with a strong jump:
//   (dp / (pL + pR))^2 + du^2 / (gamma (pL/rhoL + pR/rhoR)) >= LEARNED_JUMP2_MIN
// (dp, du the pressure and velocity jumps; the second term is the squared
// velocity jump over the sound speeds' root-sum-square), decided with
// multiplications only.  Below it the tangent-intersection start of the FP32
// Newton iteration is within a few per cent of the root (its error is of second
// order in the jump) and converges in 0-1 iterations, which the network's start
// does not beat.  A strong jump is never a uniform pair (that threshold is a
// relative 1e-6).
constexpr float LEARNED_JUMP2_MIN = 0.005f;

// Learned starting pressure of the exact solver for every lane of the warp
// whose face has a strong jump (warp-collective: all 32 lanes call it; rows:
// only lanes below it are active; the network is not run at all, nor the sound
// speeds taken, when no lane needs it).  Returns -1 where no guess applies
// (weak jump, inactive lane, a pair that would generate vacuum, a non-finite
// prediction).
__device__ __forceinline__ bool learned_strong_jump(float rhoL, float uL, float pL, float rhoR, float uR, float pR,
                                                   float g, float jump2)
{
    const float sp = pL + pR, dp = pL - pR, du = uL - uR;
    const float w = g * (pL * rhoR + pR * rhoL);  // gamma (pL/rhoL + pR/rhoR) rhoL rhoR
    return dp * dp * w + du * du * (rhoL * rhoR) * (sp * sp) >= jump2 * (sp * sp) * w;
}

// The network's start for the lanes with need set (warp-collective, as below).
__device__ __forceinline__ float learned_start(const Side<float>& L, const Side<float>& Rr, bool need,
                                               const Gas<float>& G, const MlpShared& M, int rows);

__device__ __forceinline__ float learned_guess(const Side<float>& L, const Side<float>& Rr, bool active,
                                               const Gas<float>& G, const MlpShared& M, int rows)
{
    const bool need = active && learned_strong_jump(L.rho, L.u, L.p, Rr.rho, Rr.u, Rr.p, G.g, LEARNED_JUMP2_MIN);
    return learned_start(L, Rr, need, G, M, rows);
}

__device__ __forceinline__ float learned_start(const Side<float>& L, const Side<float>& Rr, bool need,
                                               const Gas<float>& G, const MlpShared& M, int rows)
{
    float pg = -1.f;
    if (__any_sync(0xffffffffu, need)) {
        const float cL = sqrtf(G.g * L.p / L.rho), cR = sqrtf(G.g * Rr.p / Rr.rho);
        float x[6];
        float pbar = mlp_features(L.rho, L.u, L.p, cL, Rr.rho, Rr.u, Rr.p, cR, x);
        if (!need)
#pragma unroll
            for (int k = 0; k < 6; ++k)
                x[k] = 0.f;
        const float y = warp_mlp_outline(x[0], x[1], x[2], x[3], x[4], x[5], &M, rows);
        const bool vac = (Rr.u - L.u) >= 0.9f * 2.f * (cL + cR) / G.gm1;
        const float p = pbar * __expf(y);
        if (need && !vac && p > 0.f && p < INFINITY)
            pg = p;
    }
    return pg;
}
template <typename R>
__device__ __forceinline__ R learned_guess_any(const Side<R>& L, const Side<R>& Rr, bool active, const Gas<R>& G,
                                               const MlpShared& M, int rows);
template <>
__device__ __forceinline__ float learned_guess_any<float>(const Side<float>& L, const Side<float>& Rr, bool active,
                                                          const Gas<float>& G, const MlpShared& M, int rows)
{
    return learned_guess(L, Rr, active, G, M, rows);
}
template <>
__device__ __forceinline__ double learned_guess_any<double>(const Side<double>&, const Side<double>&, bool,
                                                            const Gas<double>&, const MlpShared&, int)
{
    return -1.0;
}

// ---------------------------------------------------------------------------
// unsplit step: grp_solver_2D_EUL_source.c:146-286
// ---------------------------------------------------------------------------
template <typename R, int TJ, int TI>
struct UnsplitSmem {
    static constexpr int WJ = TJ + 4, WI = TI + 4;  // values with a 2-cell halo
    static constexpr int SJ = TJ + 2, SI = TI + 2;  // slopes with a 1-cell halo
    static constexpr int nW = 4 * WJ * WI;
    static constexpr int nS = 8 * SJ * SI;
    static constexpr int nFX = 8 * (TJ + 1) * TI;
    static constexpr int nFY = 8 * TJ * (TI + 1);
    static constexpr int nQ = (TJ + 1) * TI + TJ * (TI + 1);  // queue of faces for the exact solver
    static constexpr size_t bytes_f = sizeof(R) * (size_t)(nW + nS + nFX + nFY);
    static constexpr size_t bytes = bytes_f + (2 * (size_t)nQ + 15) / 16 * 16;
    // the learned form appends the network image
    static constexpr size_t mlp_off = (bytes + 15) / 16 * 16;
    static constexpr size_t bytes_learned = mlp_off + sizeof(MlpShared);
};

// Shared-memory stage of one tile's TMA copy: box A = 5 value planes
// (rho u v p E) x rows J0-2 .. J0+TJ+1 x columns I0-X .. I0-X+BW-1, box B = 8
// previous-slope planes x rows J0-1 .. J0+TJ x the same columns.  X is 16
// bytes of elements, so every copy starts on a 16-byte column boundary.
template <typename R, int TJ, int TI>
struct StageLayout {
    static constexpr int X = 16 / (int)sizeof(R);
    static constexpr int BW = TI + 2 * X;
    static constexpr int AJ = TJ + 4, BJ = TJ + 2;
    static constexpr size_t a_bytes = sizeof(R) * 5 * AJ * BW;
    static constexpr size_t b_bytes = sizeof(R) * 8 * BJ * BW;
    static constexpr size_t a_off = 0, b_off = (a_bytes + 127) / 128 * 128;
    static constexpr size_t bytes = b_off + (b_bytes + 127) / 128 * 128;  // one stage
};

// One TJ x TI tile (cells i in [I0, I0+TI), j in [J0, J0+TJ)) of the unsplit
// step, computed by a block of NT threads.  Ends with a block barrier, so the
// shared memory can be reused for the next tile at once.
//   STAGED = false: the tile gathers its values (with boundary ghosts) from
//     global memory into W (pitch TI+4) itself; used by the one-problem kernel
//     k_step_unsplit and by the batched kernels.
//   STAGED = true: a TMA copy has already placed the 5 value planes (rows
//     J0-2.., columns I0-X.., pitch BW) at W and the 8 previous-slope planes
//     (rows J0-1.., same columns) at B; only the ghost cells of tiles at the
//     domain edge are gathered.  FX may alias B (B is dead after phase 2).
// Four consecutive values of a tile's shared-memory 4-vectors (16-byte aligned):
// one 16-byte shared load or store in FP32, two in FP64.
template <typename R>
struct Quad {
    R a, b, c, d;
    __device__ __forceinline__ R operator[](int k) const { return k == 0 ? a : (k == 1 ? b : (k == 2 ? c : d)); }
};
__device__ __forceinline__ Quad<float> lds4(const float* p)
{
    const float4 t = *reinterpret_cast<const float4*>(p);
    return {t.x, t.y, t.z, t.w};
}
__device__ __forceinline__ Quad<double> lds4(const double* p)
{
    const double2 t0 = reinterpret_cast<const double2*>(p)[0], t1 = reinterpret_cast<const double2*>(p)[1];
    return {t0.x, t0.y, t1.x, t1.y};
}
__device__ __forceinline__ void sts4(float* p, float a, float b, float c, float d)
{
    *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void sts4(double* p, double a, double b, double c, double d)
{
    reinterpret_cast<double2*>(p)[0] = make_double2(a, b);
    reinterpret_cast<double2*>(p)[1] = make_double2(c, d);
}

template <typename R, int TJ, int TI, int NT, bool LEARNED, bool STAGED, int RS = 0>
__device__ __forceinline__ void tile_body(const StepArgs<R>& a, const Gas<R>& G, const int I0, const int J0,
                                          R* __restrict__ W,
                                          const R* B, R* __restrict__ S, R* FX, R* __restrict__ FY,
                                          unsigned short* __restrict__ Q, const MlpShared& Mlp,
                                          bool last_tile = false)
{
    static_assert(!(LEARNED && RS != 0), "the learned start is built for the quasi-1D interface solver");
    using SM = UnsplitSmem<R, TJ, TI>;
    using SL = StageLayout<R, TJ, TI>;
    const int tid = threadIdx.x;
    const int m = a.m, n = a.n, slot = a.seq % 3;
    constexpr int WJ = SM::WJ, SJ = SM::SJ, SI = SM::SI;
    // face queue and FP32 retry list (read only after the barriers below;
    // the previous tile finished with them at its final barrier)
    __shared__ int s_qn;
    constexpr int RETRY_MAX = 128;  // FP32 faces whose star state failed its check, redone in FP64
    __shared__ int s_nretry;
    __shared__ unsigned short s_retry[RETRY_MAX];
    if (tid == 0) {
        s_qn = 0;
        s_nretry = 0;
    }
    // value (lj, li) = cell (J0-2+lj, I0-2+li)
    constexpr int WP = STAGED ? SL::BW : SM::WI;
    constexpr int WO = STAGED ? SL::X - 2 : 0;
    // W of a TMA-staged tile planar (plane, row, column), as the boxes deliver
    // it, and of a gathered tile one 4-vector (rho u v p) per cell; S, FX and FY
    // as two planes of 4-vectors per cell or face (x-slopes | y-slopes,
    // fluxes | t+tau interface values), so that the four components a side or a
    // face needs are one vector access (lds4 / sts4)
#define Wx(k, lj, li) (STAGED ? W[((k) * WJ + (lj)) * WP + (li) + WO] : W[((lj) * SM::WI + (li)) * 4 + (k)])
#define W4(lj, li) (W + ((lj) * SM::WI + (li)) * 4)
#define S4(p, sj, si) (S + (((p) * SJ + (sj)) * SI + (si)) * 4)
#define FX4(p, fj, fi) (FX + (((p) * (TJ + 1) + (fj)) * TI + (fi)) * 4)
#define FY4(p, gj, gi) (FY + (((p) * TJ + (gj)) * (TI + 1) + (gi)) * 4)
#define Sx(k, sj, si) S4((k) >> 2, sj, si)[(k) & 3]
#define FXx(k, fj, fi) FX4((k) >> 2, fj, fi)[(k) & 3]
#define FYx(k, gj, gi) FY4((k) >> 2, gj, gi)[(k) & 3]

    // rho u v p of value cell (lj, li)
    auto wq = [&](int lj, int li) -> Quad<R> {
        if constexpr (STAGED)
            return {Wx(0, lj, li), Wx(1, lj, li), Wx(2, lj, li), Wx(3, lj, li)};
        else
            return lds4(W4(lj, li));
    };

    // a tile whose halo lies inside the grid reads its cells directly (no
    // boundary rule applies to any of them); block-uniform
    const bool interior = J0 >= 2 && I0 >= 2 && J0 + TJ + 2 <= m && I0 + TI + 2 <= n;

    // 1. values with a 2-cell halo (staged: only the ghosts of edge tiles)
    constexpr int WI = SM::WI;
    if (!STAGED || !interior) {
        for (int idx = tid; idx < WJ * WI; idx += NT) {
            int lj = idx / WI, li = idx - lj * WI;
            const int j = J0 - 2 + lj, i = I0 - 2 + li;
            if (STAGED && j >= 0 && j < m && i >= 0 && i < n)
                continue;
            R w[4];
            if (!STAGED && interior) {
                const size_t o = (size_t)j * a.ld + i;
                w[0] = a.src_w[o];
                w[1] = a.src_w[a.plane + o];
                w[2] = a.src_w[2 * a.plane + o];
                w[3] = a.src_w[3 * a.plane + o];
            } else {
                load_prims(a, j, i, w);
            }
            if constexpr (STAGED) {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    Wx(k, lj, li) = w[k];
            } else {
                sts4(W4(lj, li), w[0], w[1], w[2], w[3]);
            }
        }
        __syncthreads();  // (an interior staged tile wrote nothing here)
    }

    // 2. limited slopes of the tile and a 1-cell halo; the 4 corners are never
    //    used, so the (SJ SI - 4) cells are enumerated without them: first and
    //    last halo rows without their end cells, the SJ - 2 full rows between
    constexpr int NSL = SJ * SI - 4;
    constexpr int ROUNDS2 = (NSL + NT - 1) / NT;
    // constant trip count, unrolled: the rounds' loads and limiter chains interleave
#pragma unroll
    for (int rr = 0; rr < ROUNDS2; ++rr) {
        const int idx = tid + rr * NT;
        if (idx >= NSL)
            break;
        int sj, si;
        if (idx < SI - 2) {
            sj = 0;
            si = idx + 1;
        } else if (idx < SI - 2 + (SJ - 2) * SI) {
            const int r = idx - (SI - 2);
            sj = 1 + r / SI;
            si = r - (sj - 1) * SI;
        } else {
            sj = SJ - 1;
            si = 1 + idx - (SI - 2) - (SJ - 2) * SI;
        }
        int j = J0 - 1 + sj, i = I0 - 1 + si;
        const bool inside = STAGED && j >= 0 && j < m && i >= 0 && i < n;
        size_t o = 0;  // global index of the previous slopes, needed only when they are not staged
        if (!STAGED && interior)
            o = (size_t)j * a.ld + i;
        else if (!inside)
            o = slope_index(a, j, i);
        // staged previous slopes: plane k at B[(k * BJ + sj) * BW + si - 1 + X]
        const R* bs = STAGED ? B + sj * SL::BW + si - 1 + SL::X : nullptr;
        R sxv[4], syv[4];
        // the centre and its four neighbours along x (rows) and y (columns)
        const Quad<R> wc = wq(sj + 1, si + 1), wxm = wq(sj, si + 1), wxp = wq(sj + 2, si + 1);
        const Quad<R> wym = wq(sj + 1, si), wyp = wq(sj + 1, si + 2);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            R ps = R(0), pt = R(0);
            if (a.find_x)
                ps = inside ? bs[k * SL::BJ * SL::BW] : a.src_s[k * a.plane + o];
            if (a.find_y)
                pt = inside ? bs[(4 + k) * SL::BJ * SL::BW] : a.src_t[k * a.plane + o];
            R sx = limit(wxm[k], wc[k], wxp[k], a.hx, a.inv_hx, a.pow2_x, a.alpha, a.find_x, ps);
            R sy = limit(wym[k], wc[k], wyp[k], a.hy, a.inv_hy, a.pow2_y, a.alpha, a.find_y, pt);
            sxv[k] = sx;
            syv[k] = sy;
        }
        sts4(S4(0, sj, si), sxv[0], sxv[1], sxv[2], sxv[3]);
        sts4(S4(1, sj, si), syv[0], syv[1], syv[2], syv[3]);
    }
    __syncthreads();

    // 2b. ghost slopes at non-periodic domain edges (edge tiles only)
    const bool ghost_x = a.bx != -7 && (J0 == 0 || m - J0 + 1 <= SJ - 1);
    const bool ghost_y = a.by != -7 && (I0 == 0 || n - I0 + 1 <= SI - 1);
    if (ghost_x) {
        const int sjg[2] = {(J0 == 0) ? 0 : -1, (m - J0 + 1 <= SJ - 1) ? m - J0 + 1 : -1};
        for (int idx = tid; idx < 2 * TI; idx += NT) {
            int side = idx / TI, si = 1 + idx % TI;
            int sj = sjg[side];
            if (sj < 0)
                continue;
            int se = side == 0 ? sj + 1 : sj - 1;  // edge cell
            // normal slopes: reflective keeps the edge's u-slope only (left side for -24)
            bool keep_su = (a.bx == -2) || (a.bx == -24 && side == 0);
            Sx(0, sj, si) = R(0);
            Sx(1, sj, si) = keep_su ? Sx(1, se, si) : R(0);
            Sx(2, sj, si) = R(0);
            Sx(3, sj, si) = R(0);
            // transversal slopes: edge cell's, zero for the fixed initial boundary
#pragma unroll
            for (int k = 0; k < 4; ++k)
                Sx(4 + k, sj, si) = (a.bx == -1) ? R(0) : Sx(4 + k, se, si);
        }
    }
    if (ghost_y) {
        const int sig[2] = {(I0 == 0) ? 0 : -1, (n - I0 + 1 <= SI - 1) ? n - I0 + 1 : -1};
        for (int idx = tid; idx < 2 * TJ; idx += NT) {
            int side = idx / TJ, sj = 1 + idx % TJ;
            int si = sig[side];
            if (si < 0)
                continue;
            int se = side == 0 ? si + 1 : si - 1;
            bool keep_tv = (a.by == -2) || (a.by == -24 && side == 0);
            Sx(4, sj, si) = R(0);
            Sx(5, sj, si) = R(0);
            Sx(6, sj, si) = keep_tv ? Sx(6, sj, se) : R(0);
            Sx(7, sj, si) = R(0);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                Sx(k, sj, si) = (a.by == -1) ? R(0) : Sx(k, sj, se);
        }
    }
    if (ghost_x || ghost_y)
        __syncthreads();

    // 3. faces, in two passes.  Pass A reconstructs every face: a pair within
    //    the uniform threshold (the acoustic case of the GRP solver) is
    //    solved at once, any other face goes to a shared-memory queue.  Pass B
    //    solves the queued faces 32 to a warp, so the exact Riemann solver
    //    (and the learned network) run on full warps instead of on the one or
    //    two lanes of a warp that need them while the rest idle.  Every face is
    //    computed by the same solve_face in either pass, so the split changes
    //    no result.
    constexpr int NFX = (TJ + 1) * TI, NFY = TJ * (TI + 1), NF = NFX + NFY;
    int my_iters = 0, my_newton = 0, my_fb = 0;
    const int lane = tid & 31;
    // sides of face f (x-faces first, then y-faces) in the face's normal frame;
    // false when the face lies outside the domain
    auto sides = [&](int f, Side<R>& L, Side<R>& Rr, int& lj, int& li, int& j, int& i) -> bool {
        if (f < NFX) {
            const int fj = f / TI, fi = f - fj * TI;
            lj = fj; li = fi;
            j = J0 + fj; i = I0 + fi;
            // left cell (j-1): slopes at (fj, fi+1), values at (fj+1, fi+2)
            {
                const Quad<R> d = lds4(S4(0, fj, fi + 1)), t = lds4(S4(1, fj, fi + 1));
                L.drho = d.a; L.du = d.b; L.dv = d.c; L.dp = d.d;
                L.trho = t.a; L.tu = t.b; L.tv = t.c; L.tp = t.d;
            }
            {
                const Quad<R> w = wq(fj + 1, fi + 2);
                L.rho = w.a + a.hhx * L.drho;
                L.u = w.b + a.hhx * L.du;
                L.v = w.c + a.hhx * L.dv;
                L.p = w.d + a.hhx * L.dp;
            }
            {
                const Quad<R> d = lds4(S4(0, fj + 1, fi + 1)), t = lds4(S4(1, fj + 1, fi + 1));
                Rr.drho = d.a; Rr.du = d.b; Rr.dv = d.c; Rr.dp = d.d;
                Rr.trho = t.a; Rr.tu = t.b; Rr.tv = t.c; Rr.tp = t.d;
            }
            {
                const Quad<R> w = wq(fj + 2, fi + 2);
                Rr.rho = w.a - a.hhx * Rr.drho;
                Rr.u = w.b - a.hhx * Rr.du;
                Rr.v = w.c - a.hhx * Rr.dv;
                Rr.p = w.d - a.hhx * Rr.dp;
            }
            return !(j > m || i >= n);
        }
        const int g = f - NFX;
        const int gj = g / (TI + 1), gi = g - gj * (TI + 1);
        lj = gj; li = gi;
        j = J0 + gj; i = I0 + gi;
        // lower cell (i-1): slopes at (gj+1, gi), values at (gj+2, gi+1); rotated to the +y normal frame:
        // normal velocity v, tangential -u; normal derivatives are the y-slopes, tangential the negated x-slopes
        {
            const Quad<R> tq = lds4(S4(1, gj + 1, gi)), sq = lds4(S4(0, gj + 1, gi));
            R t0 = tq.a, t1 = tq.b, t2 = tq.c, t3 = tq.d;
            R s0 = sq.a, s1 = sq.b, s2 = sq.c, s3 = sq.d;
            const Quad<R> w = wq(gj + 2, gi + 1);
            R rr = w.a + a.hhy * t0;
            R uu = w.b + a.hhy * t1;
            R vv = w.c + a.hhy * t2;
            R pp = w.d + a.hhy * t3;
            L.rho = rr; L.u = vv; L.v = -uu; L.p = pp;
            L.drho = t0; L.du = t2; L.dv = -t1; L.dp = t3;
            L.trho = -s0; L.tu = -s2; L.tv = s1; L.tp = -s3;
        }
        {
            const Quad<R> tq = lds4(S4(1, gj + 1, gi + 1)), sq = lds4(S4(0, gj + 1, gi + 1));
            R t0 = tq.a, t1 = tq.b, t2 = tq.c, t3 = tq.d;
            R s0 = sq.a, s1 = sq.b, s2 = sq.c, s3 = sq.d;
            const Quad<R> w = wq(gj + 2, gi + 2);
            R rr = w.a - a.hhy * t0;
            R uu = w.b - a.hhy * t1;
            R vv = w.c - a.hhy * t2;
            R pp = w.d - a.hhy * t3;
            Rr.rho = rr; Rr.u = vv; Rr.v = -uu; Rr.p = pp;
            Rr.drho = t0; Rr.du = t2; Rr.dv = -t1; Rr.dp = t3;
            Rr.trho = -s0; Rr.tu = -s2; Rr.tv = s1; Rr.tp = -s3;
        }
        return !(j >= m || i > n);
    };
    // solve face f and store its flux and time derivative
    auto solve_store = [&](auto known, int f, const Side<R>& L, const Side<R>& Rr, int lj, int li, int j, int i,
                           R p_start) {
        const bool ydir = f >= NFX;
        FaceOut<R> o;
        int it, fbk;
        int code = solve_face<R, decltype(known)::value, RS>(L, Rr, G, a.tau, a.htau, o, it, fbk, ydir, p_start);
        if (it >= 0) {
            my_newton++;
            my_iters += it;
            my_fb += fbk;
        }
        if (sizeof(R) == 4 && code == 2) {
            // FP32 star state failed its check: solve this face again in FP64 after the passes
            const int r = atomicAdd(&s_nretry, 1);
            if (r < RETRY_MAX) {
                s_retry[r] = (unsigned short)f;
                code = 0;  // reported by the retry
            }
        }
        if (!ydir) {
            report_face(a.ctl, slot, 0, (unsigned long long)i * (m + 1) + j, code);
            sts4(FX4(0, lj, li), o.F[0], o.F[1], o.F[2], o.F[3]);
            sts4(FX4(1, lj, li), o.I[0], o.I[1], o.I[2], o.I[3]);
        } else {
            report_face(a.ctl, slot, 1, (unsigned long long)j * (n + 1) + i, code);
            sts4(FY4(0, lj, li), o.F[0], o.F[1], o.F[2], o.F[3]);
            sts4(FY4(1, lj, li), o.I[0], o.I[1], o.I[2], o.I[3]);
        }
    };
    // pass A: warp-uniform rounds so the queue appends are warp-aggregated
    for (int fb = tid - lane; fb < NF; fb += NT) {
        const int f = fb + lane;
        Side<R> L, Rr;
        int lj = 0, li = 0, j = 0, i = 0;
        const bool active = f < NF && sides(f, L, Rr, lj, li, j, i);
        const bool uni = active && face_uniform<R, RS>(L, Rr, G);
        const bool need = active && !uni;
        const unsigned want = __ballot_sync(0xffffffffu, need);
        if (want) {
            int base = 0;
            if (lane == 0)
                base = atomicAdd(&s_qn, __popc(want));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (need)
                Q[base + __popc(want & ((1u << lane) - 1u))] = (unsigned short)f;
        }
        if (uni)
            solve_store(std::integral_constant<int, 1>(), f, L, Rr, lj, li, j, i, R(-1));
    }
    __syncthreads();
    // pass B: the queued faces, 32 per warp.  The learned form first runs the
    // network over the warp's 32 faces (warp-collective, tensor cores; one
    // 16-row tile when no more than 16 are queued) and then solves them; the
    // faces' sides are rebuilt after the network call, so the network and the
    // exact solver never hold their registers at the same time.
    const int qn = s_qn;
    for (int qb = tid - lane; qb < qn; qb += NT) {
        const int q = qb + lane;
        const bool act = q < qn;
        R p_start = R(-1);
        if constexpr (LEARNED) {
            Side<R> L, Rr;
            int lj = 0, li = 0, j = 0, i = 0;
            sides(act ? (int)Q[q] : 0, L, Rr, lj, li, j, i);
            p_start = learned_guess_any<R>(L, Rr, act, G, Mlp, qn - qb < 32 ? qn - qb : 32);
        }
        if (!act)
            break;
        const int f = (int)Q[q];
        Side<R> L, Rr;
        int lj = 0, li = 0, j = 0, i = 0;
        sides(f, L, Rr, lj, li, j, i);
        solve_store(std::integral_constant<int, 2>(), f, L, Rr, lj, li, j, i, p_start);
    }
    if (a.stats) {
        // warp-aggregated statistics
        __syncwarp();
        for (int off = 16; off; off >>= 1) {
            my_newton += __shfl_xor_sync(0xffffffffu, my_newton, off);
            my_iters += __shfl_xor_sync(0xffffffffu, my_iters, off);
            my_fb += __shfl_xor_sync(0xffffffffu, my_fb, off);
        }
        if ((tid & 31) == 0 && my_newton) {
            atomicAdd(&a.ctl->newton_faces, (unsigned long long)my_newton);
            atomicAdd(&a.ctl->newton_iters, (unsigned long long)my_iters);
            if (my_fb)
                atomicAdd(&a.ctl->newton_fallbacks, (unsigned long long)my_fb);
        }
    }
    if (qn > 0)  // (block-uniform) pass B wrote faces that phase 4 reads
        __syncthreads();
    if constexpr (sizeof(R) == 4) {
        const int nr = s_nretry < RETRY_MAX ? s_nretry : RETRY_MAX;
        if (nr > 0) {
            for (int r = tid; r < nr; r += NT) {
                const int f = (int)s_retry[r];
                Side<R> L, Rr;
                int lj = 0, li = 0, j = 0, i = 0;
                sides(f, L, Rr, lj, li, j, i);
                FaceOut<R> o;
                const bool ydir = f >= NFX;
                const int code = solve_face_fp64_retry<RS>(L, Rr, G.g64, G.eps64, G.dist2_max, (double)a.tau, ydir, o);
                if (!ydir) {
                    report_face(a.ctl, slot, 0, (unsigned long long)i * (m + 1) + j, code);
                    sts4(FX4(0, lj, li), o.F[0], o.F[1], o.F[2], o.F[3]);
                    sts4(FX4(1, lj, li), o.I[0], o.I[1], o.I[2], o.I[3]);
                } else {
                    report_face(a.ctl, slot, 1, (unsigned long long)j * (n + 1) + i, code);
                    sts4(FY4(0, lj, li), o.F[0], o.F[1], o.F[2], o.F[3]);
                    sts4(FY4(1, lj, li), o.I[0], o.I[1], o.I[2], o.I[3]);
                }
            }
            __syncthreads();
        }
    }

    // 4. conservative update and new slopes
    unsigned bad = 0;
    constexpr int ROUNDS4 = (TJ * TI + NT - 1) / NT;
#pragma unroll
    for (int rr = 0; rr < ROUNDS4; ++rr) {
        const int idx = tid + rr * NT;
        if (idx >= TJ * TI)
            break;
        int cj = idx / TI, ci = idx - cj * TI;
        int j = J0 + cj, i = I0 + ci;
        if (j >= m || i >= n)
            continue;
        const size_t o = (size_t)j * a.ld + i;
        const Quad<R> wcell = wq(cj + 2, ci + 2);
        R rho = wcell.a, uu = wcell.b, vv = wcell.c;
        R E;
        if constexpr (STAGED)
            E = Wx(4, cj + 2, ci + 2);
        else
            E = a.src_w[4 * a.plane + o];
        // fluxes of the cell's four faces (x: rows cj, cj+1; y: columns ci, ci+1)
        const Quad<R> fx0 = lds4(FX4(0, cj, ci)), fx1 = lds4(FX4(0, cj + 1, ci));
        const Quad<R> fy0 = lds4(FY4(0, cj, ci)), fy1 = lds4(FY4(0, cj, ci + 1));
        R mom_x = rho * uu - a.nu * (fx1.b - fx0.b) - a.mu * (fy1.b - fy0.b);
        R mom_y = rho * vv - a.nu * (fx1.c - fx0.c) - a.mu * (fy1.c - fy0.c);
        R ene = rho * E - a.nu * (fx1.d - fx0.d) - a.mu * (fy1.d - fy0.d);
        rho += -a.nu * (fx1.a - fx0.a) - a.mu * (fy1.a - fy0.a);
        R un = mom_x / rho, vn = mom_y / rho, En = ene / rho;
        R pn = (ene - R(0.5) * mom_x * un - R(0.5) * mom_y * vn) * G.gm1;
        if (pn < G.eps || rho < G.eps)
            bad = 1;
        a.dst_w[o] = rho;
        a.dst_w[a.plane + o] = un;
        a.dst_w[2 * a.plane + o] = vn;
        a.dst_w[3 * a.plane + o] = pn;
        a.dst_w[4 * a.plane + o] = En;
        {
            // new slopes from the faces' t+tau interface values
            const Quad<R> ix0 = lds4(FX4(1, cj, ci)), ix1 = lds4(FX4(1, cj + 1, ci));
            const Quad<R> iy0 = lds4(FY4(1, cj, ci)), iy1 = lds4(FY4(1, cj, ci + 1));
            const R dx[4] = {ix1.a - ix0.a, ix1.b - ix0.b, ix1.c - ix0.c, ix1.d - ix0.d};
            const R dy[4] = {iy1.a - iy0.a, iy1.b - iy0.b, iy1.c - iy0.c, iy1.d - iy0.d};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                a.dst_s[k * a.plane + o] = div_h(dx[k], a.hx, a.inv_hx, a.pow2_x);
                a.dst_t[k * a.plane + o] = div_h(dy[k], a.hy, a.inv_hy, a.pow2_y);
            }
        }
    }
    if (bad)
        atomicOr(&a.ctl->upd_bad[slot], 1u);
    if (!last_tile)  // the CTA's next tile reuses the shared memory
        __syncthreads();
#undef Wx
#undef Sx
#undef FXx
#undef FYx
#undef S4
#undef FX4
#undef FY4
#undef W4
}

// The gathered tile with its shared-memory carve-up (W | S | FX | FY).
template <typename R, int TJ, int TI, int NT, bool LEARNED, int RS = 0>
__device__ __forceinline__ void unsplit_tile(const StepArgs<R>& a, const Gas<R>& G, const int I0, const int J0,
                                             unsigned char* smem_raw, const MlpShared& Mlp, bool last_tile = false)
{
    using SM = UnsplitSmem<R, TJ, TI>;
    R* W = reinterpret_cast<R*>(smem_raw);
    R* S = W + SM::nW;
    R* FX = S + SM::nS;
    R* FY = FX + SM::nFX;
    unsigned short* Q = reinterpret_cast<unsigned short*>(smem_raw + SM::bytes_f);
    tile_body<R, TJ, TI, NT, LEARNED, false, RS>(a, G, I0, J0, W, nullptr, S, FX, FY, Q, Mlp, last_tile);
}

// The learned form reads the network's image from global memory (through L1):
// one CTA per tile would otherwise copy its 11.8 KB into shared memory per tile.
template <typename R, int TJ, int TI, int NT, int MINB = 1, bool LEARNED = false, int RS = 0>
__global__ void __launch_bounds__(NT, MINB) k_step_unsplit(const __grid_constant__ StepArgs<R> a)
{
    if (halt_prologue(a.ctl, a.seq))
        return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // (the plain form never reads it)
    const MlpShared& Mlp = *reinterpret_cast<const MlpShared*>(LEARNED ? a.mlp_img : (const void*)smem_raw);
    unsplit_tile<R, TJ, TI, NT, LEARNED, RS>(a, a.G, blockIdx.x * TI, blockIdx.y * TJ, smem_raw, Mlp, true);
}

// ---------------------------------------------------------------------------
// persistent TMA-staged unsplit step: resident CTAs walk the tiles
// t = blockIdx.x, blockIdx.x + gridDim.x, ...  With STAGES = 2, while tile k
// is computed the TMA unit copies tile k+1's values and previous slopes into
// the other stage, so global-memory latency overlaps the face solves within
// the CTA; with STAGES = 1 the CTA waits for its own copy and the other CTAs
// on the SM hide it (smaller shared memory, more CTAs per SM).
//   shared memory: stage(s) | S | FY | face queue | [network image] | 2 mbarriers
// (the x-fluxes FX reuse the slope box of the current stage, dead after the
// limiter phase).
// ---------------------------------------------------------------------------
template <typename R, int TJ, int TI, bool LEARNED, int STAGES = 2>
struct TmaSmem {
    using SM = UnsplitSmem<R, TJ, TI>;
    using SL = StageLayout<R, TJ, TI>;
    static_assert(STAGES == 1 || STAGES == 2, "one or two stages");
    static constexpr size_t s_off = STAGES * SL::bytes;
    static constexpr size_t fy_off = s_off + sizeof(R) * SM::nS;
    static constexpr size_t q_off = fy_off + sizeof(R) * SM::nFY;
    // the learned form keeps the network image here, loaded once per CTA (the
    // persistent CTA serves many tiles; read through L1 it cost ~10% of a step)
    static constexpr size_t mlp_off = (q_off + 2 * (size_t)SM::nQ + 15) / 16 * 16;
    static constexpr size_t bar_off = (mlp_off + (LEARNED ? sizeof(MlpShared) : 0) + 15) / 16 * 16;
    static constexpr size_t bytes = bar_off + 16;
    // the dynamic shared memory follows the static variables, so its start is
    // only 16-byte aligned: 128 bytes of slack let the kernel align it itself
    static constexpr size_t launch_bytes = bytes + 128;
    static_assert(sizeof(R) * SM::nFX <= SL::b_bytes, "the x-fluxes must fit in the slope box they reuse");
    static_assert(SL::bytes % 128 == 0, "stages start on 128-byte boundaries");
};

constexpr unsigned long long TMA_WAIT_NS = 2000000000ull;  // 2 s

template <typename R, int TJ, int TI, int NT, int MINB = 1, bool LEARNED = false, int STAGES = 2, int RS = 0>
__global__ void __launch_bounds__(NT, MINB) k_step_tma(const __grid_constant__ StepArgs<R> a,
                                                       const __grid_constant__ StepMaps maps)
{
    using SL = StageLayout<R, TJ, TI>;
    using TS = TmaSmem<R, TJ, TI, LEARNED, STAGES>;
    if (halt_prologue(a.ctl, a.seq))
        return;
    extern __shared__ __align__(128) unsigned char smem_dyn[];
    // tensor copies write to 128-byte aligned shared addresses only
    unsigned char* smem_raw = smem_dyn + ((128u - (smem_addr(smem_dyn) & 127u)) & 127u);
    if ((smem_addr(smem_raw) & 127u) != 0u || (reinterpret_cast<uintptr_t>(&maps.vals) & 63u) != 0u ||
        (reinterpret_cast<uintptr_t>(&maps.slopes) & 63u) != 0u) {
        // a misaligned stage or descriptor is never handed to the TMA unit
        if (threadIdx.x == 0)
            atomicExch(&a.ctl->wait_err, 2u);
        return;
    }
    R* S = reinterpret_cast<R*>(smem_raw + TS::s_off);
    R* FY = reinterpret_cast<R*>(smem_raw + TS::fy_off);
    unsigned short* Q = reinterpret_cast<unsigned short*>(smem_raw + TS::q_off);
    MlpShared& Mlp = *reinterpret_cast<MlpShared*>(smem_raw + TS::mlp_off);
    if (LEARNED)  // made visible by the barrier after the mbarrier set-up below
        mlp_load_shared(Mlp, a.mlp_frag, a.mlp_prm, threadIdx.x, NT);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + TS::bar_off);
    const int nti = (a.n + TI - 1) / TI;
    const int ntiles = nti * ((a.m + TJ - 1) / TJ);
    constexpr uint32_t STAGE_TX = (uint32_t)(SL::a_bytes + SL::b_bytes);
    if (threadIdx.x == 0) {
        tma_prefetch_desc(&maps.vals);
        tma_prefetch_desc(&maps.slopes);
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    // one thread: announce the stage's bytes and start its two box copies
    auto issue = [&](int t, int stg) {
        unsigned char* dst = smem_raw + stg * SL::bytes;
        const int I0 = (t % nti) * TI, J0 = (t / nti) * TJ;
        mbar_arrive_expect_tx(&bar[stg], STAGE_TX);
        tma_load_3d(dst + SL::a_off, &maps.vals, I0 - SL::X, J0 - 2, 0, &bar[stg]);
        tma_load_3d(dst + SL::b_off, &maps.slopes, I0 - SL::X, J0 - 1, 0, &bar[stg]);
    };
    int t = blockIdx.x, k = 0;
    if (STAGES == 2 && threadIdx.x == 0 && t < ntiles)
        issue(t, 0);
    bool failed = false;
    for (; t < ntiles; ++k, t += gridDim.x) {
        // stage of tile k and the parity of its barrier's phase (the j-th use of
        // a barrier completes phase j)
        const int stg = STAGES == 2 ? (k & 1) : 0;
        const uint32_t parity = STAGES == 2 ? (uint32_t)(k >> 1) & 1u : (uint32_t)k & 1u;
        if (threadIdx.x == 0) {
            if (STAGES == 2) {
                if (t + (int)gridDim.x < ntiles) {
                    // the other stage was last read and written by tile k-1, which ended with a block barrier
                    fence_proxy_async_smem();
                    issue(t + gridDim.x, stg ^ 1);
                }
            } else {
                // the only stage was last used by tile k-1, which ended with a block barrier
                fence_proxy_async_smem();
                issue(t, 0);
            }
        }
        const bool ok = mbar_wait_bounded(&bar[stg], parity, TMA_WAIT_NS);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        unsigned char* cur = smem_raw + stg * SL::bytes;
        R* W = reinterpret_cast<R*>(cur + SL::a_off);
        R* B = reinterpret_cast<R*>(cur + SL::b_off);
        tile_body<R, TJ, TI, NT, LEARNED, true, RS>(a, a.G, (t % nti) * TI, (t / nti) * TJ, W, B, S, B, FY, Q, Mlp);
    }
    if (failed && threadIdx.x == 0) {
        // let the copies still in flight land (bounded) before the CTA exits, then report
        if (STAGES == 2) {
            mbar_wait_bounded(&bar[k & 1], (uint32_t)(k >> 1) & 1u, TMA_WAIT_NS);
            if (t + (int)gridDim.x < ntiles)
                mbar_wait_bounded(&bar[(k + 1) & 1], (uint32_t)((k + 1) >> 1) & 1u, TMA_WAIT_NS);
        } else {
            mbar_wait_bounded(&bar[0], (uint32_t)k & 1u, TMA_WAIT_NS);
        }
        atomicExch(&a.ctl->wait_err, 1u);
    }
}

// ---------------------------------------------------------------------------
// split sweeps: grp_solver_2D_split_EUL_source.c:214-303.  YDIR = 0: x-sweep
// (x-faces, half time step, s updated); YDIR = 1: y-sweep (y-faces, t updated).
// No transversal derivatives (Transversal = false).  Written in the sweep's
// own coordinates: "a" is the sweep axis, "b" the other one.
// ---------------------------------------------------------------------------
template <typename R, int TJ, int TI>
struct SweepSmem {
    // TA cells along the sweep axis with a 2-cell halo, TB cells across
    static constexpr size_t bytes(int TA, int TB)
    {
        return sizeof(R) * (size_t)(4 * (TA + 4) * TB + 4 * (TA + 2) * TB + 8 * (TA + 1) * TB);
    }
};

template <typename R, int YDIR, int TJ, int TI, int NT, int RS = 0>
__global__ void __launch_bounds__(NT) k_sweep(const __grid_constant__ StepArgs<R> a)
{
    if (halt_prologue(a.ctl, a.seq))
        return;
    // sweep axis length TA (with halo) and cross length TB
    constexpr int TA = YDIR ? TI : TJ;
    constexpr int TB = YDIR ? TJ : TI;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* W = reinterpret_cast<R*>(smem_raw);   // [4][TA+4][TB]
    R* S = W + 4 * (TA + 4) * TB;            // [4][TA+2][TB]
    R* F = S + 4 * (TA + 2) * TB;            // [8][TA+1][TB]
    const int tid = threadIdx.x;
    const int I0 = blockIdx.x * TI, J0 = blockIdx.y * TJ;
    const int m = a.m, n = a.n, slot = a.seq % 3;
    const int A0 = YDIR ? I0 : J0, B0 = YDIR ? J0 : I0;
    const int NA = YDIR ? n : m, NB = YDIR ? m : n;
    const int bnd = YDIR ? a.by : a.bx;
    const R h = YDIR ? a.hy : a.hx, inv_h = YDIR ? a.inv_hy : a.inv_hx;
    const int pow2 = YDIR ? a.pow2_y : a.pow2_x;
    const R hh = YDIR ? a.hhy : a.hhx;
    const R fac = YDIR ? a.mu : a.nu;
    const int find = YDIR ? a.find_y : a.find_x;
    const R* src_sl = YDIR ? a.src_t : a.src_s;
    R* dst_sl = YDIR ? a.dst_t : a.dst_s;
#define Wv(k, la, lb) W[((k) * (TA + 4) + (la)) * TB + (lb)]
#define Sv(k, sa, lb) S[((k) * (TA + 2) + (sa)) * TB + (lb)]
#define Fv(k, fa, lb) F[((k) * (TA + 1) + (fa)) * TB + (lb)]

    for (int idx = tid; idx < (TA + 4) * TB; idx += NT) {
        int la, lb;
        if (YDIR) { lb = idx / (TA + 4); la = idx - lb * (TA + 4); }
        else { la = idx / TB; lb = idx - la * TB; }
        int ca = A0 - 2 + la, cb = B0 + lb;
        int j = YDIR ? cb : ca, i = YDIR ? ca : cb;
        R w[4];
        load_prims(a, j, i, w);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            Wv(k, la, lb) = w[k];
    }
    __syncthreads();
    for (int idx = tid; idx < (TA + 2) * TB; idx += NT) {
        int sa, lb;
        if (YDIR) { lb = idx / (TA + 2); sa = idx - lb * (TA + 2); }
        else { sa = idx / TB; lb = idx - sa * TB; }
        int ca = A0 - 1 + sa, cb = B0 + lb;
        int j = YDIR ? cb : ca, i = YDIR ? ca : cb;
        if (cb >= NB)
            continue;
        size_t o = slope_index(a, j, i);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            Sv(k, sa, lb) = limit(Wv(k, sa, lb), Wv(k, sa + 1, lb), Wv(k, sa + 2, lb), h, inv_h, pow2, a.alpha, find,
                                  find ? src_sl[k * a.plane + o] : R(0));
    }
    __syncthreads();
    if (bnd != -7) {
        const int sg[2] = {(A0 == 0) ? 0 : -1, (NA - A0 + 1 <= TA + 1) ? NA - A0 + 1 : -1};
        const int keep = YDIR ? 2 : 1;  // reflective keeps the normal velocity's slope
        for (int idx = tid; idx < 2 * TB; idx += NT) {
            int side = idx / TB, lb = idx % TB;
            int sa = sg[side];
            if (sa < 0)
                continue;
            int se = side == 0 ? sa + 1 : sa - 1;
            bool kp = (bnd == -2) || (bnd == -24 && side == 0);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                Sv(k, sa, lb) = (kp && k == keep) ? Sv(k, se, lb) : R(0);
        }
    }
    __syncthreads();

    int my_iters = 0, my_newton = 0, my_fb = 0;
    for (int f = tid; f < (TA + 1) * TB; f += NT) {
        int fa, lb;
        if (YDIR) { lb = f / (TA + 1); fa = f - lb * (TA + 1); }
        else { fa = f / TB; lb = f - fa * TB; }
        int ca = A0 + fa, cb = B0 + lb;
        if (ca > NA || cb >= NB)
            continue;
        R s0 = Sv(0, fa, lb), s1 = Sv(1, fa, lb), s2 = Sv(2, fa, lb), s3 = Sv(3, fa, lb);
        R r0 = Sv(0, fa + 1, lb), r1 = Sv(1, fa + 1, lb), r2 = Sv(2, fa + 1, lb), r3 = Sv(3, fa + 1, lb);
        R lr = Wv(0, fa + 1, lb) + hh * s0, lu = Wv(1, fa + 1, lb) + hh * s1;
        R lv = Wv(2, fa + 1, lb) + hh * s2, lp = Wv(3, fa + 1, lb) + hh * s3;
        R rr = Wv(0, fa + 2, lb) - hh * r0, ru = Wv(1, fa + 2, lb) - hh * r1;
        R rv = Wv(2, fa + 2, lb) - hh * r2, rp = Wv(3, fa + 2, lb) - hh * r3;
        Side<R> L, Rr;
        if (!YDIR) {
            L.rho = lr; L.u = lu; L.v = lv; L.p = lp; L.drho = s0; L.du = s1; L.dv = s2; L.dp = s3;
            Rr.rho = rr; Rr.u = ru; Rr.v = rv; Rr.p = rp; Rr.drho = r0; Rr.du = r1; Rr.dv = r2; Rr.dp = r3;
        } else {
            L.rho = lr; L.u = lv; L.v = -lu; L.p = lp; L.drho = s0; L.du = s2; L.dv = -s1; L.dp = s3;
            Rr.rho = rr; Rr.u = rv; Rr.v = -ru; Rr.p = rp; Rr.drho = r0; Rr.du = r2; Rr.dv = -r1; Rr.dp = r3;
        }
        L.trho = L.tu = L.tv = L.tp = R(0);
        Rr.trho = Rr.tu = Rr.tv = Rr.tp = R(0);
        FaceOut<R> o;
        int it;
        int fbk;
        const int code = solve_face<R, 0, RS>(L, Rr, a.G, a.tau, a.htau, o, it, fbk, YDIR != 0);
        if (it >= 0) {
            my_newton++;
            my_iters += it;
            my_fb += fbk;
        }
        int j = YDIR ? cb : ca, i = YDIR ? ca : cb;
        unsigned long long serial = YDIR ? (unsigned long long)j * (n + 1) + i : (unsigned long long)i * (m + 1) + j;
        report_face(a.ctl, slot, YDIR, serial, code);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            Fv(k, fa, lb) = o.F[k];
            Fv(4 + k, fa, lb) = o.I[k];
        }
    }
    if (a.stats) {
        __syncwarp();
        for (int off = 16; off; off >>= 1) {
            my_newton += __shfl_xor_sync(0xffffffffu, my_newton, off);
            my_iters += __shfl_xor_sync(0xffffffffu, my_iters, off);
            my_fb += __shfl_xor_sync(0xffffffffu, my_fb, off);
        }
        if ((tid & 31) == 0 && my_newton) {
            atomicAdd(&a.ctl->newton_faces, (unsigned long long)my_newton);
            atomicAdd(&a.ctl->newton_iters, (unsigned long long)my_iters);
            if (my_fb)
                atomicAdd(&a.ctl->newton_fallbacks, (unsigned long long)my_fb);
        }
    }
    __syncthreads();

    unsigned bad = 0;
    for (int idx = tid; idx < TA * TB; idx += NT) {
        int ca_l, lb;
        if (YDIR) { lb = idx / TA; ca_l = idx - lb * TA; }
        else { ca_l = idx / TB; lb = idx - ca_l * TB; }
        int ca = A0 + ca_l, cb = B0 + lb;
        if (ca >= NA || cb >= NB)
            continue;
        int j = YDIR ? cb : ca, i = YDIR ? ca : cb;
        const size_t o = (size_t)j * a.ld + i;
        R rho = Wv(0, ca_l + 2, lb);
        R uu = Wv(1, ca_l + 2, lb), vv = Wv(2, ca_l + 2, lb);
        R E = a.src_w[4 * a.plane + o];
        R mom_x = rho * uu - fac * (Fv(1, ca_l + 1, lb) - Fv(1, ca_l, lb));
        R mom_y = rho * vv - fac * (Fv(2, ca_l + 1, lb) - Fv(2, ca_l, lb));
        R ene = rho * E - fac * (Fv(3, ca_l + 1, lb) - Fv(3, ca_l, lb));
        rho += -fac * (Fv(0, ca_l + 1, lb) - Fv(0, ca_l, lb));
        R un = mom_x / rho, vn = mom_y / rho, En = ene / rho;
        R pn = (ene - R(0.5) * mom_x * un - R(0.5) * mom_y * vn) * a.G.gm1;
        if (pn < a.G.eps || rho < a.G.eps)
            bad = 1;
        a.dst_w[o] = rho;
        a.dst_w[a.plane + o] = un;
        a.dst_w[2 * a.plane + o] = vn;
        a.dst_w[3 * a.plane + o] = pn;
        a.dst_w[4 * a.plane + o] = En;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            dst_sl[k * a.plane + o] = div_h(Fv(4 + k, ca_l + 1, lb) - Fv(4 + k, ca_l, lb), h, inv_h, pow2);
    }
    if (bad)
        atomicOr(&a.ctl->upd_bad[slot], 1u);
#undef Wv
#undef Sv
#undef Fv
}

}  // namespace hydro
