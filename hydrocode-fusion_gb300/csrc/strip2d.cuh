// strip2d.cuh -- the FP32 unsplit step as column strips, one warp per strip.
//
// The same step as k_step_tma / k_step_unsplit (grp_solver_2D_EUL_source.c:
// 146-286: limiter, GRP faces, conservative update, new slopes), laid out for
// instruction throughput instead of tile reuse:
//
//   * a strip is 64 columns of cells, two adjacent columns per lane held as a
//     float2, so every add, multiply and fused multiply-add of the limiter, the
//     acoustic GRP case and the update is one packed FP32 instruction
//     (add/mul/fma.rn.f32x2) for two cells or two faces; the 4 outer columns are
//     halo, so a strip updates 60 columns and the strips overlap by 4;
//   * the warp marches down its strip one row at a time with the rows it needs
//     in registers (values of rows r-1, r, r+1, slopes of rows r-1, r, the
//     x-faces of row r-1): neighbours along the row come by warp shuffles, so
//     the kernel has no shared-memory tile and no block barrier;
//   * faces that are not a uniform pair (the exact Riemann solver's faces, a few
//     per cent or less on piecewise-smooth data) and faces whose FP32 star state
//     fails its check go to a per-warp queue in shared memory and are solved 32
//     at a time by the same solve_face / FP64 retry as the tile kernels, so the
//     exact solver runs on full warps while the acoustic faces stay packed;
//   * work units are (strip, run of STRIP_SEG rows), taken from a per-launch
//     counter by each warp; a unit recomputes the two halo rows above it.
//
// Values are loaded with 64-bit loads of the column pair straight from the
// state planes one row ahead of use; ghost cells at the domain edges go
// through load_prims and the boundary slope rules of the tile kernels.  The FP32
// arithmetic is rearranged for packed instructions (derivatives carried
// negated, the limiter on magnitudes and sign bits), so results agree with the
// tile kernels to FP32 rounding, not bit for bit.
#pragma once

#include "step2d.cuh"

namespace hydro {

constexpr int STRIP_W = 60;      // columns a strip updates (64 loaded)
constexpr int STRIP_QCAP = 64;   // queued faces per warp per flush
constexpr int STRIP_QWORDS = 28; // words per queue entry
// The learned form runs the network on a flush of at least this many faces
// (the default; a launch argument): one warp pass of the network costs about
// as much as the Newton iterations it saves on a full warp of faces, so on a
// handful it would only add time.
constexpr int STRIP_MLP_MIN = 16;

// ---------------------------------------------------------------------------
// packed FP32
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 p_s(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 p_rcp(float2 a) { return make_float2(__fdividef(1.f, a.x), __fdividef(1.f, a.y)); }
__device__ __forceinline__ float2 p_sqrt(float2 a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }
__device__ __forceinline__ float2 p_sel(bool sx, bool sy, float2 a, float2 b)
{
    return make_float2(sx ? a.x : b.x, sy ? a.y : b.y);
}
__device__ __forceinline__ float2 ldg2(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }

struct SV2 {  // values of a cell pair: rho u v p
    float2 w[4];
};
struct SS2 {  // limited slopes of a cell pair: x-slopes s, y-slopes t (rho u v p)
    float2 s[4], t[4];
};
struct SF2 {  // outputs of a face pair: fluxes F and t+tau interface values I,
              // in the face's normal frame (normal velocity first: an x-face's
              // F = rho u, rho u u + p, rho u v, rho u H; a y-face's
              // F = rho v, rho v v + p, rho v u', rho v H with u' = -u, likewise I)
    float2 F[4], I[4];
};
// a face pair's side in the normal frame, in Side<float>'s order
enum { X_RHO, X_U, X_V, X_P, X_DRHO, X_DU, X_DV, X_DP, X_TRHO, X_TU, X_TV, X_TP };
struct SSide2 {
    float2 x[12];
};

// ---------------------------------------------------------------------------
// limiter
// ---------------------------------------------------------------------------
// minmod3(a, b, sp) of the scaled differences a = alpha dL/h, b = alpha dR/h:
// zero unless the three share a sign, else the smallest magnitude with that sign
__device__ __forceinline__ float strip_mm3(float a, float b, float sp)
{
    const float mag = fminf(fminf(fabsf(a), fabsf(b)), fabsf(sp));
    const unsigned ba = __float_as_uint(a), bb = __float_as_uint(b), bm = __float_as_uint(sp);
    const bool agree = (int)((ba ^ bm) | (bb ^ bm)) >= 0;
    return agree ? __uint_as_float(__float_as_uint(mag) | (bm & 0x80000000u)) : 0.f;
}
// minmod2(a, b) of a = dL/h, b = dR/h (the first limiting of a run)
__device__ __forceinline__ float strip_mm2(float a, float b)
{
    const float mag = fminf(fabsf(a), fabsf(b));
    const unsigned ba = __float_as_uint(a), bb = __float_as_uint(b);
    return (int)(ba ^ bb) >= 0 ? __uint_as_float(__float_as_uint(mag) | (ba & 0x80000000u)) : 0.f;
}
__device__ __forceinline__ float2 strip_limit(float2 wl, float2 wc, float2 wr, float2 sp, bool find, float ah, float ih)
{
    const float2 k = p_s(find ? ah : ih);
    const float2 a = p_mul(p_sub(wc, wl), k), b = p_mul(p_sub(wr, wc), k);
    if (find)
        return make_float2(strip_mm3(a.x, b.x, sp.x), strip_mm3(a.y, b.y, sp.y));
    return make_float2(strip_mm2(a.x, b.x), strip_mm2(a.y, b.y));
}

// ---------------------------------------------------------------------------
// loads of one row of the lane's column pair (c, c+1)
// ---------------------------------------------------------------------------
template <class A>
__device__ __forceinline__ void strip_load_vals(const A& a, int j, int c, bool fast, SV2& V)
{
    if (fast) {
        const float* b = a.src_w + (size_t)j * a.ld + c;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            V.w[k] = ldg2(b + k * a.plane);
    } else {
        float w0[4], w1[4];
        load_prims(a, j, c, w0);
        load_prims(a, j, c + 1, w1);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            V.w[k] = make_float2(w0[k], w1[k]);
    }
}

template <class A>
__device__ __forceinline__ void strip_load_prev(const A& a, int j, int c, bool fast, SS2& P)
{
    if (fast) {
        const size_t o = (size_t)j * a.ld + c;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            P.s[k] = a.find_x ? ldg2(a.src_s + k * a.plane + o) : make_float2(0.f, 0.f);
            P.t[k] = a.find_y ? ldg2(a.src_t + k * a.plane + o) : make_float2(0.f, 0.f);
        }
    } else {
        const size_t o0 = slope_index(a, j, c), o1 = slope_index(a, j, c + 1);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            P.s[k] = a.find_x ? make_float2(a.src_s[k * a.plane + o0], a.src_s[k * a.plane + o1]) : make_float2(0.f, 0.f);
            P.t[k] = a.find_y ? make_float2(a.src_t[k * a.plane + o0], a.src_t[k * a.plane + o1]) : make_float2(0.f, 0.f);
        }
    }
}

// Limited slopes of row r (values Vm, V0, Vp of rows r-1, r, r+1; previous
// slopes P).  The y-neighbours of the pair come from the adjacent lanes.
template <class A>
__device__ __forceinline__ void strip_slopes(const A& a, const SV2& Vm, const SV2& V0, const SV2& Vp,
                                             const SS2& P, float ahx, float ihx, float ahy, float ihy, SS2& S)
{
    const unsigned FULL = 0xffffffffu;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 wc = V0.w[k];
        S.s[k] = strip_limit(Vm.w[k], wc, Vp.w[k], P.s[k], a.find_x, ahx, ihx);
        const float wl = __shfl_up_sync(FULL, wc.y, 1);    // column c-1
        const float wr = __shfl_down_sync(FULL, wc.x, 1);  // column c+2
        S.t[k] = strip_limit(make_float2(wl, wc.x), wc, make_float2(wc.y, wr), P.t[k], a.find_y, ahy, ihy);
    }
}

// Ghost slopes of a non-periodic x-boundary row (bound_cond_slope_limiter_x.c:
// 94-126, as phase 2b of the tile kernels): from the edge row's slopes E.
template <class A>
__device__ __forceinline__ void strip_ghost_row(const A& a, const SS2& E, bool low, SS2& S)
{
    const bool keep_su = (a.bx == -2) || (a.bx == -24 && low);
    S.s[0] = make_float2(0.f, 0.f);
    S.s[1] = keep_su ? E.s[1] : make_float2(0.f, 0.f);
    S.s[2] = make_float2(0.f, 0.f);
    S.s[3] = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        S.t[k] = (a.bx == -1) ? make_float2(0.f, 0.f) : E.t[k];
}

// Ghost slopes of the non-periodic y-boundary columns -1 and n of a row
// (bound_cond_slope_limiter_y.c:94-126): the edge column's slopes by the
// same rules.  Warp-collective; c = first column of the lane's pair.
template <class A>
__device__ __forceinline__ void strip_ghost_cols(const A& a, int c, SS2& S)
{
    const unsigned FULL = 0xffffffffu;
    const int n = a.n;
    const bool gx_lo = (c == -1), gx_hi = (c == n);          // element x is a ghost column
    const bool gy_lo = (c + 1 == -1), gy_hi = (c + 1 == n);  // element y
    const bool keep_lo = (a.by == -2) || (a.by == -24), keep_hi = (a.by == -2);
    auto fix = [&](float2& v, bool tslope, bool keep) {
        const float right_x = __shfl_down_sync(FULL, v.x, 1);
        const float left_y = __shfl_up_sync(FULL, v.y, 1);
        // edge value of each element: column 0 for column -1, column n-1 for column n
        const float ex = gx_lo ? v.y : left_y;
        const float ey = gy_lo ? right_x : v.x;
        float rx, ry;
        if (!tslope) {  // x-slopes (tangential at these faces): the edge's, or 0 for the fixed boundary
            rx = (a.by == -1) ? 0.f : ex;
            ry = (a.by == -1) ? 0.f : ey;
        } else {  // y-slopes: 0, except that the reflective boundaries keep the v-slope
            rx = (keep && ((gx_lo && keep_lo) || (gx_hi && keep_hi))) ? ex : 0.f;
            ry = (keep && ((gy_lo && keep_lo) || (gy_hi && keep_hi))) ? ey : 0.f;
        }
        if (gx_lo || gx_hi)
            v.x = rx;
        if (gy_lo || gy_hi)
            v.y = ry;
    };
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        fix(S.s[k], false, false);
        fix(S.t[k], true, k == 2);
    }
}

// ---------------------------------------------------------------------------
// the acoustic (uniform-pair) GRP case of a face pair, packed
// (linear_grp_solver_Edir_Q1D.c:92-254 with lambda = 0), then GRP_2D_flux's
// outputs (flux_solver.c:195-220).  Derivatives are carried negated (nD = -D).
// uni: each element is a uniform pair.  code: 0, 1 (ifvar_check's positivity)
// or 2 (the star/derivative check failed, or an output is not finite: the face
// is redone in FP64, which decides its code); for elements that are not
// uniform the outputs are meaningless (the queue replaces them).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void strip_face_pair(const SSide2& L, const SSide2& R, const Gas<float>& G, float tau,
                                                float htau, SF2& o, bool& uni_x, bool& uni_y, int& code_x, int& code_y)
{
    const unsigned FULL = 0xffffffffu;
    // uniform-pair test (face_uniform<float>): squared distance against the
    // squared threshold max(eps, 1e-6 scale)
    {
        const float2 dr = p_sub(L.x[X_RHO], R.x[X_RHO]), du = p_sub(L.x[X_U], R.x[X_U]), dp = p_sub(L.x[X_P], R.x[X_P]);
        const float2 d2 = p_fma(dp, dp, p_fma(du, du, p_mul(dr, dr)));
        const float2 sc = p_add(p_add(L.x[X_RHO], R.x[X_RHO]), p_add(L.x[X_P], R.x[X_P]));
        const float thx = fmaxf(G.eps, 1e-6f * (sc.x + fabsf(L.x[X_U].x) + fabsf(R.x[X_U].x)));
        const float thy = fmaxf(G.eps, 1e-6f * (sc.y + fabsf(L.x[X_U].y) + fabsf(R.x[X_U].y)));
        uni_x = d2.x < thx * thx;
        uni_y = d2.y < thy * thy;
    }
    // ifvar_check's positivity of pressure and density on both sides
    code_x = fminf(fminf(L.x[X_P].x, R.x[X_P].x), fminf(L.x[X_RHO].x, R.x[X_RHO].x)) < G.eps ? 1 : 0;
    code_y = fminf(fminf(L.x[X_P].y, R.x[X_P].y), fminf(L.x[X_RHO].y, R.x[X_RHO].y)) < G.eps ? 1 : 0;

    const float2 h = p_s(0.5f);
    const float2 irL = p_rcp(L.x[X_RHO]), irR = p_rcp(R.x[X_RHO]);
    const float2 cL2 = p_mul(p_mul(p_s(G.g), L.x[X_P]), irL), cR2 = p_mul(p_mul(p_s(G.g), R.x[X_P]), irR);
    const float2 rsL = make_float2(rsqrtf(cL2.x), rsqrtf(cL2.y)), rsR = make_float2(rsqrtf(cR2.x), rsqrtf(cR2.y));
    const float2 cL = p_mul(cL2, rsL), cR = p_mul(cR2, rsR);
    const float2 us = p_mul(h, p_add(R.x[X_U], L.x[X_U]));
    const float2 ps = p_mul(h, p_add(R.x[X_P], L.x[X_P]));
    const float2 spL = p_sub(us, cL), spR = p_add(us, cR);
    // the side upwind of the contact (u* > 0: left); a supersonic t-axis
    // (speed_L > 0 or speed_R < 0) lies on that side too
    const bool px = us.x > 0.f, py = us.y > 0.f;
    const float2 U0 = p_sel(px, py, L.x[X_RHO], R.x[X_RHO]);
    const float2 U2 = p_sel(px, py, L.x[X_V], R.x[X_V]);
    const float2 C2 = p_sel(px, py, cL2, cR2);
    const float2 rsX = p_sel(px, py, rsL, rsR);
    const float2 iU0 = p_sel(px, py, irL, irR);
    const float2 Dv = p_sel(px, py, L.x[X_DV], R.x[X_DV]);
    const float2 Tv = p_sel(px, py, L.x[X_TV], R.x[X_TV]);
    const float2 dpX = p_sel(px, py, L.x[X_DP], R.x[X_DP]), tpX = p_sel(px, py, L.x[X_TP], R.x[X_TP]);
    const float2 drX = p_sel(px, py, L.x[X_DRHO], R.x[X_DRHO]), trX = p_sel(px, py, L.x[X_TRHO], R.x[X_TRHO]);
    // subsonic: the t-axis state is the star state (acoustic case)
    const float2 rc = p_mul(U0, p_mul(C2, rsX));  // rho c
    const float2 irc = p_mul(iU0, rsX);           // 1/(rho c)
    const float2 icc = p_mul(rsX, rsX);           // 1/c^2
    float2 Dp = p_mul(h, p_sub(p_fma(L.x[X_DU], rc, L.x[X_DP]), p_fma(R.x[X_DU], rc, p_mul(p_s(-1.f), R.x[X_DP]))));
    float2 Tp = p_mul(h, p_sub(p_fma(L.x[X_TU], rc, L.x[X_TP]), p_fma(R.x[X_TU], rc, p_mul(p_s(-1.f), R.x[X_TP]))));
    float2 Du = p_mul(h, p_fma(p_sub(L.x[X_DP], R.x[X_DP]), irc, p_add(L.x[X_DU], R.x[X_DU])));
    float2 Tu = p_mul(h, p_fma(p_sub(L.x[X_TP], R.x[X_TP]), irc, p_add(L.x[X_TU], R.x[X_TU])));
    float2 Drho = p_fma(p_sub(Dp, dpX), icc, drX);
    float2 Trho = p_fma(p_sub(Tp, tpX), icc, trX);
    float2 U1 = us, U3 = ps;
    const bool ax = spL.x > 0.f || spR.x < 0.f, ay = spL.y > 0.f || spR.y < 0.f;
    if (__any_sync(FULL, ax | ay)) {
        // supersonic: that side's own state and derivatives
        U1 = p_sel(ax, ay, p_sel(px, py, L.x[X_U], R.x[X_U]), U1);
        U3 = p_sel(ax, ay, p_sel(px, py, L.x[X_P], R.x[X_P]), U3);
        Du = p_sel(ax, ay, p_sel(px, py, L.x[X_DU], R.x[X_DU]), Du);
        Tu = p_sel(ax, ay, p_sel(px, py, L.x[X_TU], R.x[X_TU]), Tu);
        Dp = p_sel(ax, ay, dpX, Dp);
        Tp = p_sel(ax, ay, tpX, Tp);
        Drho = p_sel(ax, ay, drX, Drho);
        Trho = p_sel(ax, ay, trX, Trho);
    }
    const float2 dvs = p_add(Du, Tv);
    const float2 nD0 = p_fma(U1, Drho, p_fma(U2, Trho, p_mul(U0, dvs)));
    const float2 nD1 = p_fma(U1, Du, p_fma(U2, Tu, p_mul(Dp, iU0)));
    const float2 nD2 = p_fma(U1, Dv, p_fma(U2, Tv, p_mul(Tp, iU0)));
    const float2 nD3 = p_fma(U1, Dp, p_fma(U2, Tp, p_mul(p_mul(U0, C2), dvs)));
    // fluxes at t + tau/2 and values at t + tau
    const float2 mh = p_s(-htau), mt = p_s(-tau);
    const float2 rm = p_fma(mh, nD0, U0), am = p_fma(mh, nD1, U1), bm = p_fma(mh, nD2, U2), pm = p_fma(mh, nD3, U3);
    const float2 Fr = p_mul(rm, am);
    const float2 Fe = p_fma(p_mul(p_s(G.g_g1), pm), p_rcp(rm), p_mul(h, p_fma(am, am, p_mul(bm, bm))));
    o.F[0] = Fr;
    o.F[1] = p_fma(Fr, am, pm);
    o.F[2] = p_mul(Fr, bm);
    o.F[3] = p_mul(Fr, Fe);
    o.I[0] = p_fma(mt, nD0, U0);
    o.I[1] = p_fma(mt, nD1, U1);
    o.I[2] = p_fma(mt, nD2, U2);
    o.I[3] = p_fma(mt, nD3, U3);
    // star_dire_check: positive t-axis density and pressure; a non-finite value
    // or derivative shows in the outputs (s - s is 0 exactly when s is finite)
    const float2 s = p_add(p_add(p_add(o.F[0], o.F[1]), p_add(o.F[2], o.F[3])),
                           p_add(p_add(o.I[0], o.I[1]), p_add(o.I[2], o.I[3])));
    const float2 z = p_sub(s, s);
    if (fminf(U0.x, U3.x) < G.eps || !(z.x == 0.f))
        code_x = 2;
    if (fminf(U0.y, U3.y) < G.eps || !(z.y == 0.f))
        code_y = 2;
}

// ---------------------------------------------------------------------------
// the per-warp queue of faces for the exact solver / the FP64 retry
// ---------------------------------------------------------------------------
// entry: L[12] R[12] (Side<float> order), row, col, flags (bit 0 dir (1 = y-face),
// bit 1 mode (1 = FP64 retry of an acoustic face), bit 2 counted in the
// statistics), the learned starting pressure (word 27, learned form); after
// the flush, words 0..7 hold the outputs F[4] I[4] in the
// strip's normal-frame convention.
__device__ __forceinline__ void strip_put_side(float* e, const SSide2& S, bool y)
{
#pragma unroll
    for (int k = 0; k < 12; ++k)
        e[k] = y ? S.x[k].y : S.x[k].x;
}

// What a flush needs of its grid: the gas (in the kernel's parameter space),
// the face time step, the control block and launch slot of the error keys, the
// grid's size for the keys' serial numbers.
struct StripFlushArgs {
    const Gas<float>* G;
    Ctl* ctl;
    float tau, htau;
    int m, n, slot;
    int mlp_min;  // learned form: the network runs on flushes of at least this many faces
    float mlp_jump2;  // learned form: the strong-jump threshold of learned_guess
};

template <bool LEARNED>
static __device__ __noinline__ void strip_flush(float* q, int cnt, const StripFlushArgs fa, const MlpShared* M,
                                                int* stats3)
{
    const Gas<float>& G = *fa.G;
    const int lane = threadIdx.x & 31;
    const int slot = fa.slot;
    if constexpr (LEARNED) {
        // the network's starting pressures first, into word 27 of each entry, so
        // that the solves below hold no state across the network's call
        for (int base = 0; base < cnt; base += 32) {
            if (cnt - base < fa.mlp_min)  // warp-uniform
                break;
            const int k = base + lane;
            const bool act = k < cnt;
            float* e = q + (size_t)(act ? k : 0) * STRIP_QWORDS;
            Side<float> L, Rr;
            L.rho = e[0]; L.u = e[1]; L.v = e[2]; L.p = e[3];
            Rr.rho = e[12]; Rr.u = e[13]; Rr.v = e[14]; Rr.p = e[15];
            const bool retry = (__float_as_int(e[26]) >> 1) & 1;
            const bool need = act && !retry &&
                              learned_strong_jump(L.rho, L.u, L.p, Rr.rho, Rr.u, Rr.p, G.g, fa.mlp_jump2);
            const float ps = learned_start(L, Rr, need, G, *M, cnt - base < 32 ? cnt - base : 32);
            if (act)
                e[27] = ps;
        }
    }
    for (int base = 0; base < cnt; base += 32) {
        const int k = base + lane;
        const bool act = k < cnt;
        float* e = q + (size_t)(act ? k : 0) * STRIP_QWORDS;
        Side<float> L, Rr;
        {
            const float* s = e;
            L.rho = s[0]; L.u = s[1]; L.v = s[2]; L.p = s[3]; L.drho = s[4]; L.du = s[5]; L.dv = s[6]; L.dp = s[7];
            L.trho = s[8]; L.tu = s[9]; L.tv = s[10]; L.tp = s[11];
            s += 12;
            Rr.rho = s[0]; Rr.u = s[1]; Rr.v = s[2]; Rr.p = s[3]; Rr.drho = s[4]; Rr.du = s[5]; Rr.dv = s[6];
            Rr.dp = s[7]; Rr.trho = s[8]; Rr.tu = s[9]; Rr.tv = s[10]; Rr.tp = s[11];
        }
        const int row = __float_as_int(e[24]), col = __float_as_int(e[25]), fl = __float_as_int(e[26]);
        const bool ydir = fl & 1, retry = (fl >> 1) & 1, counted = (fl >> 2) & 1;
        if (!act)
            continue;
        float p_start = -1.f;
        if constexpr (LEARNED) {
            if (cnt - base >= fa.mlp_min)
                p_start = e[27];
        }
        FaceOut<float> o;
        int code;
        if (!retry) {
            int it = 0, fb = 0;
            code = solve_face<float, 2, 0>(L, Rr, G, fa.tau, fa.htau, o, it, fb, ydir, p_start);
            if (counted && it >= 0) {
                stats3[0] += 1;
                stats3[1] += it;
                stats3[2] += fb;
            }
        } else {
            code = 2;
        }
        if (code == 2)
            code = solve_face_fp64_retry<0>(L, Rr, G.g64, G.eps64, G.dist2_max, (double)fa.tau, ydir, o);
        if (!ydir)
            report_face(fa.ctl, slot, 0, (unsigned long long)col * (fa.m + 1) + row, code);
        else
            report_face(fa.ctl, slot, 1, (unsigned long long)row * (fa.n + 1) + col, code);
        // back to the normal frame of the strip's outputs (a y-face's global
        // F = (F0, -Ft, Fn, F3), I = (I0, -B, A, I3))
        if (!ydir) {
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                e[t] = o.F[t];
                e[4 + t] = o.I[t];
            }
        } else {
            e[0] = o.F[0]; e[1] = o.F[2]; e[2] = -o.F[1]; e[3] = o.F[3];
            e[4] = o.I[0]; e[5] = o.I[2]; e[6] = -o.I[1]; e[7] = o.I[3];
        }
    }
}

// Queue the faces of a pair that need it (need_x / need_y), flush, and patch
// the outputs o of the queued elements.  Warp-collective.
template <bool LEARNED>
__device__ __forceinline__ void strip_queue(float* q, const SSide2& L, const SSide2& R, bool need_x, bool need_y,
                                            bool retry_x, bool retry_y, bool cnt_x, bool cnt_y, bool ydir, int row_x,
                                            int col_x, int row_y, int col_y, const StripFlushArgs& fa,
                                            const MlpShared* M, int* stats3, SF2& o)
{
    const unsigned FULL = 0xffffffffu;
    const unsigned bx = __ballot_sync(FULL, need_x), by = __ballot_sync(FULL, need_y);
    if ((bx | by) == 0u)
        return;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int ix = __popc(bx & lt), iy = __popc(bx) + __popc(by & lt);
    const int cnt = __popc(bx) + __popc(by);
    if (need_x) {
        float* e = q + (size_t)ix * STRIP_QWORDS;
        strip_put_side(e, L, false);
        strip_put_side(e + 12, R, false);
        e[24] = __int_as_float(row_x);
        e[25] = __int_as_float(col_x);
        e[26] = __int_as_float((ydir ? 1 : 0) | (retry_x ? 2 : 0) | (cnt_x ? 4 : 0));
    }
    if (need_y) {
        float* e = q + (size_t)iy * STRIP_QWORDS;
        strip_put_side(e, L, true);
        strip_put_side(e + 12, R, true);
        e[24] = __int_as_float(row_y);
        e[25] = __int_as_float(col_y);
        e[26] = __int_as_float((ydir ? 1 : 0) | (retry_y ? 2 : 0) | (cnt_y ? 4 : 0));
    }
    __syncwarp();
    strip_flush<LEARNED>(q, cnt, fa, M, stats3);
    __syncwarp();
    if (need_x) {
        const float* e = q + (size_t)ix * STRIP_QWORDS;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            o.F[t].x = e[t];
            o.I[t].x = e[4 + t];
        }
    }
    if (need_y) {
        const float* e = q + (size_t)iy * STRIP_QWORDS;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            o.F[t].y = e[t];
            o.I[t].y = e[4 + t];
        }
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
struct StripArgs {
    unsigned int* work;  // three rotating per-launch unit counters
    int seg;             // rows per work unit
    int mlp_min;         // learned form: smallest queue flush the network runs on
    float mlp_jump2;     // learned form: the strong-jump threshold of learned_guess
    int mlp_global;      // learned form: 1 = read the network image from global memory (through L1)
};

template <int NW, bool LEARNED>
struct StripSmem {
    static constexpr size_t q_bytes = sizeof(float) * STRIP_QCAP * STRIP_QWORDS;  // per warp
    static constexpr size_t mlp_off = NW * q_bytes;
    static constexpr size_t bytes = mlp_off + (LEARNED ? sizeof(MlpShared) : 0);
};

// One work unit of a step: columns [c0, c0 + STRIP_W) of rows [r0, r1) of the
// grid a describes, marched by the calling warp (warp-collective).  A is
// StepArgs<float> or a view with the same members (a problem of a batch); Gp
// is the gas in the kernel's parameter space.  The update's positivity flag
// and the Newton statistics accumulate in the caller's bad and stats3 (see
// strip_report).
template <bool LEARNED, class A>
__device__ __forceinline__ void strip_unit(const A& a, const Gas<float>* Gp, int c0, int r0, int r1, float* q,
                                           const MlpShared* M, int mlp_min, float mlp_jump2, int* stats3,
                                           unsigned& bad)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int m = a.m, n = a.n, slot = a.seq % 3;
    const Gas<float>& G = *Gp;
    const StripFlushArgs fa{Gp, a.ctl, a.tau, a.htau, m, n, slot, mlp_min, mlp_jump2};
    const float ihx = a.pow2_x ? a.inv_hx : 1.f / a.hx, ihy = a.pow2_y ? a.inv_hy : 1.f / a.hy;
    const float ahx = a.alpha * ihx, ahy = a.alpha * ihy;
    const float hhx = a.hhx, hhy = a.hhy;
    const bool ghost_rows = a.bx != -7, ghost_cols = a.by != -7;
    const int c = c0 - 2 + 2 * lane;
    const bool colfast = c >= 0 && c + 1 < n;
    const bool edge_cols = ghost_cols && !__all_sync(FULL, colfast);
    // columns this lane's cells update / faces it owns
    const bool upd_x = lane >= 1 && lane <= 30 && c < n, upd_y = lane >= 1 && lane <= 30 && c + 1 < n;
    // y-faces: A at column c (between c-1 and c), B at c+1 (between c and c+1); needed for columns in
    // [c0, min(c0+60, n)]; the statistics count each face once (face n with the last strip)
    const int cA = c, cB = c + 1;
    const bool needA = lane >= 1 && cA >= c0 && cA <= c0 + STRIP_W && cA <= n;
    const bool needB = lane >= 1 && cB >= c0 && cB <= c0 + STRIP_W && cB <= n;
    const bool ownA = needA && (cA < c0 + STRIP_W || cA == n), ownB = needB && (cB < c0 + STRIP_W || cB == n);

    // prologue: values of rows r0-2 .. r0+1, previous slopes of rows r0-1, r0
    SV2 Vm, V0, Vp, Va;
    SS2 Sm, P;
    {
        auto rowfast = [&](int j) { return colfast && j >= 0 && j < m; };
        strip_load_vals(a, r0 - 2, c, rowfast(r0 - 2), Va);
        strip_load_vals(a, r0 - 1, c, rowfast(r0 - 1), Vm);
        strip_load_vals(a, r0, c, rowfast(r0), V0);
        strip_load_vals(a, r0 + 1, c, rowfast(r0 + 1), Vp);
        SS2 Pm;
        strip_load_prev(a, r0 - 1, c, rowfast(r0 - 1), Pm);
        strip_load_prev(a, r0, c, rowfast(r0), P);
        if (r0 == 0 && ghost_rows) {
            // slopes of ghost row -1 from row 0's
            SS2 S0;
            strip_slopes(a, Vm, V0, Vp, P, ahx, ihx, ahy, ihy, S0);
            if (edge_cols)
                strip_ghost_cols(a, c, S0);
            strip_ghost_row(a, S0, true, Sm);
        } else {
            strip_slopes(a, Va, Vm, V0, Pm, ahx, ihx, ahy, ihy, Sm);
            if (edge_cols)
                strip_ghost_cols(a, c, Sm);
        }
    }
    float2 E = make_float2(0.f, 0.f);
    SF2 XFm;
#pragma unroll 1
    for (int r = r0; r <= r1; ++r) {
        // slopes of row r
        SS2 S0;
        if (r == m && ghost_rows) {
            strip_ghost_row(a, Sm, false, S0);
        } else {
            strip_slopes(a, Vm, V0, Vp, P, ahx, ihx, ahy, ihy, S0);
            if (edge_cols)
                strip_ghost_cols(a, c, S0);
        }
        // x-faces of row r: between cells (r-1, col) and (r, col)
        SF2 XF0;
        {
            SSide2 L, R;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                L.x[X_RHO + k] = p_fma(p_s(hhx), Sm.s[k], Vm.w[k]);
                L.x[X_DRHO + k] = Sm.s[k];
                L.x[X_TRHO + k] = Sm.t[k];
                R.x[X_RHO + k] = p_fma(p_s(-hhx), S0.s[k], V0.w[k]);
                R.x[X_DRHO + k] = S0.s[k];
                R.x[X_TRHO + k] = S0.t[k];
            }
            bool ux, uy;
            int kx, ky;
            strip_face_pair(L, R, G, a.tau, a.htau, XF0, ux, uy, kx, ky);
            const bool vx = upd_x, vy = upd_y;  // x-faces of the columns this strip updates
            const bool qx = vx && (!ux || kx == 2), qy = vy && (!uy || ky == 2);
            if (vx && !qx && kx)
                report_face(a.ctl, slot, 0, (unsigned long long)c * (m + 1) + r, kx);
            if (vy && !qy && ky)
                report_face(a.ctl, slot, 0, (unsigned long long)(c + 1) * (m + 1) + r, ky);
            const bool own_row = r < r1 || r == m;
            strip_queue<LEARNED>(q, L, R, qx, qy, ux && qx, uy && qy, own_row, own_row, false, r, c, r, c + 1, fa, M,
                                 stats3, XF0);
        }
        // prefetch the next rows (after the x-faces, while the y-faces are computed)
        SV2 Vn;
        SS2 Pn;
        float2 En = make_float2(0.f, 0.f);
        if (r < r1) {
            const bool fv = colfast && r + 2 < m && r + 2 >= 0;
            strip_load_vals(a, r + 2, c, fv, Vn);
            strip_load_prev(a, r + 1, c, colfast && r + 1 < m, Pn);
            if (colfast)
                En = ldg2(a.src_w + 4 * a.plane + (size_t)r * a.ld + c);
            else if (upd_x || upd_y) {
                const size_t o = (size_t)r * a.ld;
                En = make_float2(upd_x ? a.src_w[4 * a.plane + o + c] : 0.f,
                                 upd_y ? a.src_w[4 * a.plane + o + c + 1] : 0.f);
            }
        }
        if (r > r0) {
            // y-faces of row r-1 (Vm, Sm): A between columns c-1 and c, B between c and c+1
            const int q1 = r - 1;
            SF2 YF;
            {
                float2 plus[4], minus[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    plus[k] = p_fma(p_s(hhy), Sm.t[k], Vm.w[k]);
                    minus[k] = p_fma(p_s(-hhy), Sm.t[k], Vm.w[k]);
                }
                // column c-1 (the lane below's second column)
                float pl[4], tl[4], sl[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    pl[k] = __shfl_up_sync(FULL, plus[k].y, 1);
                    tl[k] = __shfl_up_sync(FULL, Sm.t[k].y, 1);
                    sl[k] = __shfl_up_sync(FULL, Sm.s[k].y, 1);
                }
                // normal frame of a y-face: normal velocity v, tangential -u; normal derivatives
                // the y-slopes (t0, t2, -t1, t3), tangential the x-slopes (-s0, -s2, s1, -s3)
                SSide2 L, R;
                L.x[X_RHO] = make_float2(pl[0], plus[0].x);
                L.x[X_U] = make_float2(pl[2], plus[2].x);
                L.x[X_V] = make_float2(-pl[1], -plus[1].x);
                L.x[X_P] = make_float2(pl[3], plus[3].x);
                L.x[X_DRHO] = make_float2(tl[0], Sm.t[0].x);
                L.x[X_DU] = make_float2(tl[2], Sm.t[2].x);
                L.x[X_DV] = make_float2(-tl[1], -Sm.t[1].x);
                L.x[X_DP] = make_float2(tl[3], Sm.t[3].x);
                L.x[X_TRHO] = make_float2(-sl[0], -Sm.s[0].x);
                L.x[X_TU] = make_float2(-sl[2], -Sm.s[2].x);
                L.x[X_TV] = make_float2(sl[1], Sm.s[1].x);
                L.x[X_TP] = make_float2(-sl[3], -Sm.s[3].x);
                const float2 neg = p_s(-1.f);
                R.x[X_RHO] = minus[0];
                R.x[X_U] = minus[2];
                R.x[X_V] = p_mul(neg, minus[1]);
                R.x[X_P] = minus[3];
                R.x[X_DRHO] = Sm.t[0];
                R.x[X_DU] = Sm.t[2];
                R.x[X_DV] = p_mul(neg, Sm.t[1]);
                R.x[X_DP] = Sm.t[3];
                R.x[X_TRHO] = p_mul(neg, Sm.s[0]);
                R.x[X_TU] = p_mul(neg, Sm.s[2]);
                R.x[X_TV] = Sm.s[1];
                R.x[X_TP] = p_mul(neg, Sm.s[3]);
                bool ux, uy;
                int kx, ky;
                strip_face_pair(L, R, G, a.tau, a.htau, YF, ux, uy, kx, ky);
                const bool qx = needA && (!ux || kx == 2), qy = needB && (!uy || ky == 2);
                if (needA && !qx && kx)
                    report_face(a.ctl, slot, 1, (unsigned long long)q1 * (n + 1) + cA, kx);
                if (needB && !qy && ky)
                    report_face(a.ctl, slot, 1, (unsigned long long)q1 * (n + 1) + cB, ky);
                strip_queue<LEARNED>(q, L, R, qx, qy, ux && qx, uy && qy, ownA, ownB, true, q1, cA, q1, cB, fa,
                                     M, stats3, YF);
            }
            // update of row r-1: x-faces r-1 (XFm) and r (XF0), y-faces A, B and the next lane's A
            float2 Ar[8];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                Ar[t] = make_float2(YF.F[t].y, __shfl_down_sync(FULL, YF.F[t].x, 1));
                Ar[4 + t] = make_float2(YF.I[t].y, __shfl_down_sync(FULL, YF.I[t].x, 1));
            }
            if (upd_x || upd_y) {
                const float2 nu = p_s(a.nu), mu = p_s(a.mu);
                // y-face fluxes in the global frame: x-momentum -Ft, y-momentum Fn
                const float2 dFx0 = p_sub(XF0.F[0], XFm.F[0]), dFy0 = p_sub(Ar[0], YF.F[0]);
                const float2 dFx1 = p_sub(XF0.F[1], XFm.F[1]), dFy1 = p_sub(YF.F[2], Ar[2]);  // -(Ft_r - Ft_l)
                const float2 dFx2 = p_sub(XF0.F[2], XFm.F[2]), dFy2 = p_sub(Ar[1], YF.F[1]);
                const float2 dFx3 = p_sub(XF0.F[3], XFm.F[3]), dFy3 = p_sub(Ar[3], YF.F[3]);
                const float2 rho = Vm.w[0];
                const float2 mom_x = p_sub(p_sub(p_mul(rho, Vm.w[1]), p_mul(nu, dFx1)), p_mul(mu, dFy1));
                const float2 mom_y = p_sub(p_sub(p_mul(rho, Vm.w[2]), p_mul(nu, dFx2)), p_mul(mu, dFy2));
                const float2 ene = p_sub(p_sub(p_mul(rho, E), p_mul(nu, dFx3)), p_mul(mu, dFy3));
                const float2 rn = p_sub(p_sub(rho, p_mul(nu, dFx0)), p_mul(mu, dFy0));
                const float2 irn = p_rcp(rn);
                const float2 un = p_mul(mom_x, irn), vn = p_mul(mom_y, irn), En2 = p_mul(ene, irn);
                const float2 pn = p_mul(p_sub(p_sub(ene, p_mul(p_mul(p_s(0.5f), mom_x), un)), p_mul(p_mul(p_s(0.5f), mom_y), vn)),
                                        p_s(G.gm1));
                if ((upd_x && (pn.x < G.eps || rn.x < G.eps)) || (upd_y && (pn.y < G.eps || rn.y < G.eps)))
                    bad = 1u;
                float2 ns[4], nt[4];
                const float2 ihx2 = p_s(ihx), ihy2 = p_s(ihy);
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    ns[t] = p_mul(p_sub(XF0.I[t], XFm.I[t]), ihx2);
                // y-face I in the global frame: (I0, -B, A, I3)
                nt[0] = p_mul(p_sub(Ar[4], YF.I[0]), ihy2);
                nt[1] = p_mul(p_sub(YF.I[2], Ar[6]), ihy2);
                nt[2] = p_mul(p_sub(Ar[5], YF.I[1]), ihy2);
                nt[3] = p_mul(p_sub(Ar[7], YF.I[3]), ihy2);
                const size_t o = (size_t)q1 * a.ld + c;
                float* dw = a.dst_w + o;
                if (upd_x && upd_y) {
                    *reinterpret_cast<float2*>(dw) = rn;
                    *reinterpret_cast<float2*>(dw + a.plane) = un;
                    *reinterpret_cast<float2*>(dw + 2 * a.plane) = vn;
                    *reinterpret_cast<float2*>(dw + 3 * a.plane) = pn;
                    *reinterpret_cast<float2*>(dw + 4 * a.plane) = En2;
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        *reinterpret_cast<float2*>(a.dst_s + t * a.plane + o) = ns[t];
                        *reinterpret_cast<float2*>(a.dst_t + t * a.plane + o) = nt[t];
                    }
                } else {  // upd_x only (the last column of the domain is this pair's first)
                    dw[0] = rn.x;
                    dw[a.plane] = un.x;
                    dw[2 * a.plane] = vn.x;
                    dw[3 * a.plane] = pn.x;
                    dw[4 * a.plane] = En2.x;
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        a.dst_s[t * a.plane + o] = ns[t].x;
                        a.dst_t[t * a.plane + o] = nt[t].x;
                    }
                }
            }
        }
        // advance
        Vm = V0;
        V0 = Vp;
        Vp = Vn;
        Sm = S0;
        P = Pn;
        XFm = XF0;
        E = En;
    }
}

// The warp's update positivity flag and Newton statistics into the control
// block ctl (launch slot `slot`); clears them.  Warp-collective.
__device__ __forceinline__ void strip_report(Ctl* ctl, int slot, int stats, int* stats3, unsigned& bad)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    if (__any_sync(FULL, bad != 0u) && lane == 0)
        atomicOr(&ctl->upd_bad[slot], 1u);
    if (stats) {
        for (int off = 16; off; off >>= 1) {
            stats3[0] += __shfl_xor_sync(FULL, stats3[0], off);
            stats3[1] += __shfl_xor_sync(FULL, stats3[1], off);
            stats3[2] += __shfl_xor_sync(FULL, stats3[2], off);
        }
        if (lane == 0 && stats3[0]) {
            atomicAdd(&ctl->newton_faces, (unsigned long long)stats3[0]);
            atomicAdd(&ctl->newton_iters, (unsigned long long)stats3[1]);
            if (stats3[2])
                atomicAdd(&ctl->newton_fallbacks, (unsigned long long)stats3[2]);
        }
    }
    bad = 0u;
    stats3[0] = stats3[1] = stats3[2] = 0;
}

template <int NW, int MINB, bool LEARNED>
__global__ void __launch_bounds__(NW * 32, MINB) k_step_strip(const __grid_constant__ StepArgs<float> a,
                                                              const __grid_constant__ StripArgs sa)
{
    using SM = StripSmem<NW, LEARNED>;
    const unsigned FULL = 0xffffffffu;
    if (halt_prologue(a.ctl, a.seq))
        return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* q = reinterpret_cast<float*>(smem_raw + warp * SM::q_bytes);
    const MlpShared* M = reinterpret_cast<const MlpShared*>(smem_raw + SM::mlp_off);
    if (LEARNED) {
        if (sa.mlp_global) {  // (block-uniform) no shared-memory image: the launch did not allocate one
            M = reinterpret_cast<const MlpShared*>(a.mlp_img);
        } else {
            mlp_load_shared(*reinterpret_cast<MlpShared*>(smem_raw + SM::mlp_off), a.mlp_frag, a.mlp_prm,
                            threadIdx.x, NW * 32);
            __syncthreads();
        }
    }
    if (threadIdx.x == 0 && blockIdx.x == 0)
        sa.work[(a.seq + 1) % 3] = 0u;  // the next launch's counter (this launch's was cleared by the previous one)
    unsigned int* counter = sa.work + a.seq % 3;
    const int nstrip = (a.n + STRIP_W - 1) / STRIP_W;
    const int nunits = nstrip * ((a.m + sa.seg - 1) / sa.seg);
    int stats3[3] = {0, 0, 0};
    unsigned bad = 0;
    for (;;) {
        int u = 0;
        if (lane == 0)
            u = (int)atomicAdd(counter, 1u);
        u = __shfl_sync(FULL, u, 0);
        if (u >= nunits)
            break;
        const int seg = u / nstrip, strip = u - seg * nstrip;
        const int r0 = seg * sa.seg;
        strip_unit<LEARNED>(a, &a.G, strip * STRIP_W, r0, (r0 + sa.seg < a.m) ? r0 + sa.seg : a.m, q, M, sa.mlp_min,
                            sa.mlp_jump2, stats3, bad);
    }
    strip_report(a.ctl, a.seq % 3, a.stats, stats3, bad);
}

}  // namespace hydro
