// hydro_device.cuh -- device point solvers of the Eulerian Godunov/GRP step.
//
// Everything here is per-interface arithmetic: the minmod limiters, the exact
// Riemann solver (Newton on the star pressure), the quasi-1D direct-Eulerian
// GRP solver and the GRP flux of an axis-aligned interface.  The templates are
// instantiated in FP64 (parity form: each expression keeps the reference's
// operand order; the translation unit is compiled with --fmad=false so no
// multiply-add is contracted, and division/sqrt are IEEE) and in FP32.
//
// Algorithms follow (file:line in the reference project):
//   minmod2 / minmod3            src/include/tools.h:44-73
//   exact Riemann solver         src/riemann_solver/riemann_solver_exact_Ben.c:30-211
//   quasi-1D GRP (lambda = 0)    src/riemann_solver/linear_grp_solver_Edir_Q1D.c:38-554
//   GRP_2D_flux                  src/flux_calc/flux_solver.c:158-237
//   star_dire_check (dim 2)      src/inter_process/fluid_var_check.c:111-128
//
// Two exact simplifications relative to the reference's generic code, both
// identical in value up to the sign of a zero result: the frame velocity is 0
// (GRP_2D_flux sets lambda_u = lambda_v = 0, so every `x - lambda` is `x`), and
// the interface normal is (1,0) or (0,1), so the rotation to the normal frame
// is a relabelling (x-faces: normal u, tangential v; y-faces: normal v,
// tangential -u).  The sign of a zero never changes a comparison, so every
// branch is taken exactly as in the reference.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "hydro_pow.cuh"
#include "libm_pow.cuh"

// FP64 pow: by default the C library's method (libm_pow.cuh), so that the
// parity form rounds every pow as the reference does; compiled with
// -DHYDRO_POW_CR=1, the correctly rounded double-double pow (hydro_pow.cuh),
// kept for comparison.
#ifndef HYDRO_POW_CR
#define HYDRO_POW_CR 0
#endif

namespace hydro {

template <typename R> struct M;
template <> struct M<double> {
    static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
#if HYDRO_POW_CR
    static __device__ __forceinline__ double pow_(double x, double y) { return dd_pow(x, y); }
#else
    static __device__ __forceinline__ double pow_(double x, double y) { return lpow(x, y); }
#endif
    static __device__ __forceinline__ double abs_(double x) { return fabs(x); }
    static __device__ __forceinline__ double log_(double x) { return log(x); }
    static __device__ __forceinline__ bool finite_(double x)
    {
        return (__double_as_longlong(x) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
    }
};
template <> struct M<float> {
    static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
    static __device__ __forceinline__ float pow_(float x, float y) { return exp2f(y * __log2f(x)); }
    static __device__ __forceinline__ float abs_(float x) { return fabsf(x); }
    static __device__ __forceinline__ float log_(float x) { return logf(x); }
    static __device__ __forceinline__ bool finite_(float x)
    {
        return (__float_as_int(x) & 0x7f800000) != 0x7f800000;
    }
};

// ---------------------------------------------------------------------------
// minmod limiters (tools.h:44-73)
// ---------------------------------------------------------------------------
// FP32 form: the same values without branches.  When the arguments share a
// sign (the only case that does not return 0), the reference's comparison
// sequence returns the argument of smallest magnitude, i.e. the minimum of
// positive or the maximum of negative arguments; fminf/fmaxf return that
// argument exactly.  (They differ from the sequence only for NaN arguments,
// which the reconstruction check rejects anyway.)
__device__ __forceinline__ float minmod2_sel(float sL, float sR)
{
    const float r = sR > 0.f ? fminf(sL, sR) : fmaxf(sL, sR);
    return sL * sR <= 0.f ? 0.f : r;
}
__device__ __forceinline__ float minmod3_sel(float sL, float sR, float sm)
{
    const float r = sm > 0.f ? fminf(fminf(sL, sR), sm) : fmaxf(fmaxf(sL, sR), sm);
    return (sL * sm <= 0.f || sR * sm <= 0.f) ? 0.f : r;
}

// FP64 form: the reference's comparison sequence with the comparisons done on
// the bit patterns, exactly.  On GB300 an FP64 comparison occupies the FP64
// pipe; done as integer operations the FP64 step measured 2% faster
// (30.9 against 31.5 ms at 4096², the same results bit for bit).  Only finite
// arguments take this path (others keep
// the IEEE comparisons); the products stay FP64, because "s sm <= 0" must see
// an underflow to zero as the reference does.  With finite arguments:
//  - a product is never NaN, so "p <= 0" is "p is a zero or negative";
//  - past that test the arguments are non-zero and share a sign, where "a < b"
//    is an unsigned comparison of the bit patterns (reversed for negatives).
__device__ __forceinline__ bool d_finite(double x)
{
    return (__double_as_longlong(x) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool d_le0(double p)  // p <= 0 for a p that is not NaN
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(p);
    return (b >> 63) != 0ull || b == 0ull;
}
// a < b for non-zero, non-NaN a and b of the sign neg
__device__ __forceinline__ bool d_lt_same_sign(double a, double b, bool neg)
{
    const unsigned long long x = (unsigned long long)__double_as_longlong(a),
                             y = (unsigned long long)__double_as_longlong(b);
    return neg ? x > y : x < y;
}
__device__ __forceinline__ double minmod2_d(double sL, double sR)
{
    if (!(d_finite(sL) && d_finite(sR))) {  // the reference's sequence as written
        if (sL * sR <= 0.0)
            return 0.0;
        if (sR > 0.0 && sR < sL)
            return sR;
        if (sR <= 0.0 && sR > sL)
            return sR;
        return sL;
    }
    if (d_le0(sL * sR))
        return 0.0;
    const bool neg = __double_as_longlong(sR) < 0;
    // positive: sR < sL; negative: sR > sL
    if (neg ? d_lt_same_sign(sL, sR, true) : d_lt_same_sign(sR, sL, false))
        return sR;
    return sL;
}
__device__ __forceinline__ double minmod3_d(double sL, double sR, double sm)
{
    if (!(d_finite(sL) && d_finite(sR) && d_finite(sm))) {
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
    if (d_le0(sL * sm) || d_le0(sR * sm))
        return 0.0;
    const bool neg = __double_as_longlong(sm) < 0;
    // positive: sm < sL && sm < sR; negative: sm > sL && sm > sR
    if (neg ? (d_lt_same_sign(sL, sm, true) && d_lt_same_sign(sR, sm, true))
            : (d_lt_same_sign(sm, sL, false) && d_lt_same_sign(sm, sR, false)))
        return sm;
    // positive: sR < sL; negative: sR > sL
    if (neg ? d_lt_same_sign(sL, sR, true) : d_lt_same_sign(sR, sL, false))
        return sR;
    return sL;
}

template <typename R>
__device__ __forceinline__ R minmod2(R sL, R sR)
{
    if constexpr (sizeof(R) == 4)
        return minmod2_sel(sL, sR);
    else
        return minmod2_d(sL, sR);
    if (sL * sR <= R(0))
        return R(0);
    if (sR > R(0) && sR < sL)
        return sR;
    if (sR <= R(0) && sR > sL)
        return sR;
    return sL;
}

template <typename R>
__device__ __forceinline__ R minmod3(R sL, R sR, R sm)
{
    if constexpr (sizeof(R) == 4)
        return minmod3_sel(sL, sR, sm);
    else
        return minmod3_d(sL, sR, sm);
    if (sL * sm <= R(0) || sR * sm <= R(0))
        return R(0);
    if (sm > R(0) && sm < sL && sm < sR)
        return sm;
    if (sm <= R(0) && sm > sL && sm > sR)
        return sm;
    if (sR > R(0) && sR < sL)
        return sR;
    if (sR <= R(0) && sR > sL)
        return sR;
    return sL;
}

// ---------------------------------------------------------------------------
// gas constants of one run, computed once on the host with the same IEEE
// operations the reference performs inline
// ---------------------------------------------------------------------------
template <typename R>
struct Gas {
    R g;      // gamma
    R gm1;    // gamma - 1
    R zeta;   // (gamma-1)/(gamma+1)
    R mu;     // (gamma-1)/(2 gamma)
    R nu;     // (gamma+1)/(2 gamma)
    R g_g1;   // gamma/(gamma-1), flux energy factor
    R inv_g;  // 1/gamma (star density on a rarefaction)
    R cexp;   // 0.5*(gamma-1)/gamma (star sound speed on a rarefaction)
    R sexp;   // 2 gamma/(gamma-1) (sonic-point pressure)
    R e1;     // 0.5/zeta
    R e2;     // (1+zeta)/zeta
    R opz;    // 1 + zeta
    R op2z;   // 1 + 2 zeta
    R eps;
    double g64, eps64;  // FP64 copies for the FP32 form's FP64 Newton fallback
    double dist2_max;   // FP64 uniform-pair test: sqrt(d2) < eps exactly when d2 <= dist2_max
                        // (set on the host; a device-side gas_fill leaves -1, no pair uniform)
};

// The largest double d2 whose correctly rounded square root is below eps, or -1
// when there is none (eps <= 0 or NaN).  The rounded square root is
// non-decreasing in its argument, so for every double d2 >= 0, NaN and +inf
// included, sqrt(d2) < eps holds exactly when d2 <= dist2_max: the FP64 form's
// uniform-pair test makes the reference's decision without the square root.
// eps * eps lies within a few units in the last place of the limit; each walk
// below takes a few steps (bounded all the same).
__host__ __device__ inline double uniform_dist2_max(double eps)
{
    if (!(eps > 0.0))
        return -1.0;
    const double big = 1.7976931348623157e308;  // the largest finite double
    double x = eps * eps;
    if (!(x <= big))
        x = big;
    for (int k = 0; k < 4096 && !(sqrt(x) < eps); ++k)  // down into the set (sqrt(0) = 0 < eps)
        x = nextafter(x, 0.0);
    for (int k = 0; k < 4096; ++k) {  // up to its last element
        const double y = nextafter(x, 2.0 * big);
        if (!(y <= big) || !(sqrt(y) < eps))
            break;
        x = y;
    }
    return x;
}

// The constants of a Gas, derived in FP64 (host for the kernels' arguments;
// device for the FP32 form's FP64 retry of a face).
template <typename R>
__host__ __device__ inline void gas_fill(Gas<R>& G, double g, double eps)
{
    double zeta = (g - 1.0) / (g + 1.0);
    G.g = (R)g;
    G.gm1 = (R)(g - 1.0);
    G.zeta = (R)zeta;
    G.mu = (R)((g - 1.0) / (2.0 * g));
    G.nu = (R)((g + 1.0) / (2.0 * g));
    G.g_g1 = (R)(g / (g - 1.0));
    G.inv_g = (R)(1.0 / g);
    G.cexp = (R)(0.5 * (g - 1.0) / g);
    G.sexp = (R)(2.0 * g / (g - 1.0));
    G.e1 = (R)(0.5 / zeta);
    G.e2 = (R)((1.0 + zeta) / zeta);
    G.opz = (R)(1.0 + zeta);
    G.op2z = (R)(1.0 + 2.0 * zeta);
    G.eps = (R)eps;
    G.g64 = g;
    G.eps64 = eps;
#ifdef __CUDA_ARCH__
    G.dist2_max = -1.0;  // the caller passes the host's value where the test runs
#else
    G.dist2_max = uniform_dist2_max(eps);
#endif
}

// Velocity on the 1-wave curve through (uL,pL) at pressure pp (shock for pp > pL,
// rarefaction otherwise): riemann_solver_exact_Ben.c:50-62.
template <typename R>
__device__ __forceinline__ R curve_left(R pp, R uL, R pL, R cL, const Gas<R>& G)
{
    R w;
    if (pp > pL) {
        R dp = pp - pL;
        w = M<R>::sqrt_(R(1) + G.nu * dp / pL);
        w = dp * cL / G.g / pL / w;
        return uL - w;
    }
    w = M<R>::pow_(pp / pL, G.mu) - R(1);
    w = R(2) * cL * w / G.gm1;
    return uL - w;
}

// 3-wave curve through (uR,pR): riemann_solver_exact_Ben.c:64-76.
template <typename R>
__device__ __forceinline__ R curve_right(R pp, R uR, R pR, R cR, const Gas<R>& G)
{
    R w;
    if (pp > pR) {
        R dp = pp - pR;
        w = M<R>::sqrt_(R(1) + G.nu * dp / pR);
        w = dp * cR / G.g / pR / w;
        return uR + w;
    }
    w = M<R>::pow_(pp / pR, G.mu) - R(1);
    w = R(2) * cR * w / G.gm1;
    return uR + w;
}

// Derivative du/dp of the 1-wave curve at pp (k1 of the Newton loop, :136-149).
template <typename R>
__device__ __forceinline__ R slope_left(R pp, R pL, R cL, const Gas<R>& G)
{
    R t1, t2, t3;
    if (pp > pL) {
        R dp = pp - pL;
        t1 = R(1) / M<R>::sqrt_(R(1) + G.nu * dp / pL);
        t2 = cL / G.g / pL;
        t3 = R(0.5) * t2 * G.nu / pL;
        return t3 * dp * M<R>::pow_(t1, R(3)) - t2 * t1;
    }
    t2 = cL / G.g / pL;
    t1 = R(1) / M<R>::pow_(pp / pL, G.nu);
    return -t1 * t2;
}

// Derivative of the 3-wave curve (k3, :150-164).
template <typename R>
__device__ __forceinline__ R slope_right(R pp, R pR, R cR, const Gas<R>& G)
{
    R t1, t2, t3;
    if (pp > pR) {
        R dp = pp - pR;
        t1 = R(1) / M<R>::sqrt_(R(1) + G.nu * dp / pR);
        t2 = cR / G.g / pR;
        t3 = R(0.5) * t2 * G.nu / pR;
        return t2 * t1 - t3 * dp * M<R>::pow_(t1, R(3));
    }
    t2 = cR / G.g / pR;
    t1 = R(1) / M<R>::pow_(pp / pR, G.nu);
    return t1 * t2;
}

// Powers of one base x with the logarithm computed once: pow(y) equals
// M<R>::pow_(x, y) bit for bit (for FP64 it is the pow's own path after its
// logarithm).  The wave curve of a rarefaction side and the curve's slope need
// x^mu and x^nu of the same pressure ratio.
template <typename R> struct PowBase;
#if !HYDRO_POW_CR
template <> struct PowBase<double> {
    LpowBase b;
    __device__ __forceinline__ void init(double x) { b.init(x); }
    __device__ __forceinline__ double pow(double y) const { return b.pow_y(y); }
};
#else
template <> struct PowBase<double> {
    double x, lh, ll;
    bool dd;  // x in (0, inf): the double-double path of dd_pow
    __device__ __forceinline__ void init(double x_)
    {
        x = x_;
        dd = (x > 0.0) && (x < INFINITY);
        lh = ll = 0.0;
        if (dd)
            dd_log(x, lh, ll);
    }
    __device__ __forceinline__ double pow(double y) const
    {
        if (!dd || !(y - y == 0.0))
            return ::pow(x, y);
        if (y == 0.0 || x == 1.0)
            return 1.0;
        const double th = y * lh;
        const double tl = fma(y, lh, -th) + y * ll;
        if (!(fabs(th) < 700.0))
            return ::pow(x, y);
        return dd_exp(th, tl);
    }
};
#endif
template <> struct PowBase<float> {
    float l2;
    __device__ __forceinline__ void init(float x) { l2 = __log2f(x); }
    __device__ __forceinline__ float pow(float y) const { return exp2f(y * l2); }
};

// One side's wave curve at pressure pp (curve_left / curve_right) and the
// curve's slope there (slope_left / slope_right, k1 / k3 of the Newton loop),
// computed together so that they share the square root of a shock side and the
// logarithm of a rarefaction side; each value equals the separate function's
// bit for bit.  LEFT: the 1-wave (u - w), else the 3-wave (u + w).
template <typename R>
struct CurveSlope {
    R v, k;
};

// The per-side quantities of the slope that do not change with the pressure:
// t2 = c / gamma / p and t3 = 0.5 t2 nu / p (slope_left :136-149, slope_right
// :150-164 recompute them every iteration; the values are the same).
template <typename R>
struct SideConst {
    R t2, t3;
};

template <typename R>
__device__ __forceinline__ SideConst<R> side_const(R p, R c, const Gas<R>& G)
{
    SideConst<R> s;
    s.t2 = c / G.g / p;
    s.t3 = R(0.5) * s.t2 * G.nu / p;
    return s;
}

template <typename R, bool LEFT>
__device__ __forceinline__ CurveSlope<R> curve_slope_body(R pp, R u, R p, R c, const Gas<R>& G, SideConst<R> K)
{
    CurveSlope<R> r;
    R w;
    if (pp > p) {
        const R dp = pp - p;
        const R sq = M<R>::sqrt_(R(1) + G.nu * dp / p);
        w = dp * c / G.g / p / sq;
        const R t1 = R(1) / sq;
        const R cube = M<R>::pow_(t1, R(3));
        r.k = LEFT ? K.t3 * dp * cube - K.t2 * t1 : K.t2 * t1 - K.t3 * dp * cube;
    } else {
        PowBase<R> pb;
        pb.init(pp / p);
        w = pb.pow(G.mu) - R(1);
        w = R(2) * c * w / G.gm1;
        const R t1 = R(1) / pb.pow(G.nu);
        r.k = LEFT ? -t1 * K.t2 : t1 * K.t2;
    }
    r.v = LEFT ? u - w : u + w;
    return r;
}

// FP64: out of line (its double-double temporaries stay out of the callers'
// register allocation; the result comes back in registers).
template <bool LEFT>
__device__ __noinline__ CurveSlope<double> curve_slope_f64(double pp, double u, double p, double c, double g,
                                                          double gm1, double mu, double nu, double t2, double t3)
{
    Gas<double> G;
    G.g = g;
    G.gm1 = gm1;
    G.mu = mu;
    G.nu = nu;
    return curve_slope_body<double, LEFT>(pp, u, p, c, G, SideConst<double>{t2, t3});
}

template <typename R, bool LEFT>
__device__ __forceinline__ void curve_slope_at(R pp, R u, R p, R c, const Gas<R>& G, SideConst<R> K, R& v, R& k)
{
    CurveSlope<R> r;
    if constexpr (sizeof(R) == 8)
        r = curve_slope_f64<LEFT>(pp, u, p, c, G.g, G.gm1, G.mu, G.nu, K.t2, K.t3);
    else
        r = curve_slope_body<R, LEFT>(pp, u, p, c, G, K);
    v = r.v;
    k = r.k;
}

struct StarInfo {
    int iters;     // Newton iterations taken (-1 when the uniform-pair shortcut was used)
    int crw0, crw1;
    int fallback;  // FP32 form: 1 when the FP64 Newton iteration was used
};

// Exact Riemann solver, riemann_solver_exact_Ben.c:30-211 (single gamma).
// Starting pressure: the reference's half linearised intersection (:86-93).
// FUSED: each Newton pressure's curves and slopes come from curve_slope_at;
// otherwise the curves and slopes are evaluated separately, as the reference
// writes them (the same values; the FP32 forms' FP64 retry keeps this form,
// whose smaller footprint leaves their kernels' register allocation alone).
template <typename R, bool FUSED = true>
__device__ __forceinline__ void exact_riemann(R uL, R uR, R pL, R pR, R cL, R cR, R tol, int N,
                                              const Gas<R>& G, R& u_star, R& p_star, StarInfo& st)
{
    R uLR = curve_left(pR, uL, pL, cL, G);
    R uRL = curve_right(pL, uR, pR, cR, G);
    st.crw1 = (uLR > uR + G.eps) ? 0 : 1;
    st.crw0 = (uRL > uL - G.eps) ? 1 : 0;

    R k1 = -cL / pL / G.g;
    R k3 = cR / pR / G.g;
    R p_int = (k1 * pL - k3 * pR - uL + uR) / (k1 - k3);
    if (p_int < R(0))
        p_int = (pL < pR) ? pL : pR;
    p_int = R(0.5) * p_int;

    if (M<R>::abs_(uL - uR) < tol && M<R>::abs_(pL - pR) < tol) {
        p_star = R(0.5) * (pL + pR);
        u_star = R(0.5) * (uL + uR);
        st.iters = 0;
        return;
    }
    if constexpr (!FUSED) {
        R vL = curve_left(p_int, uL, pL, cL, G);
        R vR = curve_right(p_int, uR, pR, cR, G);
        R gap = M<R>::abs_(vL - vR);
        int it = 0;
        while ((gap > tol) && (it != N)) {
            k1 = slope_left(p_int, pL, cL, G);
            k3 = slope_right(p_int, pR, cR, G);
            R p_new = p_int + (vR - vL) / (k1 - k3);
            if (p_new < R(0))
                p_int = R(0.5) * p_int;
            else
                p_int = p_new;
            ++it;
            vL = curve_left(p_int, uL, pL, cL, G);
            vR = curve_right(p_int, uR, pR, cR, G);
            gap = M<R>::abs_(vL - vR);
        }
        u_star = k1 * (vR - vL) / (k1 - k3) + vL;
        p_star = p_int;
        st.iters = it;
        return;
    }
    // curves and slopes at the current pressure (the slopes are the next
    // iteration's k1, k3; k1, k3 themselves stay those of the last iteration)
    R vL, vR, k1n, k3n;
    const SideConst<R> KL = side_const(pL, cL, G), KR = side_const(pR, cR, G);
    curve_slope_at<R, true>(p_int, uL, pL, cL, G, KL, vL, k1n);
    curve_slope_at<R, false>(p_int, uR, pR, cR, G, KR, vR, k3n);
    R gap = M<R>::abs_(vL - vR);
    int it = 0;
    while ((gap > tol) && (it != N)) {
        k1 = k1n;
        k3 = k3n;
        R p_new = p_int + (vR - vL) / (k1 - k3);
        if (p_new < R(0))
            p_int = R(0.5) * p_int;
        else
            p_int = p_new;
        ++it;
        curve_slope_at<R, true>(p_int, uL, pL, cL, G, KL, vL, k1n);
        curve_slope_at<R, false>(p_int, uR, pR, cR, G, KR, vR, k3n);
        gap = M<R>::abs_(vL - vR);
    }
    u_star = k1 * (vR - vL) / (k1 - k3) + vL;
    p_star = p_int;
    st.iters = it;
}

// One side of an interface in the interface's normal frame.
template <typename R>
struct Side {
    R rho, u, v, p;      // u normal, v tangential velocity
    R drho, du, dv, dp;  // normal derivatives
    R trho, tu, tv, tp;  // tangential derivatives
};

// Star-region state handed from the Riemann solve to the GRP case tree.
template <typename R>
struct Star {
    R u_star, p_star, rho_star_L, rho_star_R, c_star_L, c_star_R, speed_L, speed_R, c_L, c_R;
    int crw0, crw1;
    int acoustic;  // dist < atc (the uniform-pair shortcut of the 2D path)
};

// How the star state is found, per precision.
//  FP64: exactly the reference (uniform-pair shortcut dist < eps, exact solver
//        with tol = eps, at most 500 iterations).
//  FP32: the shortcut and the Newton tolerance are relative to the states'
//        magnitudes (an absolute 1e-9 is below FP32 resolution), Newton runs in
//        FP32 from the given starting pressure (the learned guess) or the
//        reference's start, and falls back to the FP64 reference iteration when
//        FP32 does not converge or the star pressure is near vacuum
//        (p* < 1e-3 min(pL, pR): strong rarefactions).
template <typename R> struct StarPolicy;

template <> struct StarPolicy<double> {
    static __device__ __forceinline__ bool uniform(double dist, double, const Gas<double>& G) { return dist < G.eps; }
    template <bool FUSED = true>
    static __device__ __forceinline__ void solve(double uL, double uR, double pL, double pR, double cL, double cR,
                                                 const Gas<double>& G, double, double& u_star, double& p_star,
                                                 StarInfo& st)
    {
        exact_riemann<double, FUSED>(uL, uR, pL, pR, cL, cR, G.eps, 500, G, u_star, p_star, st);
        st.fallback = 0;
    }
};


// FP64 reference iteration used by the FP32 form for hard faces; kept out of
// line so its FP64 register footprint does not burden the common path.
static __device__ __noinline__ void exact_riemann_fp64_fallback(float uL, float uR, float pL, float pR, float cL, float cR,
                                                         double g, double eps, float& u_star, float& p_star,
                                                         StarInfo& st);

template <> struct StarPolicy<float> {
    static __device__ __forceinline__ bool uniform(float dist, float scale, const Gas<float>& G)
    {
        return dist < threshold(scale, G);
    }
    // the uniform-pair distance threshold, relative to the states' magnitude
    static __device__ __forceinline__ float threshold(float scale, const Gas<float>& G)
    {
        return fmaxf(G.eps, 1e-6f * scale);
    }
    template <bool FUSED = true>  // (FP32: one form)
    static __device__ void solve(float uL, float uR, float pL, float pR, float cL, float cR, const Gas<float>& G,
                                 float p_start, float& u_star, float& p_star, StarInfo& st)
    {
        st.fallback = 0;
        float uLR = curve_left(pR, uL, pL, cL, G);
        float uRL = curve_right(pL, uR, pR, cR, G);
        st.crw1 = (uLR > uR + G.eps) ? 0 : 1;
        st.crw0 = (uRL > uL - G.eps) ? 1 : 0;
        const float tol = 1e-6f * (cL + cR);
        float k1 = -cL / pL / G.g;
        float k3 = cR / pR / G.g;
        float p;
        if (p_start > 0.f) {
            p = p_start;
        } else {
            // the intersection of the wave curves' tangents at the two states
            // (riemann_solver_exact_Ben.c:87-93).  The reference starts from half
            // of it (p_start <= -2 asks for that start); the FP32 form starts from
            // the intersection itself: for the weak waves that make up most exact
            // faces it is second-order accurate, and Newton from it needs 0-1
            // iterations instead of about 4 (on an increasing concave function a
            // start right of the root costs one step to its left)
            p = (k1 * pL - k3 * pR - uL + uR) / (k1 - k3);
            if (p < 0.f)
                p = 0.5f * fminf(pL, pR);  // the reference's fallback, halved as it halves it
            else if (p_start <= -2.f)
                p = 0.5f * p;
        }
        float vL = curve_left(p, uL, pL, cL, G);
        float vR = curve_right(p, uR, pR, cR, G);
        float gap = fabsf(vL - vR);
        int it = 0;
        while (gap > tol && it < 24) {
            k1 = slope_left(p, pL, cL, G);
            k3 = slope_right(p, pR, cR, G);
            float pn = p + (vR - vL) / (k1 - k3);
            p = (pn < 0.f) ? 0.5f * p : pn;
            ++it;
            vL = curve_left(p, uL, pL, cL, G);
            vR = curve_right(p, uR, pR, cR, G);
            gap = fabsf(vL - vR);
        }
        st.iters = it;
        if (!(gap <= tol) || p < 1e-3f * fminf(pL, pR)) {
            int it32 = st.iters;
            exact_riemann_fp64_fallback(uL, uR, pL, pR, cL, cR, G.g64, G.eps64, u_star, p_star, st);
            st.iters += it32;
            st.fallback = 1;
            return;
        }
        u_star = (it > 0) ? k1 * (vR - vL) / (k1 - k3) + vL : 0.5f * (vL + vR);
        p_star = p;
    }
};

static __device__ __noinline__ void exact_riemann_fp64_fallback(float uL, float uR, float pL, float pR, float cL, float cR,
                                                         double g, double eps, float& u_star, float& p_star,
                                                         StarInfo& st)
{
    Gas<double> D;
    double zeta = (g - 1.0) / (g + 1.0);
    D.g = g;
    D.gm1 = g - 1.0;
    D.zeta = zeta;
    D.mu = (g - 1.0) / (2.0 * g);
    D.nu = (g + 1.0) / (2.0 * g);
    D.eps = eps;
    double us, ps;
    exact_riemann<double, false>((double)uL, (double)uR, (double)pL, (double)pR, (double)cL, (double)cR, eps, 500, D, us, ps,
                          st);
    u_star = (float)us;
    p_star = (float)ps;
}

template <typename R>
__device__ __forceinline__ void q1d_waves(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G, Star<R>& S);

// Non-uniform pairs: exact solver and the waves of the star state.  Out of line:
// only a few percent of the faces of piecewise-smooth data get here, and
// keeping it separate leaves the common (uniform-pair) path its registers.
template <typename R, bool FUSED = true>
__device__ __forceinline__ void q1d_star_exact_body(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G, Star<R>& S,
                                                    StarInfo& st, R p_start)
{
    StarPolicy<R>::template solve<FUSED>(L.u, Rr.u, L.p, Rr.p, S.c_L, S.c_R, G, p_start, S.u_star, S.p_star, st);
    S.crw0 = st.crw0;
    S.crw1 = st.crw1;
    q1d_waves(L, Rr, G, S);
}
template <typename R, bool FUSED = true>
__device__ __noinline__ void q1d_star_exact(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G, Star<R>& S,
                                            StarInfo& st, R p_start)
{
    q1d_star_exact_body<R, FUSED>(L, Rr, G, S, st, p_start);
}

// Star state of linear_GRP_solver_Edir_Q1D (:92-134) with atc = eps:
// uniform pairs (dist < eps) take the averaged state, all others the exact solver.
// The uniform-pair test of q1d_star (the acoustic case), on its own: used to
// sort faces before solving them; q1d_star makes the decision again itself.
// RS selects the interface solver: 0 = quasi-1D (linear_grp_solver_Edir_Q1D.c:95-96),
// 1 = genuinely 2D, whose distance also counts the tangential velocity jump
// (linear_grp_solver_Edir_G2D.c:112).
template <typename R, int RS = 0>
__device__ __forceinline__ bool face_uniform(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G)
{
    const R rho_L = L.rho, rho_R = Rr.rho, u_L = L.u, u_R = Rr.u, p_L = L.p, p_R = Rr.p;
    if constexpr (sizeof(R) == 8) {
        // dist = sqrt(d2) < eps, decided on d2 itself (uniform_dist2_max): the
        // same decision as the reference's, without an IEEE square root per face
        R d2 = (rho_L - rho_R) * (rho_L - rho_R) + (u_L - u_R) * (u_L - u_R);
        if constexpr (RS == 1)
            d2 = d2 + (L.v - Rr.v) * (L.v - Rr.v);
        d2 = d2 + (p_L - p_R) * (p_L - p_R);
        return d2 <= G.dist2_max;
    } else {
        // FP32: the squared distance against the squared threshold (as the strip
        // kernel's packed test), no square root
        R d2 = (rho_L - rho_R) * (rho_L - rho_R) + (u_L - u_R) * (u_L - u_R) + (p_L - p_R) * (p_L - p_R);
        R scale = rho_L + rho_R + p_L + p_R + M<R>::abs_(u_L) + M<R>::abs_(u_R);
        if constexpr (RS == 1) {
            d2 = d2 + (L.v - Rr.v) * (L.v - Rr.v);
            scale = scale + M<R>::abs_(L.v) + M<R>::abs_(Rr.v);
        }
        const R th = StarPolicy<R>::threshold(scale, G);
        return d2 < th * th;
    }
}

// KNOWN: 0 = make the uniform-pair decision here; 1 / 2 = the caller has
// already made it with face_uniform (1 uniform, 2 not), so only that branch
// is compiled into the caller.  FUSED: as for exact_riemann.
template <typename R, int KNOWN = 0, int RS = 0, bool FUSED = true>
__device__ __forceinline__ void q1d_star(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G, Star<R>& S,
                                         StarInfo& st, R p_start = R(-1))
{
    const R rho_L = L.rho, rho_R = Rr.rho, u_L = L.u, u_R = Rr.u, p_L = L.p, p_R = Rr.p;
    S.c_L = M<R>::sqrt_(G.g * p_L / rho_L);
    S.c_R = M<R>::sqrt_(G.g * p_R / rho_R);
    if constexpr (KNOWN == 0)
        S.acoustic = face_uniform<R, RS>(L, Rr, G);
    else
        S.acoustic = (KNOWN == 1);
    if (S.acoustic) {
        S.u_star = R(0.5) * (u_R + u_L);
        S.p_star = R(0.5) * (p_R + p_L);
        S.rho_star_L = rho_L;
        S.c_star_L = S.c_L;
        S.speed_L = S.u_star - S.c_star_L;
        S.rho_star_R = rho_R;
        S.c_star_R = S.c_R;
        S.speed_R = S.u_star + S.c_star_R;
        S.crw0 = S.crw1 = 0;
        st.iters = -1;
        st.crw0 = st.crw1 = 0;
        st.fallback = 0;
        return;
    }
    if constexpr (KNOWN != 1)  // no out-of-line call (and its addressed arguments) on the uniform path
    {
        // FP32: the exact path inline (no call, no arguments through the stack);
        // FP64: out of line, as its register footprint would burden the common path
        if constexpr (sizeof(R) == 4)
            q1d_star_exact_body<R, FUSED>(L, Rr, G, S, st, p_start);
        else
            q1d_star_exact<R, FUSED>(L, Rr, G, S, st, p_start);
    }
}

// Waves of the star state (linear_grp_solver_Edir_Q1D.c:110-133).
template <typename R>
__device__ __forceinline__ void q1d_waves(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G, Star<R>& S)
{
    if (S.acoustic)
        return;
    const R rho_L = L.rho, rho_R = Rr.rho, u_L = L.u, u_R = Rr.u, p_L = L.p, p_R = Rr.p;
    const R p_star = S.p_star;
    if (S.crw0) {
        S.rho_star_L = rho_L * M<R>::pow_(p_star / p_L, G.inv_g);
        S.c_star_L = S.c_L * M<R>::pow_(p_star / p_L, G.cexp);
        S.speed_L = u_L - S.c_L;
    } else {
        S.rho_star_L = rho_L * (p_star + G.zeta * p_L) / (p_L + G.zeta * p_star);
        S.c_star_L = M<R>::sqrt_(G.g * p_star / S.rho_star_L);
        S.speed_L = u_L - S.c_L * M<R>::sqrt_(R(0.5) * ((G.g + R(1)) * (p_star / p_L) + G.gm1) / G.g);
    }
    if (S.crw1) {
        S.rho_star_R = rho_R * M<R>::pow_(p_star / p_R, G.inv_g);
        S.c_star_R = S.c_R * M<R>::pow_(p_star / p_R, G.cexp);
        S.speed_R = u_R + S.c_R;
    } else {
        S.rho_star_R = rho_R * (p_star + G.zeta * p_R) / (p_R + G.zeta * p_star);
        S.c_star_R = M<R>::sqrt_(G.g * p_star / S.rho_star_R);
        S.speed_R = u_R + S.c_R * M<R>::sqrt_(R(0.5) * ((G.g + R(1)) * (p_star / p_R) + G.gm1) / G.g);
    }
}

template <typename R>
__device__ __noinline__ void q1d_derivs_exact(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G, const Star<R>& S,
                                              R D[4], R U[4]);
template <typename R>
__device__ __forceinline__ void q1d_derivs_exact_body(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G,
                                                      const Star<R>& S, R D[4], R U[4]);

template <typename R>
__device__ __noinline__ void g2d_derivs_exact(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G,
                                              const Star<R>& S, R D[4], R U[4]);

// Time derivatives D and t-axis values U of the quasi-1D GRP given the star
// state: linear_grp_solver_Edir_Q1D.c:139-545 with lambda = 0.
// KNOWN as in q1d_star (1: S is the acoustic case, 2: it is not).  RS = 1: the
// genuinely-2D solver, whose acoustic case is this one
// (linear_grp_solver_Edir_G2D.c:156-271) and whose non-acoustic case is
// g2d_derivs_exact (g2d.cuh).
template <typename R, int KNOWN = 0, int RS = 0>
__device__ __forceinline__ void q1d_derivs(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G, const Star<R>& S,
                                           R D[4], R U[4])
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
    R C = R(0);

    if (KNOWN != 2 && S.acoustic) {  // acoustic case (:139-254); CRW branches are unreachable here
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
        R D_rho, D_u, D_v, D_p, T_rho, T_u, T_v, T_p;
        if (u_star > R(0)) {
            U[0] = rho_star_L; U[1] = u_star; U[2] = v_L; U[3] = p_star;
            C = c_star_L;
        } else {
            U[0] = rho_star_R; U[1] = u_star; U[2] = v_R; U[3] = p_star;
            C = c_star_R;
        }
        const R rc = U[0] * C;
        D_p = R(0.5) * ((d_u_L * rc + d_p_L) - (d_u_R * rc - d_p_R));
        T_p = R(0.5) * ((t_u_L * rc + t_p_L) - (t_u_R * rc - t_p_R));
        D_u = R(0.5) * (d_u_L + d_p_L / rc + d_u_R - d_p_R / rc);
        T_u = R(0.5) * (t_u_L + t_p_L / rc + t_u_R - t_p_R / rc);
        const R cc = C * C;
        if (u_star > R(0)) {
            D_v = d_v_L;
            T_v = t_v_L;
            D_rho = d_rho_L - d_p_L / cc + D_p / cc;
            T_rho = t_rho_L - t_p_L / cc + T_p / cc;
        } else {
            D_v = d_v_R;
            T_v = t_v_R;
            D_rho = d_rho_R - d_p_R / cc + D_p / cc;
            T_rho = t_rho_R - t_p_R / cc + T_p / cc;
        }
        D[0] = -U[1] * D_rho - U[2] * T_rho - U[0] * (D_u + T_v);
        D[1] = -U[1] * D_u - U[2] * T_u - D_p / U[0];
        D[2] = -U[1] * D_v - U[2] * T_v - T_p / U[0];
        D[3] = -U[1] * D_p - U[2] * T_p - U[0] * C * C * (D_u + T_v);
        return;
    }
    if constexpr (KNOWN != 1) {
        if constexpr (RS == 1)
            g2d_derivs_exact(L, Rr, G, S, D, U);
        else if constexpr (sizeof(R) == 4)
            q1d_derivs_exact_body<R>(L, Rr, G, S, D, U);
        else
            q1d_derivs_exact(L, Rr, G, S, D, U);
    }
}

// Non-acoustic case of the quasi-1D GRP (:256-547), out of line like q1d_star_exact.
template <typename R>
__device__ __forceinline__ void q1d_derivs_exact_body(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G,
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
    R C = R(0);

    // non-acoustic case (:256-547)
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
    if (S.crw0 && ((u_star - c_star_L) > R(0))) {  // sonic point in the 1-rarefaction
        U[1] = zetaL * (u_L + R(2) * c_L / G.gm1);
        C = U[1];
        U[3] = M<R>::pow_(C / c_L, G.sexp) * p_L;
        U[0] = gL * U[3] / C / C;
        U[2] = v_L;
        R c_frac = C / c_L;
        R TdS = (d_p_L - d_rho_L * c_L * c_L) / G.gm1 / rho_L;
        R d_Psi = d_u_L + (gL * d_p_L / c_L - c_L * d_rho_L) / G.gm1 / rho_L;
        R pe1 = M<R>::pow_(c_frac, G.e1), pe2 = M<R>::pow_(c_frac, G.e2);
        D[1] = (G.opz * pe1 + zetaL * pe2);
        D[1] = D[1] / G.op2z * TdS;
        D[1] = D[1] - c_L * pe1 * d_Psi;
        D[3] = U[0] * U[1] * D[1];
        D[0] = U[0] * U[1] * pe2 * TdS * G.gm1;
        D[0] = (D[0] + D[3]) / C / C;
        D[2] = -U[1] * d_v_L * U[0] / rho_L;
    } else if (S.crw1 && ((u_star + c_star_R) < R(0))) {  // sonic point in the 3-rarefaction
        U[1] = zetaR * (u_R - R(2) * c_R / G.gm1);
        C = R(0) - U[1];
        U[3] = M<R>::pow_(C / c_R, G.sexp) * p_R;
        U[0] = gR * U[3] / C / C;
        U[2] = v_R;
        R c_frac = C / c_R;
        R TdS = (d_p_R - d_rho_R * c_R * c_R) / G.gm1 / rho_R;
        R d_Phi = d_u_R - (gR * d_p_R / c_R - c_R * d_rho_R) / G.gm1 / rho_R;
        R pe1 = M<R>::pow_(c_frac, G.e1), pe2 = M<R>::pow_(c_frac, G.e2);
        D[1] = (G.opz * pe1 + zetaR * pe2);
        D[1] = D[1] / G.op2z * TdS;
        D[1] = D[1] + c_R * pe1 * d_Phi;
        D[3] = U[0] * U[1] * D[1];
        D[0] = U[0] * U[1] * pe2 * TdS * G.gm1;
        D[0] = (D[0] + D[3]) / C / C;
        D[2] = -U[1] * d_v_R * U[0] / rho_R;
    } else {  // non-sonic case
        R a_L, b_L, d_L, a_R, b_R, d_R;
        if (u_star < R(0)) {
            U[0] = rho_star_R; U[1] = u_star; U[2] = v_R; U[3] = p_star;
            C = c_star_R;
        } else {
            U[0] = rho_star_L; U[1] = u_star; U[2] = v_L; U[3] = p_star;
            C = c_star_L;
        }
        if (S.crw0) {
            a_L = R(1);
            b_L = R(1) / rho_star_L / c_star_L;
            R c_frac = c_star_L / c_L;
            R TdS = (d_p_L - d_rho_L * c_L * c_L) / G.gm1 / rho_L;
            R d_Psi = d_u_L + (gL * d_p_L / c_L - c_L * d_rho_L) / G.gm1 / rho_L;
            R pe1 = M<R>::pow_(c_frac, G.e1), pe2 = M<R>::pow_(c_frac, G.e2);
            d_L = (G.opz * pe1 + zetaL * pe2);
            d_L = d_L / G.op2z * TdS;
            d_L = d_L - c_L * pe1 * d_Psi;
        } else {
            R SmUs = -M<R>::sqrt_(R(0.5) * ((gL + R(1)) * p_L + G.gm1 * p_star) / rho_star_L);
            R SmUL = -M<R>::sqrt_(R(0.5) * ((gL + R(1)) * p_star + G.gm1 * p_L) / rho_L);
            R VAR = M<R>::sqrt_((R(1) - zetaL) / (rho_L * (p_star + zetaL * p_L)));
            R H1 = R(0.5) * VAR * (p_star + G.op2z * p_L) / (p_star + zetaL * p_L);
            R H2 = R(-0.5) * VAR * ((R(2) + zetaL) * p_star + zetaL * p_L) / (p_star + zetaL * p_L);
            R H3 = R(-0.5) * VAR * (p_star - p_L) / rho_L;
            R L_p = R(-1) / rho_L - SmUL * H2;
            R L_u = SmUL + rho_L * (c_L * c_L * H2 + H3);
            R L_rho = -SmUL * H3;
            a_L = R(1) - rho_star_L * SmUs * H1;
            b_L = -SmUs / (rho_star_L * c_star_L * c_star_L) + H1;
            d_L = L_rho * d_rho_L + L_u * d_u_L + L_p * d_p_L;
        }
        if (S.crw1) {
            a_R = R(1);
            b_R = R(-1) / rho_star_R / c_star_R;
            R c_frac = c_star_R / c_R;
            R TdS = (d_p_R - d_rho_R * c_R * c_R) / G.gm1 / rho_R;
            R d_Phi = d_u_R - (gR * d_p_R / c_R - c_R * d_rho_R) / G.gm1 / rho_R;
            R pe1 = M<R>::pow_(c_frac, G.e1), pe2 = M<R>::pow_(c_frac, G.e2);
            d_R = (G.opz * pe1 + zetaR * pe2);
            d_R = d_R / G.op2z * TdS;
            d_R = d_R + c_R * pe1 * d_Phi;
        } else {
            R SmUs = M<R>::sqrt_(R(0.5) * ((gR + R(1)) * p_R + G.gm1 * p_star) / rho_star_R);
            R SmUR = M<R>::sqrt_(R(0.5) * ((gR + R(1)) * p_star + G.gm1 * p_R) / rho_R);
            R VAR = M<R>::sqrt_((R(1) - zetaR) / (rho_R * (p_star + zetaR * p_R)));
            R H1 = R(0.5) * VAR * (p_star + G.op2z * p_R) / (p_star + zetaR * p_R);
            R H2 = R(-0.5) * VAR * ((R(2) + zetaR) * p_star + zetaR * p_R) / (p_star + zetaR * p_R);
            R H3 = R(-0.5) * VAR * (p_star - p_R) / rho_R;
            R L_p = R(-1) / rho_R + SmUR * H2;
            R L_u = SmUR - rho_R * (c_R * c_R * H2 + H3);
            R L_rho = SmUR * H3;
            a_R = R(1) + rho_star_R * SmUs * H1;
            b_R = -(SmUs / (rho_star_R * c_star_R * c_star_R) + H1);
            d_R = L_rho * d_rho_R + L_u * d_u_R + L_p * d_p_R;
        }
        R detA = a_L * b_R - b_L * a_R;
        R u_t_mat = (b_R * d_L - b_L * d_R) / detA;
        R p_t_mat = (a_L * d_R - a_R * d_L) / detA;
        D[1] = u_t_mat + u_star / U[0] / C / C * p_t_mat;
        D[3] = p_t_mat + u_star * U[0] * u_t_mat;
        if (u_star < R(0)) {
            if (S.crw1) {
                D[0] = rho_star_R * u_star * M<R>::pow_(c_star_R / c_R, G.e2) * (d_p_R - d_rho_R * c_R * c_R) / rho_R;
                D[0] = (D[0] + D[3]) / c_star_R / c_star_R;
                D[2] = -U[1] * d_v_R * U[0] / rho_R;
                D[2] = D[2] + R(0) * d_v_R;
            } else {
                R SmUs = M<R>::sqrt_(R(0.5) * ((gR + R(1)) * p_R + G.gm1 * p_star) / rho_star_R);
                R SmUR = M<R>::sqrt_(R(0.5) * ((gR + R(1)) * p_star + G.gm1 * p_R) / rho_R);
                R VAR = p_R + zetaR * p_star;
                R H1 = rho_R * p_R * (R(1) - zetaR * zetaR) / VAR / VAR;
                R H2 = rho_R * p_star * (zetaR * zetaR - R(1)) / VAR / VAR;
                R H3 = (p_star + zetaR * p_R) / VAR;
                R L_rho = SmUR * H3 * d_rho_R;
                R L_u = -rho_R * (H2 * c_R * c_R + H3) * d_u_R;
                R L_p = H2 * SmUR * d_p_R;
                D[0] = ((u_star + SmUs) / c_star_R / c_star_R - u_star * H1) * p_t_mat + rho_star_R * u_star * SmUs * H1 * u_t_mat;
                D[0] = (D[0] - u_star * (L_p + L_rho + L_u)) / SmUs;
                // the frame-velocity term lambda*rho_x is 0*rho_x; it is kept because a
                // stationary 3-shock (SmUR + u_R == 0) makes it NaN in the reference too
                R f = SmUR * (H2 * d_p_R + H3 * d_rho_R) - rho_R * (H2 * c_R * c_R + H3) * d_u_R;
                R rho_x = (f + H1 * (p_t_mat - rho_star_R * SmUs * u_t_mat) - D[0]) / (SmUR + u_R);
                D[0] = D[0] + R(0) * rho_x;
                D[2] = -U[1] * SmUR * d_v_R / SmUs;
                D[2] = D[2] + R(0) * d_v_R;
            }
        } else {
            if (S.crw0) {
                D[0] = rho_star_L * u_star * M<R>::pow_(c_star_L / c_L, G.e2) * (d_p_L - d_rho_L * c_L * c_L) / rho_L;
                D[0] = (D[0] + D[3]) / c_star_L / c_star_L;
                D[2] = -U[1] * d_v_L * U[0] / rho_L;
                D[2] = D[2] + R(0) * d_v_L;
            } else {
                R SmUs = -M<R>::sqrt_(R(0.5) * ((gL + R(1)) * p_L + G.gm1 * p_star) / rho_star_L);
                R SmUL = -M<R>::sqrt_(R(0.5) * ((gL + R(1)) * p_star + G.gm1 * p_L) / rho_L);
                R VAR = p_L + zetaL * p_star;
                R H1 = rho_L * p_L * (R(1) - zetaL * zetaL) / VAR / VAR;
                R H2 = rho_L * p_star * (zetaL * zetaL - R(1)) / VAR / VAR;
                R H3 = (p_star + zetaL * p_L) / VAR;
                R L_rho = SmUL * H3 * d_rho_L;
                R L_u = -rho_L * (H2 * c_L * c_L + H3) * d_u_L;
                R L_p = H2 * SmUL * d_p_L;
                D[0] = ((u_star + SmUs) / c_star_L / c_star_L - H1 * u_star) * p_t_mat + rho_star_L * u_star * SmUs * H1 * u_t_mat;
                D[0] = (D[0] - u_star * (L_p + L_rho + L_u)) / SmUs;
                R f = SmUL * (H2 * d_p_L + H3 * d_rho_L) - rho_L * (H2 * c_L * c_L + H3) * d_u_L;
                R rho_x = (f + H1 * (p_t_mat - rho_star_L * SmUs * u_t_mat) - D[0]) / (SmUL + u_L);
                D[0] = D[0] + R(0) * rho_x;
                D[2] = -U[1] * SmUL * d_v_L / SmUs;
                D[2] = D[2] + R(0) * d_v_L;
            }
        }
    }
    // transversal terms (:524-545)
    const R rc = U[0] * C;
    R T_p = R(0.5) * ((t_u_L * rc + t_p_L) - (t_u_R * rc - t_p_R));
    R T_u = R(0.5) * (t_u_L + t_p_L / rc + t_u_R - t_p_R / rc);
    const R cc = C * C;
    if (u_star > R(0)) {
        R T_rho = t_rho_L - t_p_L / cc + T_p / cc;
        D[0] = D[0] - U[2] * T_rho - U[0] * t_v_L;
        D[1] = D[1] - U[2] * T_u;
        D[2] = D[2] - U[2] * t_v_L - T_p / U[0];
        D[3] = D[3] - U[2] * T_p - U[0] * C * C * t_v_L;
    } else {
        R T_rho = t_rho_R - t_p_R / cc + T_p / cc;
        D[0] = D[0] - U[2] * T_rho - U[0] * t_v_R;
        D[1] = D[1] - U[2] * T_u;
        D[2] = D[2] - U[2] * t_v_R - T_p / U[0];
        D[3] = D[3] - U[2] * T_p - U[0] * C * C * t_v_R;
    }
}
template <typename R>
__device__ __noinline__ void q1d_derivs_exact(const Side<R>& L, const Side<R>& Rr, const Gas<R>& G, const Star<R>& S,
                                              R D[4], R U[4])
{
    q1d_derivs_exact_body<R>(L, Rr, G, S, D, U);
}

// Interface result: mid-time flux (F_rho, F_u, F_v, F_e) in the x/y frame and
// the t+tau interface values (rho, u, v, p).
template <typename R>
struct FaceOut {
    R F[4];
    R I[4];
};

// Assemble the GRP_2D_flux outputs (flux_solver.c:195-220) of an axis-aligned
// face from the normal-frame t-axis values U and derivatives D.  YDIR: the
// normal is +y, so the x-velocity is minus the tangential velocity.
template <typename R>
__device__ __forceinline__ void face_flux(const R D[4], const R U[4], R tau, R htau, const Gas<R>& G, FaceOut<R>& o,
                                          bool YDIR)
{
    R rho_mid = U[0] + htau * D[0];
    R a = U[1] + htau * D[1];  // normal velocity at t + tau/2
    R b = U[2] + htau * D[2];  // tangential velocity at t + tau/2
    R p_mid = U[3] + htau * D[3];
    R F_rho = rho_mid * a;
    R F_e = G.g_g1 * p_mid / rho_mid + R(0.5) * (a * a + b * b);
    if (!YDIR) {
        o.F[0] = F_rho;
        o.F[1] = F_rho * a + p_mid;
        o.F[2] = F_rho * b;
    } else {
        o.F[0] = F_rho;
        o.F[1] = F_rho * (-b);
        o.F[2] = F_rho * a + p_mid;
    }
    o.F[3] = F_rho * F_e;
    R A = U[1] + tau * D[1];
    R B = U[2] + tau * D[2];
    o.I[0] = U[0] + tau * D[0];
    o.I[3] = U[3] + tau * D[3];
    if (!YDIR) {
        o.I[1] = A;
        o.I[2] = B;
    } else {
        o.I[1] = -B;
        o.I[2] = A;
    }
}

// star_dire_check (dim 2): 1 = non-positive, 2 = non-finite t-axis value,
// 3 = non-finite derivative, 0 = fine.
template <typename R>
__device__ __forceinline__ int star_dire_check2(const R U[4], const R D[4], R eps)
{
    if (U[3] < eps || U[0] < eps)
        return 1;
    if constexpr (sizeof(R) == 4) {
        // FP32 form: a sum of magnitudes is finite iff every term is (barring
        // an overflow of the sum itself, which no usable state reaches): one
        // add per value instead of an exponent test
        if (!(fabsf(U[0]) + fabsf(U[1]) + fabsf(U[2]) + fabsf(U[3]) <= 3.402823466e38f))
            return 2;
        if (!(fabsf(D[0]) + fabsf(D[1]) + fabsf(D[2]) + fabsf(D[3]) <= 3.402823466e38f))
            return 3;
        return 0;
    } else {
        if (!(M<R>::finite_(U[0]) && M<R>::finite_(U[1]) && M<R>::finite_(U[2]) && M<R>::finite_(U[3])))
            return 2;
        if (!(M<R>::finite_(D[0]) && M<R>::finite_(D[1]) && M<R>::finite_(D[2]) && M<R>::finite_(D[3])))
            return 3;
        return 0;
    }
}

// ifvar_check (dim 2), fluid_var_check.c:21-51: reconstructed positivity and
// finite derivatives; non-zero means the interface reports error code 1.
template <typename R>
__device__ __forceinline__ bool ifvar_bad(const Side<R>& L, const Side<R>& Rr, R eps)
{
    if (L.p < eps || Rr.p < eps || L.rho < eps || Rr.rho < eps)
        return true;
    if constexpr (sizeof(R) == 4) {
        // FP32 form: finiteness of all 16 slopes from one sum of magnitudes (see star_dire_check2)
        const float s = fabsf(L.dp) + fabsf(Rr.dp) + fabsf(L.du) + fabsf(Rr.du) + fabsf(L.dv) + fabsf(Rr.dv) +
                        fabsf(L.drho) + fabsf(Rr.drho) + fabsf(L.tp) + fabsf(Rr.tp) + fabsf(L.tu) + fabsf(Rr.tu) +
                        fabsf(L.tv) + fabsf(Rr.tv) + fabsf(L.trho) + fabsf(Rr.trho);
        return !(s <= 3.402823466e38f);
    } else {
        bool f = M<R>::finite_(L.dp) && M<R>::finite_(Rr.dp) && M<R>::finite_(L.du) && M<R>::finite_(Rr.du) &&
                 M<R>::finite_(L.dv) && M<R>::finite_(Rr.dv) && M<R>::finite_(L.drho) && M<R>::finite_(Rr.drho) &&
                 M<R>::finite_(L.tp) && M<R>::finite_(Rr.tp) && M<R>::finite_(L.tu) && M<R>::finite_(Rr.tu) &&
                 M<R>::finite_(L.tv) && M<R>::finite_(Rr.tv) && M<R>::finite_(L.trho) && M<R>::finite_(Rr.trho);
        return !f;
    }
}

}  // namespace hydro

#include "g2d.cuh"
