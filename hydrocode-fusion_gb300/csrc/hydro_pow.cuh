// hydro_pow.cuh -- double-double pow(x, y) for the FP64 parity form.
//
// Why: every FP64 operation of the parity form rounds exactly as the
// reference's C code except pow(), where CUDA's libm (a couple of ulp) and
// glibc's (within ~0.52 ulp, i.e. almost always correctly rounded) disagree in
// the last bit for a sizeable fraction of arguments.  Those 1-ulp differences
// flip the reference's Newton stopping test (gap > 1e-9) on some faces, which
// moves p* by up to ~1e-9 there.  Computing pow to about 2^-70 relative
// before the final rounding makes it agree with a correctly rounded pow --
// and so with glibc -- on all but ~1e-5 of the arguments.
//
// Method: P.T.P. Tang's table-driven logarithm ("Table-driven implementation of
// the logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4),
// 1990) and exponential (ACM TOMS 15(2), 1989), carried in double-double
// arithmetic (exact products via fma, exact sums via Knuth's two-sum):
//   x = 2^e m, m in [1,2);  c = 1/(1+(i+1/2)/128) from the top 7 bits of m;
//   r = m c - 1 (exact as a double-double), |r| < 2^-8;
//   log x = e ln2 - log c + log1p(r)    (log1p by its Taylor series to r^8);
//   t = y log x;  t = k ln2/128 + s,  |s| <= ln2/256;
//   pow = 2^(k div 128) * 2^((k mod 128)/128) * (1 + expm1(s))  (series to s^7).
// The tables come from csrc/gen_pow_tables.py (60-digit decimal arithmetic).
// Arguments outside the solver's domain (x <= 0, non-finite, results near
// overflow/underflow) fall back to the platform pow.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define HYDRO_HD __device__
#define HYDRO_POW_TABLE(name, n) static __device__ const double name[n]
#else  // plain C++ build of the same code (host-side accuracy test)
#define HYDRO_HD
#define HYDRO_POW_TABLE(name, n) static const double name[n]
#endif

#include "hydro_pow_tables.h"

namespace hydro {

HYDRO_HD static inline void two_sum(double a, double b, double& s, double& e)
{
    s = a + b;
    double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

HYDRO_HD static inline void fast_two_sum(double a, double b, double& s, double& e)
{
    s = a + b;
    e = b - (s - a);
}

HYDRO_HD static inline double bits_to_double(uint64_t b)
{
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
}

HYDRO_HD static inline uint64_t double_to_bits(double d)
{
    uint64_t b;
    memcpy(&b, &d, sizeof(b));
    return b;
}

// log(x) as hi + lo for finite x > 0.
HYDRO_HD static inline void dd_log(double x, double& lh, double& ll)
{
    uint64_t b = double_to_bits(x);
    int e = (int)((b >> 52) & 0x7ff);
    if (e == 0) {  // subnormal: scale into the normal range
        b = double_to_bits(x * 0x1p54);
        e = (int)((b >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    const uint64_t mant = b & 0x000fffffffffffffull;
    const double m = bits_to_double(mant | 0x3ff0000000000000ull);  // [1, 2)
    const int i = (int)(mant >> 45);                                  // top 7 bits
    const double c = hydro_log_tab[3 * i], tlh = hydro_log_tab[3 * i + 1], tll = hydro_log_tab[3 * i + 2];
    // r = m c - 1 exactly: m c = ph + pl (fma), ph - 1 is exact (ph in [1-2^-8, 1+2^-8])
    const double ph = m * c;
    const double pl = fma(m, c, -ph);
    double rh, rl;
    fast_two_sum(ph - 1.0, pl, rh, rl);
    // log1p(r) = r - r^2/2 + r^3 (1/3 - r/4 + r^2/5 - r^3/6 + r^4/7 - r^5/8)
    const double r2h = rh * rh;
    const double r2l = fma(rh, rh, -r2h) + 2.0 * rh * rl;
    const double r3 = r2h * rh;
    const double tail =
        r3 * (1.0 / 3.0 + rh * (-0.25 + rh * (0.2 + rh * (-1.0 / 6.0 + rh * (1.0 / 7.0 + rh * (-0.125))))));
    double l1h, l1l;
    two_sum(rh, -0.5 * r2h, l1h, l1l);
    l1l += rl - 0.5 * r2l + tail;
    // e ln2 + (-log c) + log1p(r)
    const double ed = (double)e;
    double ah, al, bh, bl;
    two_sum(ed * HYDRO_LN2_HI, tlh, ah, al);
    two_sum(ah, l1h, bh, bl);
    const double low = al + bl + ed * HYDRO_LN2_LO + tll + l1l;
    fast_two_sum(bh, low, lh, ll);
}

// exp(th + tl) for |th| < 708.
HYDRO_HD static inline double dd_exp(double th, double tl)
{
    const double kd = rint(th * HYDRO_INV_LN2N);
    const long long k = (long long)kd;
    double sh, se;
    two_sum(th, -kd * HYDRO_LN2N_HI, sh, se);
    double sl = se + tl - kd * HYDRO_LN2N_LO;
    fast_two_sum(sh, sl, sh, sl);
    // expm1(s) = s + s^2/2 + s^3 (1/6 + s/24 + s^2/120 + s^3/720 + s^4/5040)
    const double qh = sh * sh;
    const double ql = fma(sh, sh, -qh) + 2.0 * sh * sl;
    const double tail = qh * sh * (1.0 / 6.0 + sh * (1.0 / 24.0 + sh * (1.0 / 120.0 + sh * (1.0 / 720.0 + sh * (1.0 / 5040.0)))));
    double eh, el;
    two_sum(sh, 0.5 * qh, eh, el);
    el += sl + 0.5 * ql + tail;
    const int j = (int)(k & 127);
    const long long q = (k - j) / 128;
    const double Th = hydro_exp_tab[2 * j], Tl = hydro_exp_tab[2 * j + 1];
    // T (1 + em1) = Th + Th eh + (Tl + Tl eh + Th el)
    const double ph = Th * eh;
    const double pl = fma(Th, eh, -ph);
    double rh, re;
    two_sum(Th, ph, rh, re);
    const double r = rh + (re + pl + Tl + Tl * eh + Th * el);
    // scale by 2^q (q in the normal range here)
    return r * bits_to_double((uint64_t)(q + 1023) << 52);
}

// x^3 for 2^-300 < x < 2^300: x*x exactly as a double-double (fma), times x
// again with the product's high part exact, so the value before the final
// rounding is within about 2^-104 of x^3 -- a correctly rounded cube except for
// arguments within that distance of a rounding boundary, which is far tighter
// than the general path's ~2^-70.  (The solvers' Newton slope takes
// pow(t, 3.0) of every shock side in every iteration.)
HYDRO_HD static inline double dd_cube(double x)
{
    const double ph = x * x;
    const double pl = fma(x, x, -ph);
    const double qh = ph * x;
    const double ql = fma(ph, x, -qh) + pl * x;
    return qh + ql;
}

HYDRO_HD static inline double dd_pow(double x, double y)
{
    if (!(x > 0.0) || !(x < INFINITY) || !(y - y == 0.0))
        return pow(x, y);
    if (y == 0.0 || x == 1.0)
        return 1.0;
    if (y == 3.0 && x > 0x1p-300 && x < 0x1p300)
        return dd_cube(x);
    double lh, ll;
    dd_log(x, lh, ll);
    const double th = y * lh;
    const double tl = fma(y, lh, -th) + y * ll;
    if (!(fabs(th) < 700.0))
        return pow(x, y);
    return dd_exp(th, tl);
}

}  // namespace hydro
