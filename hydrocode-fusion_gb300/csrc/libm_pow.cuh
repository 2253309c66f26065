// libm_pow.cuh -- pow(x, y) computed the way the reference's C library
// computes it, for the FP64 parity form.
//
// Why: the reference calls the C library's pow (GNU libc) ten times per exact
// Riemann solve (riemann_solver_exact_Ben.c:59-197).  That pow is accurate to
// about 0.52 ulp, not correctly rounded: on a small fraction of arguments its
// last bit differs from the correctly rounded value, and over hundreds of
// steps those last-bit differences grow through the Newton stopping test and
// the limiter's switches.  Parity with the reference therefore needs the same
// rounding as the C library, which a correctly rounded pow cannot give.
//
// Method: the table-driven pow published by Szabolcs Nagy in Arm Optimized
// Routines, which GNU libc uses since version 2.28 (the variant for targets
// with fused multiply-add, which both x86-64 with FMA and AArch64 run):
//   log: x = 2^k z, z in [0x1.69555p-1, 0x1.69555p0) split into 128
//        subintervals; r = z/c - 1 exactly (one fma), c from the table with
//        log(c) as a 2^-43-rounded head and a tail; log x = k ln2 + log c + r
//        - r^2/2 + r^3 P(r), gathered as hi + lo with the r^2 term's rounding
//        error kept;
//   y log x as ehi + elo (one fma for the product's error);
//   exp: ehi = k ln2/128 + r (round-to-nearest k through the 1.5*2^52 shift),
//        r += elo, 2^(k/128) = H (1 + T) from the table, and the result
//        scale + scale * (T + r + C2 r^2 + ... + C5 r^5), scale = H 2^(k>>7).
// The tables and the polynomial coefficients are this project's own, made by
// csrc/gen_libm_pow_tables.py from that published description (its header
// says how each constant follows from it).  Operand order matters: the file is
// compiled without multiply-add contraction (FP64 translation units use
// --fmad=false, host builds -ffp-contract=off).
//
// Arguments outside what the Eulerian solvers can produce -- x <= 0 or not
// finite, y tiny/huge/not finite, |y log x| >= 512 (results near overflow or
// underflow) -- are passed to the platform's pow.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define LPOW_HD __device__
#define LPOW_TABLE(name, n) static __device__ const double name[n]
#define LPOW_UTABLE(name, n) static __device__ const uint64_t name[n]
#else  // plain C++ build of the same code (host-side tests, the oracle's twin)
#define LPOW_HD
#define LPOW_TABLE(name, n) static const double name[n]
#define LPOW_UTABLE(name, n) static const uint64_t name[n]
#endif

#include "libm_pow_tables.h"

namespace hydro {

LPOW_HD static inline double lpow_as_double(uint64_t b)
{
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
}

LPOW_HD static inline uint64_t lpow_as_bits(double d)
{
    uint64_t b;
    memcpy(&b, &d, sizeof(b));
    return b;
}

// log(x) = hi + lo for the bit pattern ix of a positive normal double.
LPOW_HD static inline void lpow_log(uint64_t ix, double& hi, double& lo)
{
    const uint64_t tmp = ix - LPOW_LOG_OFF;
    const int i = (int)((tmp >> 45) & 127);
    const int64_t k = (int64_t)tmp >> 52;
    const double z = lpow_as_double(ix - (tmp & (0xfffull << 52)));
    const double kd = (double)k;
    const double invc = lpow_log_tab[3 * i];
    const double logc = lpow_log_tab[3 * i + 1];
    const double logctail = lpow_log_tab[3 * i + 2];
    const double r = fma(z, invc, -1.0);  // exact: 1/c has few bits, |r| < 2^-7
    // k ln2 + log c + r, the first sum exact
    const double t1 = fma(kd, LPOW_LN2HI, logc);
    const double t2 = t1 + r;
    const double lo1 = fma(kd, LPOW_LN2LO, logctail);
    const double lo2 = t1 - t2 + r;
    // + (-r^2/2) with its rounding error
    const double ar = -0.5 * r;
    const double ar2 = r * ar;
    const double ar3 = r * ar2;
    const double h = t2 + ar2;
    const double lo3 = fma(ar, r, -ar2);
    const double lo4 = t2 - h + ar2;
    // + r^3 P(r); the coefficients carry the scale of ar2 = -r^2/2 and ar3 = -r^3/2
    const double q = fma(ar2, fma(ar2, fma(r, LPOW_A6, LPOW_A5), fma(r, LPOW_A4, LPOW_A3)), fma(r, LPOW_A2, LPOW_A1));
    const double l = fma(ar3, q, lo1 + lo2 + lo3 + lo4);
    hi = h + l;
    lo = h - hi + l;
}

// exp(x + xtail) for 2^-54 <= |x| < 512, |xtail| tiny against x.
LPOW_HD static inline double lpow_exp(double x, double xtail)
{
    double kd = fma(LPOW_INVLN2N, x, 0x1.8p52);  // round(x 128/ln2) in the low bits
    const uint64_t ki = lpow_as_bits(kd);
    kd -= 0x1.8p52;
    double r = fma(kd, LPOW_NEGLN2LON, fma(kd, LPOW_NEGLN2HIN, x));
    r += xtail;
    const int idx = 2 * (int)(ki & 127);
    const uint64_t top = ki << 45;  // (k >> 7) into the exponent field, mod 2^64
    const double tail = lpow_as_double(lpow_exp_tab[idx]);
    const uint64_t sbits = lpow_exp_tab[idx + 1] + top;
    const double r2 = r * r;
    const double tmp = fma(r2 * r2, fma(r, LPOW_C5, LPOW_C4), fma(r2, fma(r, LPOW_C3, LPOW_C2), tail + r));
    const double scale = lpow_as_double(sbits);
    return fma(scale, tmp, scale);
}

// Bit pattern of a positive finite x with its logarithm's head and tail, for
// several exponents of one base (the wave curve and its slope take x^mu and
// x^nu of the same pressure ratio): pow_y(y) equals lpow(x, y) bit for bit.
struct LpowBase {
    double x, hi, lo;
    bool main;  // x positive, finite and normal or subnormal: the table path
    LPOW_HD inline void init(double x_)
    {
        x = x_;
        uint64_t ix = lpow_as_bits(x);
        const uint32_t topx = (uint32_t)(ix >> 52);
        main = (topx - 0x001u < 0x7ffu - 0x001u) || (x > 0.0 && topx == 0);
        hi = lo = 0.0;
        if (!main)
            return;
        if (topx == 0) {  // subnormal: normalise
            ix = lpow_as_bits(x * 0x1p52) & 0x7fffffffffffffffull;
            ix -= 52ull << 52;
        }
        lpow_log(ix, hi, lo);
    }
    LPOW_HD inline double pow_y(double y) const
    {
        const uint32_t topy = (uint32_t)(lpow_as_bits(y) >> 52) & 0x7ffu;
        if (!main || topy - 0x3beu >= 0x43eu - 0x3beu)
            return ::pow(x, y);
        const double ehi = y * hi;
        const double elo = fma(y, lo, fma(y, hi, -ehi));
        const uint32_t abstop = (uint32_t)(lpow_as_bits(ehi) >> 52) & 0x7ffu;
        if (abstop - 0x3c9u >= 0x408u - 0x3c9u) {
            if (abstop < 0x3c9u)  // |y log x| < 2^-54
                return 1.0;
            return ::pow(x, y);  // near overflow/underflow
        }
        return lpow_exp(ehi, elo);
    }
};

LPOW_HD static inline double lpow(double x, double y)
{
    LpowBase b;
    b.init(x);
    return b.pow_y(y);
}

}  // namespace hydro
