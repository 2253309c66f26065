"""Generates csrc/libm_pow_tables.h: the constants of libm_pow.cuh, the pow()
that follows the method of the C library the reference links against.

The method is the table-driven pow published by Szabolcs Nagy (Arm
Optimized Routines, the pow of GNU libc since version 2.28).  Its parameters,
as published, and how each constant below is derived from them:

  logarithm, N = 128 subintervals of z in [0x1.69555p-1, 0x1.69555p0), split
  evenly in the bit pattern of z (bits 45..51 above the interval's start):
    1/c  = round(N/m)/N     for a subinterval whose midpoint m < 1,
           round(2N/m)/(2N) otherwise,
           so r = z/c - 1 is exact in double precision and c = 1 exactly
           around z = 1;
    logc = log(c) rounded to a multiple of 2^-43,  logctail = double(log(c) - logc);
    ln2 = Ln2hi + Ln2lo, Ln2hi rounded to a multiple of 2^-42, so that
    k*Ln2hi + logc is exact for every exponent k of a double;
    log1p(r) - r + r^2/2 ~ r^3 .. r^8 terms, fitted for least relative error
    on |r| <= 0x1.6bp-8;
  exponential, N = 128 table points:
    2^(j/N) ~ H_j (1 + T_j), H_j = 2^(j/N) rounded to double,
    T_j = double(2^(j/N)/H_j - 1); the table holds the bits of T_j and the bits
    of H_j minus j << 45 (so adding (k << 45) for k = N q + j scales by 2^q);
    x = k ln2/N + r, k = round(x N/ln2) (the 1.5*2^52 shifter), ln2/N split as
    Ln2hiN (a multiple of 2^-43, so k*Ln2hiN is exact for |x| < 512) + Ln2loN;
    exp(r) - 1 - r ~ C2 r^2 + C3 r^3 + C4 r^4 + C5 r^5, fitted for least
    absolute error on |r| <= ln2/(2N).

Polynomial coefficients: a minimax fit in which the coefficients are fixed
one at a time, lowest degree first -- each is rounded to double and the
higher-degree ones are fitted again around it, so they absorb the rounding
of the ones below.  Each fit is a discrete minimax over a Chebyshev grid,
solved as a linear program (scipy's HiGHS) with the residuals refined in
200-bit arithmetic (mpmath).

Run: python csrc/gen_libm_pow_tables.py > csrc/libm_pow_tables.h
"""
import struct

import mpmath as mp
import numpy as np
from scipy.optimize import linprog

mp.mp.prec = 200
N = 128
LOG_OFF = 0x3FE6955500000000  # bits of 0x1.69555p-1
LOG_FIT = mp.mpf(float.fromhex("0x1.6bp-8"))


def d2b(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def b2d(b: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", b & 0xFFFFFFFFFFFFFFFF))[0]


def to_double(x) -> float:
    """Nearest double of an mpmath number (round to nearest even)."""
    return float(mp.mpf(x))


def round_to_multiple(x, q):
    return mp.nint(x / q) * q


def minimax(f, w, ks, a, grid=4000, rounds=4):
    """Coefficients c_k (k in ks) minimising max |w(x) (f(x) - sum c_k x^k)|
    over a Chebyshev grid of [-a, a], and that maximum."""
    xs = [a * mp.cos(mp.pi * (j + mp.mpf(0.5)) / grid) for j in range(grid)]
    wx = [w(x) for x in xs]
    c = [mp.mpf(0)] * len(ks)
    basis = np.array([[float(wj * (x / a) ** k) for k in ks] for x, wj in zip(xs, wx)])

    def resid():
        return [wj * (f(x) - mp.fsum(ci * x**k for ci, k in zip(c, ks))) for x, wj in zip(xs, wx)]

    n = len(ks)
    for _ in range(rounds):  # each round solves for the correction of the previous one
        r = resid()
        s = max(abs(v) for v in r)
        rv = np.array([float(v / s) for v in r])
        P = basis / float(s)
        cmax = np.abs(P).max(axis=0)
        P = P / cmax
        A = np.vstack([np.hstack([-P, -np.ones((grid, 1))]), np.hstack([P, -np.ones((grid, 1))])])
        b = np.concatenate([-rv, rv])
        res = linprog(np.r_[np.zeros(n), 1.0], A_ub=A, b_ub=b, bounds=[(None, None)] * n + [(0, None)],
                      method="highs", options={"primal_feasibility_tolerance": 1e-10,
                                               "dual_feasibility_tolerance": 1e-10})
        if res.status != 0:
            raise RuntimeError(res.message)
        d = res.x[:n] / cmax
        c = [ci + mp.mpf(float(di)) / a**k for ci, di, k in zip(c, d, ks)]
    return c, max(abs(v) for v in resid())


def fit_rounded(f, w, ks, a):
    """The degree-by-degree rounded fit described in the module docstring."""
    fixed = {}
    err = None
    for i, k in enumerate(ks):
        def rest(x, fx=dict(fixed)):
            return f(x) - mp.fsum(c * x**kk for kk, c in fx.items())

        c, err = minimax(rest, w, ks[i:], a)
        fixed[k] = mp.mpf(to_double(c[0]))
    return [fixed[k] for k in ks], err


def main():
    out = ["// Generated by csrc/gen_libm_pow_tables.py -- do not edit.", "#pragma once", ""]
    ln2 = mp.log(2)

    # ---- logarithm table ----
    rows = []
    for i in range(N):
        mid = mp.mpf(b2d(LOG_OFF + (i << 45) + (1 << 44)))
        if mid < 1:
            invc = mp.nint(N / mid) / N
        else:
            invc = mp.nint(2 * N / mid) / (2 * N)
        logc_exact = -mp.log(invc)
        logc = round_to_multiple(logc_exact, mp.mpf(2) ** -43)
        rows.append((to_double(invc), to_double(logc), to_double(logc_exact - logc)))
    ln2hi = round_to_multiple(ln2, mp.mpf(2) ** -42)
    out.append(f"#define LPOW_LN2HI {to_double(ln2hi).hex()}")
    out.append(f"#define LPOW_LN2LO {to_double(ln2 - ln2hi).hex()}")
    out.append(f"#define LPOW_LOG_OFF 0x{LOG_OFF:016x}ull")

    cl, el = fit_rounded(lambda x: mp.log1p(x) - x + x * x / 2, lambda x: 1 / abs(mp.log1p(x)),
                         list(range(3, 9)), LOG_FIT)
    scale = [-2, -2, 4, 4, -8, -8]
    out.append(f"// log1p(r) - r + r^2/2 on |r| <= {to_double(LOG_FIT).hex()}: relative error {float(el):.3e}")
    out.append("// (coefficients of r^3..r^8, scaled by -2, -2, 4, 4, -8, -8 for the evaluation order)")
    for j, (cj, s) in enumerate(zip(cl, scale)):
        out.append(f"#define LPOW_A{j + 1} {to_double(cj * s).hex()}")
    out.append("")

    # ---- exponential ----
    ln2n = ln2 / N
    hiN = round_to_multiple(ln2n, mp.mpf(2) ** -43)
    out.append(f"#define LPOW_INVLN2N {to_double(N / ln2).hex()}")
    out.append(f"#define LPOW_NEGLN2HIN {to_double(-hiN).hex()}")
    out.append(f"#define LPOW_NEGLN2LON {to_double(-(ln2n - hiN)).hex()}")
    ce, ee = fit_rounded(lambda x: mp.exp(x) - 1 - x, lambda x: mp.mpf(1), [2, 3, 4, 5], ln2 / (2 * N))
    out.append(f"// exp(r) - 1 - r on |r| <= ln2/256: absolute error {float(ee):.3e}")
    for j, cj in enumerate(ce):
        out.append(f"#define LPOW_C{j + 2} {to_double(cj).hex()}")
    out.append("")

    out.append("// {1/c, log(c) rounded to 2^-43, log(c) - that}")
    out.append("LPOW_TABLE(lpow_log_tab, 3 * 128) = {")
    for invc, logc, tail in rows:
        out.append(f"    {invc.hex()}, {logc.hex()}, {tail.hex()},")
    out.append("};")
    out.append("")
    out.append("// {bits of T_j, bits of H_j - (j << 45)}: 2^(j/128) ~ H_j (1 + T_j)")
    out.append("LPOW_UTABLE(lpow_exp_tab, 2 * 128) = {")
    for j in range(N):
        v = mp.power(2, mp.mpf(j) / N)
        H = to_double(v)
        T = to_double(v / mp.mpf(H) - 1)
        sb = (d2b(H) - (j << 45)) & 0xFFFFFFFFFFFFFFFF
        out.append(f"    0x{d2b(T):016x}ull, 0x{sb:016x}ull,")
    out.append("};")
    print("\n".join(out))


if __name__ == "__main__":
    main()
