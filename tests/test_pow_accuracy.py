"""The FP64 form's pow (double-double, csrc/hydro_pow.cuh) against the C
library's pow -- the one the reference calls -- on the arguments the solver
produces (pressure/sound-speed ratios; the exponents of the exact Riemann
solver and the GRP for several gammas) and on arbitrary ones.  They agree on
all but a small fraction, and wherever they disagree the double-double result
is the correctly rounded one (checked with 60-digit decimal arithmetic): the
residue is the C library's own last-bit rounding.  Host build of the same code."""
import ctypes
import os
import subprocess
import tempfile
from decimal import Decimal, getcontext

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _lib():
    d = tempfile.mkdtemp()
    so = os.path.join(d, "pow_check.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "native", "pow_check.cpp"), "-lm"], check=True)
    L = ctypes.CDLL(so)
    dp = np.ctypeslib.ndpointer(np.float64, flags="C")
    L.pow_pair.argtypes = [dp, dp, ctypes.c_longlong, dp, dp]
    L.pow_pair.restype = None
    return L


def _check(L, x, y):
    n = len(x)
    a, b = np.zeros(n), np.zeros(n)
    L.pow_pair(np.ascontiguousarray(x), np.ascontiguousarray(y), n, a, b)
    idx = np.nonzero(a != b)[0]
    assert len(idx) <= n * 1e-3, len(idx)
    getcontext().prec = 60
    for i in idx[:100]:
        t = Decimal(float(x[i])) ** Decimal(float(y[i]))
        assert abs(Decimal(float(a[i])) - t) <= abs(Decimal(float(b[i])) - t), (x[i], y[i])
    return len(idx)


def test_dd_pow_matches_libm():
    L = _lib()
    rng = np.random.default_rng(0)
    n = 1_000_000
    exps = []
    for g in (1.4, 5.0 / 3.0, 1.2, 3.0):
        zeta = (g - 1.0) / (g + 1.0)
        exps += [(g - 1.0) / (2.0 * g), (g + 1.0) / (2.0 * g), 1.0 / g, 0.5 * (g - 1.0) / g,
                 2.0 * g / (g - 1.0), 0.5 / zeta, (1.0 + zeta) / zeta, g / (g - 1.0), 3.0]
    y = np.array(exps)[rng.integers(0, len(exps), n)]
    x = np.exp(rng.uniform(np.log(1e-6), np.log(1e6), n))
    x[: n // 4] = 1.0 + rng.normal(0, 1e-6, n // 4)  # ratios near 1 (Newton near convergence)
    _check(L, x, y)
    _check(L, np.exp(rng.uniform(-5, 5, n)), rng.uniform(-8, 8, n))


def test_dd_cube_is_correctly_rounded():
    """pow(t, 3.0) takes the double-double cube: on random arguments across the
    range it returns the correctly rounded cube (exact in 60-digit decimal
    arithmetic), and it agrees with the C library wherever that one is
    correctly rounded."""
    L = _lib()
    rng = np.random.default_rng(3)
    n = 200_000
    x = np.concatenate([rng.uniform(0, 1, n // 2), np.exp(rng.uniform(-300, 300, n // 2) * np.log(2.0) / 1.2)])
    y = np.full(n, 3.0)
    a, b = np.zeros(n), np.zeros(n)
    L.pow_pair(x, y, n, a, b)
    getcontext().prec = 60
    for i in rng.choice(n, 3000, replace=False):
        assert a[i] == float(Decimal(float(x[i])) ** 3), x[i]
    for i in np.nonzero(a != b)[0][:200]:
        t = Decimal(float(x[i])) ** 3
        assert abs(Decimal(float(a[i])) - t) <= abs(Decimal(float(b[i])) - t), x[i]
    assert (a != b).mean() < 1e-3
