"""The FP64 form's pow functions against the C library's pow -- the one the
reference calls -- on the arguments the solver produces (pressure/sound-speed
ratios; the exponents of the exact Riemann solver and the GRP for several
gammas) and on arbitrary ones.  Host builds of the device code.

* libm_pow.cuh (the device default) follows the C library's own method and
  returns the C library's bits: no argument of the solver sample differs, and
  at most a handful in tens of millions of arbitrary ones.
* hydro_pow.cuh (correctly rounded double-double pow, kept for comparison)
  differs from the C library on ~0.06% of the arguments, and wherever they
  differ it is the correctly rounded one (60-digit decimal arithmetic): the
  residue is the C library's own last-bit rounding."""
import ctypes
import os
import subprocess
import tempfile
from decimal import Decimal, getcontext

import numpy as np
import pytest

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
    L.lpow_pair.argtypes = [dp, dp, ctypes.c_longlong, dp, dp]
    L.lpow_pair.restype = None
    L.lpow_shared_log_mismatch.argtypes = [dp, ctypes.c_longlong, ctypes.c_double, ctypes.c_double]
    L.lpow_shared_log_mismatch.restype = ctypes.c_longlong
    return L


def _solver_args(rng, n):
    exps = []
    for g in (1.4, 5.0 / 3.0, 1.2, 3.0):
        zeta = (g - 1.0) / (g + 1.0)
        exps += [(g - 1.0) / (2.0 * g), (g + 1.0) / (2.0 * g), 1.0 / g, 0.5 * (g - 1.0) / g,
                 2.0 * g / (g - 1.0), 0.5 / zeta, (1.0 + zeta) / zeta, g / (g - 1.0), 3.0]
    y = np.array(exps)[rng.integers(0, len(exps), n)]
    x = np.exp(rng.uniform(np.log(1e-6), np.log(1e6), n))
    x[: n // 4] = 1.0 + rng.normal(0, 1e-6, n // 4)  # ratios near 1 (Newton near convergence)
    x[n // 4: n // 2] = 1.0 + rng.normal(0, 5e-3, n // 4)
    return x, y


def _libm_is_the_fma_variant():
    """The C library's pow computes with fused multiply-adds on AArch64 and on
    x86-64 processors with FMA (the case the reference's fixtures were made
    in); elsewhere it takes another variant of the method."""
    import platform
    if platform.machine() in ("aarch64", "arm64"):
        return True
    try:
        with open("/proc/cpuinfo") as f:
            flags = next((ln for ln in f if ln.startswith("flags")), "").split()
        return "fma" in flags and "avx2" in flags
    except OSError:
        return False


def test_libm_method_pow_returns_the_c_library_bits():
    if not _libm_is_the_fma_variant():
        pytest.skip("this host's C library pow takes its variant without fused multiply-add")
    L = _lib()
    rng = np.random.default_rng(11)
    n = 2_000_000
    x, y = _solver_args(rng, n)
    a, b = np.zeros(n), np.zeros(n)
    L.lpow_pair(x, y, n, a, b)
    assert np.array_equal(a, b), int((a != b).sum())
    x, y = np.exp(rng.uniform(-5, 5, n)), rng.uniform(-8, 8, n)
    L.lpow_pair(x, y, n, a, b)
    assert (a != b).sum() <= 2, int((a != b).sum())
    # the solver's whole range of pressure ratios, and subnormal, tiny and huge bases
    x = np.concatenate([np.exp(rng.uniform(-700, 700, n // 2)), np.ldexp(rng.uniform(0.5, 1, 1000), -1060)])
    y = np.concatenate([rng.uniform(-0.7, 0.7, n // 2), np.full(1000, 0.2)])
    a, b = np.zeros(len(x)), np.zeros(len(x))
    L.lpow_pair(x, y, len(x), a, b)
    assert (a != b).sum() <= 2, int((a != b).sum())


def test_libm_method_pow_shares_one_logarithm():
    """x^mu and x^nu from one logarithm equal two separate calls bit for bit."""
    L = _lib()
    rng = np.random.default_rng(12)
    x = np.exp(rng.uniform(-10, 10, 500_000))
    for g in (1.4, 5.0 / 3.0):
        assert L.lpow_shared_log_mismatch(x, len(x), (g - 1) / (2 * g), (g + 1) / (2 * g)) == 0


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
