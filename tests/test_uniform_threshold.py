"""The FP64 form decides the reference's uniform-pair test sqrt(d2) < eps
(linear_grp_solver_Edir_Q1D.c:95-96,139) as d2 <= hydro_uniform_dist2_max(eps),
without the square root.  The threshold is host arithmetic of the library, so
this runs without a GPU: the boundary is exact (the threshold passes, the next
double does not), and random d2 around it and across the range decide alike."""
import ctypes
import math
import os

import numpy as np
import pytest


@pytest.fixture(scope="module")
def dist2_max():
    import hydro_gb300 as hg

    if not os.path.exists(hg.LIB_PATH):
        hg.build()
    L = ctypes.CDLL(hg.LIB_PATH)
    f = L.hydro_uniform_dist2_max
    f.argtypes = [ctypes.c_double]
    f.restype = ctypes.c_double
    return f


EPS = [1e-9, 1e-12, 1e-6, 1e-15, 0.1, 1.0, 3.0, 1e-150, 1e-160, 1e-170, 1e-200, 1e-300, 5e-324, 1e100, 1e154,
       1e155, 1e200, 1.7976931348623157e308]


@pytest.mark.parametrize("eps", EPS)
def test_threshold_is_the_exact_boundary(dist2_max, eps):
    x = dist2_max(eps)
    assert x >= 0.0
    assert math.sqrt(x) < eps
    y = math.nextafter(x, math.inf)
    assert math.isinf(y) or not (math.sqrt(y) < eps)


@pytest.mark.parametrize("eps", [0.0, -0.0, -1e-9, float("nan"), -math.inf])
def test_no_pair_is_uniform_without_a_positive_eps(dist2_max, eps):
    assert dist2_max(eps) == -1.0
    for d2 in (0.0, 1e-300, 1.0):
        assert not (math.sqrt(d2) < eps)


@pytest.mark.parametrize("eps", [1e-9, 1e-12, 1e-200, 1e200])
def test_random_d2_decide_alike(dist2_max, eps):
    x = dist2_max(eps)
    rng = np.random.default_rng(7)
    # around the boundary, in units in the last place, and across the range
    near = [x]
    for _ in range(64):
        near = [math.nextafter(near[0], 0.0)] + near + [math.nextafter(near[-1], math.inf)]
    wide = list(x * np.exp(rng.uniform(-40.0, 40.0, 20000)))
    for d2 in near + wide + [0.0, math.inf, float("nan")]:
        assert (math.sqrt(d2) < eps) == (d2 <= x), d2
