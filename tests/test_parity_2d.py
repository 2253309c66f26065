"""GPU parity of the 2D FP64 form against the oracle (C restatement, itself
pinned bit-for-bit to the reference).  Bar: relative L1 <= 1e-12 in rho, u, v, p
after the final step (the only inexact operation on the device is pow(), which
differs from glibc's by at most a couple of ulp), plus identical step count,
final time and halting behaviour."""
import numpy as np
import pytest

from helpers import compare_states
from hydro_gb300 import cases

TOL = 1e-12

CASES = [
    # (name, m, n, generator, bx, by, steps, split)
    ("fq_free_17x13", 17, 13, "fq", -4, -4, 40, 0),
    ("fq_free_64x48", 64, 48, "fq", -4, -4, 80, 0),
    ("shear_periodic_32", 32, 32, "sh", -7, -7, 60, 0),
    ("fq_reflect_mixed", 20, 24, "fq", -2, -24, 50, 0),
    ("fq_fixed_initial", 19, 15, "fq", -1, -1, 40, 0),
    ("fq_periodic_x_reflect_y", 24, 20, "fq", -7, -2, 40, 0),
    ("fq_split_free", 17, 13, "fq", -4, -4, 30, 1),
    ("shear_split_periodic", 32, 24, "sh", -7, -7, 30, 1),
    ("fq_split_mixed", 21, 18, "fq", -24, -1, 30, 1),
    ("tiny_2x2", 2, 2, "fq", -4, -4, 10, 0),
    ("odd_33x17", 33, 17, "fq", -4, -7, 40, 0),
]


def _gen(kind, m, n, seed):
    return cases.four_quadrant(m, n, seed) if kind == "fq" else cases.shear_layer(m, n, seed)


@pytest.mark.gpu
@pytest.mark.parametrize("name,m,n,kind,bx,by,steps,split", CASES, ids=[c[0] for c in CASES])
def test_fp64_matches_oracle(gpu_lib, port, name, m, n, kind, bx, by, steps, split):
    hg = gpu_lib
    rho, u, v, p = _gen(kind, m, n, seed=7)
    cfg = hg.config_2d(t_all=-1, steps=steps, hx=1.0 / m, hy=1.0 / n, bx=bx, by=by, split=split)
    want = port.run_2d(rho, u, v, p, cfg, split=split)
    got, info = hg.run_2d(rho, u, v, p, cfg, split=split)
    d = compare_states(got, want, ("rho", "u", "v", "p", "E"))
    assert info.k_out == int(want["steps"]), (info.as_dict(), want["steps"])
    assert info.time == want["time"]
    assert max(d.values()) <= TOL, d


@pytest.mark.gpu
def test_fp64_time_limited_run(gpu_lib, port):
    """t_all given: the last step is clipped to land on t_all exactly."""
    hg = gpu_lib
    m, n = 40, 32
    rho, u, v, p = cases.four_quadrant(m, n, 11)
    cfg = hg.config_2d(t_all=0.05, steps=100000, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4)
    want = port.run_2d(rho, u, v, p, cfg)
    got, info = hg.run_2d(rho, u, v, p, cfg)
    assert info.k_out == int(want["steps"])
    assert info.time == want["time"] == 0.05
    assert max(compare_states(got, want).values()) <= TOL


@pytest.mark.gpu
def test_fp64_bitwise_deterministic(gpu_lib):
    """Two runs on the same input are bitwise equal (no float atomics in results)."""
    hg = gpu_lib
    rho, u, v, p = cases.shear_layer(48, 40, 3)
    cfg = hg.config_2d(t_all=-1, steps=30, hx=1 / 48, hy=1 / 40, bx=-7, by=-7)
    a, _ = hg.run_2d(rho, u, v, p, cfg)
    b, _ = hg.run_2d(rho, u, v, p, cfg)
    for f in ("rho", "u", "v", "p", "E"):
        assert np.array_equal(a[f], b[f])
