"""The headline parity case: 2D unsplit GRP, FP64, 1024 x 1024 seeded
four-quadrant Riemann data, transmissive boundaries, CFL 0.45, 500 steps.
Bar: relative L1 <= 1e-12 in rho, u, v, p after the final step.

* against the reference's own run (tests/golden/fq1024_500.npz: a strided
  subsample, one row, one column and the field sums, produced by
  tests/golden/make_golden.py from the reference's unmodified sources);
* against the oracle on the full field (the C restatement, OpenMP on the
  host cores: slow, about a minute)."""
import os

import numpy as np
import pytest

from helpers import rel_l1

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


def _gpu_run(hg):
    from hydro_gb300 import cases

    m = n = 1024
    rho, u, v, p = cases.four_quadrant(m, n, seed=2024)
    cfg = hg.config_2d(t_all=-1, steps=500, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4)
    got, info = hg.run_2d(rho, u, v, p, cfg, stats=True)
    return (rho, u, v, p), cfg, got, info


@pytest.mark.gpu
def test_config2_against_reference_golden(gpu_lib):
    d = np.load(os.path.join(GOLD, "fq1024_500.npz"))
    _, _, got, info = _gpu_run(gpu_lib)
    assert info.k_out == int(d["meta"][0]) and info.time == d["meta"][1]
    m = 1024
    for f in ("rho", "u", "v", "p", "E"):
        assert rel_l1(got[f][::16, ::16], d[f"sub/{f}"]) <= TOL, f
        assert rel_l1(got[f][m // 2 + 3, :], d[f"row/{f}"]) <= TOL, f
        assert rel_l1(got[f][:, m // 2 - 5], d[f"col/{f}"]) <= TOL, f
        assert abs(np.abs(got[f]).sum() - d[f"abs_sum/{f}"]) <= TOL * d[f"abs_sum/{f}"], f
    assert info.newton_faces > 0


@pytest.mark.gpu
def test_config2_full_field_against_oracle(gpu_lib, port):
    (rho, u, v, p), cfg, got, info = _gpu_run(gpu_lib)
    want = port.run_2d(rho, u, v, p, cfg)
    assert info.k_out == int(want["steps"]) and info.time == want["time"]
    for f in ("rho", "u", "v", "p"):
        assert rel_l1(got[f], want[f]) <= TOL, f
