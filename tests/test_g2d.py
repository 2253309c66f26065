"""The genuinely-2D GRP interface solver (config[301] = 1, HYDRO_SOLVER_G2D):
the GPU's FP64 form against the reference's own runs with that solver
(tests/golden/runs_2d_g2d.npz) and against the oracle, every compiled
variant, the FP32 form against FP64, and the drop-in scheme entry points."""
import os

import numpy as np
import pytest

from helpers import FIELDS, rel_l1

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12   # FP64 form vs the reference (relative L1)
FP32_TOL = 2e-5


def _golden_runs():
    d = np.load(os.path.join(GOLD, "runs_2d_g2d.npz"))
    names = sorted({k.split("/")[0] for k in d.files})
    return d, names


@pytest.mark.gpu
def test_g2d_fp64_matches_reference_runs(gpu_lib):
    hg = gpu_lib
    d, names = _golden_runs()
    assert len(names) >= 5
    for name in names:
        cfg = d[f"{name}/cfg"].copy()
        split = int(d[f"{name}/meta"][2])
        out, info = hg.run_2d(d[f"{name}/in_rho"], d[f"{name}/in_u"], d[f"{name}/in_v"], d[f"{name}/in_p"], cfg,
                              split=bool(split), form=hg.FORM_FP64, solver=hg.SOLVER_G2D)
        assert info.k_out == d[f"{name}/meta"][0] and info.time == d[f"{name}/meta"][1], name
        for f in FIELDS + ("E",):
            assert rel_l1(out[f], d[f"{name}/{f}"]) <= TOL, (name, f, rel_l1(out[f], d[f"{name}/{f}"]))


CASES = [
    # m, n, bx, by, seed, split
    (70, 45, -4, -4, 3, 0),
    (45, 70, -7, -2, 5, 0),
    (33, 50, -24, -1, 8, 0),
    (40, 36, -7, -7, 6, 1),
]


def _cfg(hg, m, n, bx, by, split, steps=12):
    c = hg.config_2d(t_all=-1, steps=steps, hx=1.0 / m, hy=1.0 / n, bx=bx, by=by, split=split)
    c[301] = hg.SOLVER_G2D
    return c


@pytest.mark.gpu
@pytest.mark.parametrize("m,n,bx,by,seed,split", CASES)
def test_g2d_fp64_variants_match_oracle(gpu_lib, port, m, n, bx, by, seed, split):
    hg = gpu_lib
    from hydro_gb300 import cases

    rho, u, v, p = cases.four_quadrant(m, n, seed)
    cfg = _cfg(hg, m, n, bx, by, split)
    want = port.run_2d(rho, u, v, p, cfg, split=split)
    q1d = cfg.copy()
    q1d[301] = np.inf
    other = port.run_2d(rho, u, v, p, q1d, split=split)
    s = hg.Solver2D(m, n, hg.FORM_FP64, hg.SOLVER_G2D)
    try:
        for k in range(s.num_variants()):
            s.set_variant(k)
            s.upload(rho, u, v, p)
            info = s.run(cfg, split=bool(split))
            assert info.halted == 0
            got = s.download()
            for f in FIELDS + ("E",):
                assert rel_l1(got[f], want[f]) <= TOL, (k, f, rel_l1(got[f], want[f]))
    finally:
        s.close()
    if not split:  # the solvers differ once tangential derivatives enter
        assert rel_l1(want["rho"], other["rho"]) > 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("m,n,bx,by,seed,split", CASES)
def test_g2d_fp32_against_fp64(gpu_lib, m, n, bx, by, seed, split):
    hg = gpu_lib
    from hydro_gb300 import cases

    rho, u, v, p = cases.four_quadrant(m, n, seed)
    cfg = _cfg(hg, m, n, bx, by, split)
    ref, _ = hg.run_2d(rho, u, v, p, cfg, split=bool(split), form=hg.FORM_FP64, solver=hg.SOLVER_G2D)
    s = hg.Solver2D(m, n, hg.FORM_FP32, hg.SOLVER_G2D)
    try:
        base = None
        for k in range(s.num_variants()):
            s.set_variant(k)
            s.upload(rho, u, v, p)
            assert s.run(cfg, split=bool(split)).halted == 0
            got = s.download()
            base = got if base is None else base
            for f in FIELDS:
                assert rel_l1(got[f], ref[f]) <= FP32_TOL, (k, f, rel_l1(got[f], ref[f]))
                assert rel_l1(got[f], base[f]) <= 1e-6, (k, f)
    finally:
        s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("split", [0, 1])
def test_g2d_dropin_entry(gpu_lib, port, split):
    """config[301] = 1 through GRP_solver_2D_EUL_source / _split_EUL_source."""
    hg = gpu_lib
    from hydro_gb300 import cases
    from hydro_gb300.dropin import call_2d

    m, n = 23, 19
    rho, u, v, p = cases.four_quadrant(m, n, 4)
    cfg = hg.config_2d(t_all=0.04, steps=1000, hx=1 / m, hy=1 / n, bx=-4, by=-2, split=split)
    cfg[301] = 1
    data, nplot, time_plot, k_out = call_2d(hg.lib(), rho, u, v, p, 1.4, cfg.copy(), split=split)
    want = port.run_2d(rho, u, v, p, cfg, split=split)
    assert k_out == want["steps"] and time_plot[nplot - 1] == want["time"]
    for f, key in enumerate(("rho", "u", "v", "p", "E")):
        assert rel_l1(data[nplot - 1, f], want[key]) <= TOL


@pytest.mark.gpu
def test_g2d_unsupported_combinations_fail_loudly(gpu_lib):
    hg = gpu_lib
    with pytest.raises(RuntimeError, match="quasi-1D"):
        hg.Solver2D(32, 32, hg.FORM_FP32_LEARNED, hg.SOLVER_G2D)
    with pytest.raises(RuntimeError, match="interface solver"):
        hg.Solver2D(32, 32, hg.FORM_FP64, 7)
    b = hg.Batch([(32, 32)])
    try:
        from hydro_gb300 import cases

        b.upload(0, *cases.four_quadrant(32, 32, 1))
        cfg = hg.config_2d(t_all=-1, steps=2, bx=-4, by=-4)
        cfg[301] = 1
        with pytest.raises(RuntimeError, match="quasi-1D"):
            b.run(cfg, 2)
    finally:
        b.close()
