"""Every compiled configuration of the unsplit step kernel (tile shape, threads,
occupancy; gathered or TMA-staged persistent) gives the same answer.

The autotuner may pick any of them, so each is checked on grids with partial
edge tiles and on every boundary kind: the FP64 form against the oracle, the
FP32 forms against the FP64 form and against each other.
"""
import numpy as np
import pytest

from helpers import FIELDS, rel_l1

CASES = [
    # m, n, bx, by, seed
    (70, 45, -4, -4, 3),
    (45, 70, -7, -2, 5),
    (33, 96, -24, -1, 8),
    # strips and row units with interior ones on both axes (the strip kernel's fast path)
    (150, 200, -4, -7, 9),
    # a grid smaller than one tile and one strip unit
    (3, 5, -4, -4, 12),
    # one full strip and a strip of four columns, rows not a multiple of a unit
    (61, 64, -2, -7, 13),
]
STEPS = 12


def _cfg(hg, m, n, bx, by):
    return hg.config_2d(t_all=-1, steps=STEPS, hx=1.0 / m, hy=1.0 / n, bx=bx, by=by)


def _all_variants(hg, form, rho, u, v, p, cfg):
    s = hg.Solver2D(*rho.shape, form)
    out = []
    try:
        if form == hg.FORM_FP32_LEARNED:
            s.set_mlp(hg.load_weights())
        for k in range(s.num_variants()):
            s.set_variant(k)
            s.upload(rho, u, v, p)
            info = s.run(cfg)
            assert info.halted == 0
            out.append((s.variant()[1], s.download()))
    finally:
        s.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("m,n,bx,by,seed", CASES)
def test_fp64_variants_match_oracle(gpu_lib, port, m, n, bx, by, seed):
    hg = gpu_lib
    from hydro_gb300 import cases

    rho, u, v, p = cases.four_quadrant(m, n, seed)
    cfg = _cfg(hg, m, n, bx, by)
    want = port.run_2d(rho, u, v, p, cfg)
    runs = _all_variants(hg, hg.FORM_FP64, rho, u, v, p, cfg)
    for shape, got in runs:
        for f in FIELDS + ("E",):
            assert rel_l1(got[f], want[f]) <= 1e-12, (shape, f, rel_l1(got[f], want[f]))
    # every FP64 variant computes each face, slope and cell with the same code
    # from the same inputs: the same bits, whatever the tiling or the march
    for shape, got in runs[1:]:
        for f in FIELDS + ("E",):
            assert np.array_equal(got[f], runs[0][1][f]), (shape, f)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp32", "fp32_learned"])
@pytest.mark.parametrize("m,n,bx,by,seed", CASES)
def test_fp32_variants_agree(gpu_lib, m, n, bx, by, seed, form):
    hg = gpu_lib
    from hydro_gb300 import cases

    rho, u, v, p = cases.four_quadrant(m, n, seed)
    cfg = _cfg(hg, m, n, bx, by)
    ref, _ = hg.run_2d(rho, u, v, p, cfg, form=hg.FORM_FP64)
    code = hg.FORM_FP32 if form == "fp32" else hg.FORM_FP32_LEARNED
    outs = _all_variants(hg, code, rho, u, v, p, cfg)
    base = outs[0][1]
    for shape, got in outs:
        for f in FIELDS:
            assert rel_l1(got[f], ref[f]) <= 2e-5, (shape, f, rel_l1(got[f], ref[f]))
            assert rel_l1(got[f], base[f]) <= 1e-6, (shape, f, rel_l1(got[f], base[f]))


@pytest.mark.gpu
def test_tma_variants_present(gpu_lib):
    """The persistent TMA-staged kernels are among the autotuner's choices."""
    hg = gpu_lib
    for form in (hg.FORM_FP64, hg.FORM_FP32, hg.FORM_FP32_LEARNED):
        s = hg.Solver2D(64, 64, form)
        try:
            kinds = []
            for k in range(s.num_variants()):
                s.set_variant(k)
                kinds.append(s.variant()[1]["tma"])
            assert any(kinds) and not all(kinds), kinds
        finally:
            s.close()
