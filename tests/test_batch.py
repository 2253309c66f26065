"""Batched problems of uneven size (hydro_batch_* / hydro_gb300_batch_run).

Every problem of a batch must come out exactly as a one-problem FP32 run of
the same grid (the batch runs the same per-tile code), whatever the tile shape
or schedule, and within the FP32 form's tolerance of the FP64 oracle.
"""
import ctypes

import numpy as np
import pytest

from helpers import FIELDS, rel_l1

SIZES = [(17, 13), (40, 33), (64, 64), (20, 70), (96, 32), (33, 47), (5, 9)]
STEPS = 20
FP32_TOL = 2e-5  # relative L1 of the FP32 form against the FP64 oracle on these cases


def _cfg(hg, bx=-4, by=-4):
    return hg.config_2d(t_all=-1, steps=STEPS, bx=bx, by=by)


def _problems(hg):
    from hydro_gb300 import cases

    return cases.batch_problems(SIZES, seed=11)


def _run_batch(hg, probs, cfg, shape, schedule, steps=STEPS):
    b = hg.Batch(SIZES)
    try:
        for k, (rho, u, v, p) in enumerate(probs):
            b.upload(k, rho, u, v, p, gamma=float(cfg[6]))
        b.set_schedule(shape, schedule)
        info = b.run(cfg, steps)
        return [b.download(k) for k in range(len(SIZES))], info, [b.problem_info(k) for k in range(len(SIZES))]
    finally:
        b.close()


def _one_problem_fp32(hg, prob, m, n, bx=-4, by=-4, steps=STEPS):
    """The one-problem FP32 run with a tile kernel, the code the batch runs per
    tile (the strip kernels arrange the FP32 arithmetic differently), so that
    states compare bit for bit where the test asks for it."""
    cfg = hg.config_2d(t_all=-1, steps=steps, hx=1.0 / m, hy=1.0 / n, bx=bx, by=by)
    s = hg.Solver2D(m, n, hg.FORM_FP32)
    try:
        for k in range(s.num_variants()):
            s.set_variant(k)
            if s.variant()[1]["kernel"] != "strip":
                break
        s.upload(*prob, None, float(cfg[6]))
        info = s.run(cfg)
        return s.download(), info
    finally:
        s.close()


def _one_problem_strip(hg, prob, m, n, rows, bx=-4, by=-4, steps=STEPS):
    """The one-problem FP32 run with the strip kernel of `rows` rows per work
    unit, the per-unit march the batch's strip shapes run."""
    cfg = hg.config_2d(t_all=-1, steps=steps, hx=1.0 / m, hy=1.0 / n, bx=bx, by=by)
    s = hg.Solver2D(m, n, hg.FORM_FP32)
    try:
        for k in range(s.num_variants()):
            s.set_variant(k)
            v = s.variant()[1]
            if v["kernel"] == "strip" and v["tile_x"] == rows:
                break
        else:
            raise AssertionError(f"no strip variant with {rows} rows per unit")
        s.upload(*prob, None, float(cfg[6]))
        info = s.run(cfg)
        return s.download(), info
    finally:
        s.close()


def _strip_shapes(hg):
    return [(k, sh["tile_y"]) for k, sh in enumerate(hg.Batch.shapes()) if sh["kind"] == "strip"]


@pytest.mark.gpu
def test_batch_matches_one_problem_runs(gpu_lib):
    hg = gpu_lib
    probs = _problems(hg)
    cfg = _cfg(hg)
    got, info, pinfo = _run_batch(hg, probs, cfg, shape=0, schedule=0)
    assert info.steps == STEPS and info.halted_problems == 0
    for k, (m, n) in enumerate(SIZES):
        want, winfo = _one_problem_fp32(hg, probs[k], m, n)
        assert pinfo[k]["tau"] == winfo.tau
        for f in FIELDS + ("E",):
            assert rel_l1(got[k][f], want[f]) <= 1e-6, (k, f, rel_l1(got[k][f], want[f]))


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", [0, 3, 4])
def test_batch_strip_shapes_match_one_problem_strip_runs(gpu_lib, schedule):
    """The strip shapes run the one-grid strip kernel's per-unit march on each
    problem: every problem equals its one-problem strip run (same rows per
    unit) to FP32 rounding, and its time step bit for bit."""
    hg = gpu_lib
    probs = _problems(hg)
    cfg = _cfg(hg, bx=-7, by=-2)
    strips = _strip_shapes(hg)
    assert strips
    for sh, rows in strips:
        got, info, pinfo = _run_batch(hg, probs, cfg, sh, schedule)
        assert info.steps == STEPS and info.halted_problems == 0 and info.shape == sh
        for k, (m, n) in enumerate(SIZES):
            want, winfo = _one_problem_strip(hg, probs[k], m, n, rows, bx=-7, by=-2)
            assert pinfo[k]["tau"] == winfo.tau
            for f in FIELDS + ("E",):
                assert rel_l1(got[k][f], want[f]) <= 1e-6, (sh, k, f, rel_l1(got[k][f], want[f]))


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", [2, 4])
def test_batch_strip_halts_per_problem(gpu_lib, schedule):
    """A problem whose state goes bad halts alone in a strip shape too, at the
    step and with the state of its one-problem strip run (the step it halted
    on is the tile shapes' too)."""
    hg = gpu_lib
    probs = [list(a) for a in _problems(hg)]
    bad = 2
    probs[bad][3] = probs[bad][3].copy()
    probs[bad][3][10, 10] = -1.0
    cfg = _cfg(hg)
    sh, rows = _strip_shapes(hg)[0]
    got, info, pinfo = _run_batch(hg, probs, cfg, shape=sh, schedule=schedule)
    _, _, tinfo = _run_batch(hg, probs, cfg, shape=0, schedule=2)
    assert pinfo[bad]["halted"] != 0
    assert pinfo[bad]["halted"] == tinfo[bad]["halted"]
    assert pinfo[bad]["halted_step"] == tinfo[bad]["halted_step"]
    for k, (m, n) in enumerate(SIZES):
        if k != bad:
            assert pinfo[k]["halted"] == 0
    want, winfo = _one_problem_strip(hg, probs[bad], *SIZES[bad], rows)
    assert winfo.halted == pinfo[bad]["halted"]
    for f in FIELDS:
        ok = ~np.isnan(want[f])
        assert np.array_equal(np.isnan(got[bad][f]), ~ok), f
        assert rel_l1(got[bad][f][ok], want[f][ok]) <= 1e-6, f


@pytest.mark.gpu
def test_batch_against_fp64_oracle(gpu_lib, port):
    hg = gpu_lib
    probs = _problems(hg)
    cfg = _cfg(hg)
    got, _, _ = _run_batch(hg, probs, cfg, shape=1, schedule=2)
    for k, (m, n) in enumerate(SIZES):
        c = hg.config_2d(t_all=-1, steps=STEPS, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4)
        want = port.run_2d(*probs[k], c)
        for f in FIELDS:
            assert rel_l1(got[k][f], want[f]) <= FP32_TOL, (k, f, rel_l1(got[k][f], want[f]))


@pytest.mark.gpu
@pytest.mark.parametrize("bx,by", [(-2, -7), (-24, -1), (-7, -2), (-1, -24)])
def test_batch_boundaries_against_fp64_oracle(gpu_lib, port, bx, by):
    """Every boundary kind the scheme reads (reflective -2, periodic -7, the
    half-reflective -24, the fixed initial values -1), on the shape and
    schedule the autotuner picks on the bench's batch (16x16 tiles, one launch
    per step): each problem within the FP32 form's tolerance of the FP64
    oracle run of its own grid."""
    hg = gpu_lib
    probs = _problems(hg)
    cfg = _cfg(hg, bx, by)
    got, info, _ = _run_batch(hg, probs, cfg, shape=2, schedule=4)
    assert info.halted_problems == 0
    for k, (m, n) in enumerate(SIZES):
        c = hg.config_2d(t_all=-1, steps=STEPS, hx=1.0 / m, hy=1.0 / n, bx=bx, by=by)
        want = port.run_2d(*probs[k], c)
        for f in FIELDS:
            assert rel_l1(got[k][f], want[f]) <= FP32_TOL, (k, f, rel_l1(got[k][f], want[f]))


@pytest.mark.gpu
def test_batch_schedules_and_shapes_agree(gpu_lib):
    """Each tile is computed once per step from the previous step's state, in
    any order, so the order cannot change a result: the persistent schedules
    (0-3, one compiled kernel whatever the tile order) agree bit for bit and
    a repeated run reproduces itself bit for bit; the per-step kernel (4) and
    other tile shapes are separately compiled instances of the same code and
    agree to FP32 rounding."""
    hg = gpu_lib
    probs = _problems(hg)
    cfg = _cfg(hg, bx=-7, by=-2)
    nsh = len(hg.Batch.shapes())
    base = None
    for sh in range(nsh):
        first = None
        for sc in range(len(hg.SCHEDULES)):
            got, info, _ = _run_batch(hg, probs, cfg, sh, sc)
            assert info.schedule == sc and info.shape == sh
            again, _, _ = _run_batch(hg, probs, cfg, sh, sc)
            for k in range(len(SIZES)):
                for f in FIELDS:
                    assert np.array_equal(got[k][f], again[k][f]), ("repeat", sh, sc, k, f)
            if first is None:
                first = got
            else:
                for k in range(len(SIZES)):
                    for f in FIELDS:
                        if sc < 4:
                            assert np.array_equal(got[k][f], first[k][f]), (sh, sc, k, f)
                        else:
                            assert rel_l1(got[k][f], first[k][f]) <= 1e-6, (sh, sc, k, f)
        if base is None:
            base = first
        else:
            for k in range(len(SIZES)):
                for f in FIELDS:
                    assert rel_l1(first[k][f], base[k][f]) <= 1e-6, (sh, k, f)


@pytest.mark.gpu
def test_batch_persistent_runs_as_graph(gpu_lib):
    hg = gpu_lib
    probs = _problems(hg)
    _, info, _ = _run_batch(hg, probs, _cfg(hg), shape=0, schedule=0)
    assert info.graphed == 1
    _, info, _ = _run_batch(hg, probs, _cfg(hg), shape=0, schedule=4)
    assert info.graphed == 1


@pytest.mark.gpu
def test_batch_autotune_restores_state(gpu_lib):
    hg = gpu_lib
    probs = _problems(hg)
    cfg = _cfg(hg)
    b = hg.Batch(SIZES)
    try:
        for k, pr in enumerate(probs):
            b.upload(k, *pr)
        best, times = b.autotune(cfg, steps=3)
        assert times.shape == (len(hg.Batch.shapes()), len(hg.SCHEDULES))
        assert np.all(np.isfinite(times)) and np.all(times > 0)
        assert times.flat[best] == times.min()
        info = b.run(cfg, STEPS)
        assert info.shape * len(hg.SCHEDULES) + info.schedule == best
        got = [b.download(k) for k in range(len(SIZES))]
    finally:
        b.close()
    ref, _, _ = _run_batch(hg, probs, cfg, best // len(hg.SCHEDULES), best % len(hg.SCHEDULES))
    for k in range(len(SIZES)):
        for f in FIELDS:
            assert np.array_equal(got[k][f], ref[k][f])


@pytest.mark.gpu
def test_batch_halts_per_problem(gpu_lib):
    """A problem whose state goes bad halts alone; the others run to the end."""
    hg = gpu_lib
    probs = [list(a) for a in _problems(hg)]
    bad = 2
    probs[bad][3] = probs[bad][3].copy()
    probs[bad][3][10, 10] = -1.0  # negative pressure: the reconstruction check fails on step 1
    cfg = _cfg(hg)
    got, info, pinfo = _run_batch(hg, probs, cfg, shape=0, schedule=2)
    assert info.halted_problems >= 1
    assert pinfo[bad]["halted"] != 0
    for k, (m, n) in enumerate(SIZES):
        if k == bad:
            continue
        assert pinfo[k]["halted"] == 0
        want, _ = _one_problem_fp32(hg, probs[k], m, n)
        assert rel_l1(got[k]["rho"], want["rho"]) <= 1e-6
    want, winfo = _one_problem_fp32(hg, probs[bad], *SIZES[bad])
    assert winfo.halted == pinfo[bad]["halted"]
    for f in FIELDS:
        np.testing.assert_array_equal(got[bad][f], want[f])


@pytest.mark.gpu
def test_one_call_batch_entry(gpu_lib):
    """hydro_gb300_batch_run through its C structs (the call a C user makes)."""
    hg = gpu_lib
    L = hg.lib()

    class Info(ctypes.Structure):
        _fields_ = hg.BatchInfo._fields_

    class Problem(ctypes.Structure):
        _fields_ = [("m", ctypes.c_int), ("n", ctypes.c_int)] + [
            (f, ctypes.POINTER(ctypes.c_double)) for f in ("rho", "u", "v", "p", "E")] + [
            ("halted", ctypes.c_int), ("halted_step", ctypes.c_int), ("tau", ctypes.c_double)]

    class Opts(ctypes.Structure):
        _fields_ = [("cfg", ctypes.POINTER(ctypes.c_double)), ("ncfg", ctypes.c_int),
                    ("autotune_steps", ctypes.c_int), ("shape", ctypes.c_int), ("schedule", ctypes.c_int),
                    ("stats", ctypes.c_int), ("info", Info)]

    probs = _problems(hg)
    cfg = _cfg(hg)
    arrs = []
    P = (Problem * len(SIZES))()
    dp = ctypes.POINTER(ctypes.c_double)
    for k, (m, n) in enumerate(SIZES):
        a = [np.ascontiguousarray(x, np.float64).copy() for x in probs[k]] + [np.zeros((m, n))]
        arrs.append(a)
        P[k].m, P[k].n = m, n
        P[k].rho, P[k].u, P[k].v, P[k].p = (x.ctypes.data_as(dp) for x in a[:4])
        P[k].E = None
    o = Opts(cfg.ctypes.data_as(dp), len(cfg), 0, 0, 2, 0)
    L.hydro_gb300_batch_run.argtypes = [ctypes.POINTER(Problem), ctypes.c_int, ctypes.c_int, ctypes.POINTER(Opts)]
    assert L.hydro_gb300_batch_run(P, len(SIZES), STEPS, ctypes.byref(o)) == 0, hg.last_error()
    assert o.info.steps == STEPS and o.info.schedule == 2
    ref, _, pinfo = _run_batch(hg, probs, cfg, 0, 2)
    for k in range(len(SIZES)):
        assert P[k].tau == pinfo[k]["tau"]
        for i, f in enumerate(FIELDS):
            assert np.array_equal(arrs[k][i], ref[k][f])


def test_batch_sizes_are_seeded_and_in_range():
    from hydro_gb300 import cases

    s1 = cases.batch_sizes(512, seed=4)
    s2 = cases.batch_sizes(512, seed=4)
    assert s1 == s2 and len(s1) == 512
    Ns = {m for m, n in s1}
    assert all(m == n for m, n in s1)
    assert Ns <= set(range(64, 513, 32)) and len(Ns) == 15


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["tile", "strip"])
def test_batch_barrier_wait_runs_out(gpu_lib, kind):
    """The persistent schedule's grid barrier gives up when its wait limit runs
    out: with a limit of a nanosecond the first block to arrive stops waiting,
    every block leaves the time loop, the run returns -2 with the barrier error
    reported, and the same handle then runs normally with the limit restored."""
    hg = gpu_lib
    probs = _problems(hg)
    cfg = _cfg(hg)
    b = hg.Batch(SIZES)
    try:
        shape = 0 if kind == "tile" else _strip_shapes(hg)[0][0]
        b.set_schedule(shape, 0)  # one persistent cooperative kernel for all steps
        for k, (rho, u, v, p) in enumerate(probs):
            b.upload(k, rho, u, v, p, gamma=float(cfg[6]))
        b.set_wait_limit(1e-9)
        info = hg.BatchInfo()
        c = np.ascontiguousarray(cfg, np.float64)
        L = hg.lib()
        L.hydro_batch_run.restype = ctypes.c_int
        rc = L.hydro_batch_run(b._h, c, len(c), STEPS, 0, ctypes.byref(info))
        assert rc == -2, rc
        assert "barrier" in hg.last_error()
        b.set_wait_limit(5.0)
        for k, (rho, u, v, p) in enumerate(probs):
            b.upload(k, rho, u, v, p, gamma=float(cfg[6]))
        info = b.run(cfg, STEPS)
        assert info.steps == STEPS and info.halted_problems == 0
        got = [b.download(k) for k in range(len(SIZES))]
    finally:
        b.close()
    ref, _, _ = _run_batch(hg, probs, cfg, shape, 0)
    for k in range(len(SIZES)):
        for f in FIELDS:
            assert np.array_equal(got[k][f], ref[k][f])
