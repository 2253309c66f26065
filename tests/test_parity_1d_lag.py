"""GPU parity of the 1D Lagrangian Godunov and GRP schemes (FP64) with the
reference's golden runs (tests/golden/runs_1d_lag.npz: Sod, every boundary
code, a fixed time step), with the oracle on fresh data, and through the
reference's entry points Godunov_solver_LAG_source / GRP_solver_LAG_source
(caller-owned CV and X slots, plot snapshots)."""
import ctypes
import os

import numpy as np
import pytest

from helpers import rel_l1

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


def _run(hg, rho, u, p, cfg, order):
    L = hg.lib()
    L.hydro1d_run_lag.restype = ctypes.c_int
    rho, u, p = (np.array(a, np.float64) for a in (rho, u, p))
    g = float(cfg[6])
    E = 0.5 * u * u + p / (g - 1.0) / rho
    X = np.zeros(len(rho) + 1)
    info = hg.RunInfo()
    cfg = np.ascontiguousarray(cfg, np.float64)
    P = ctypes.POINTER(ctypes.c_double)
    rc = L.hydro1d_run_lag(len(rho), rho.ctypes.data_as(P), u.ctypes.data_as(P), p.ctypes.data_as(P),
                           E.ctypes.data_as(P), X.ctypes.data_as(P), cfg.ctypes.data_as(P), len(cfg), order,
                           ctypes.byref(info))
    assert rc == 0, hg.last_error()
    return dict(rho=rho, u=u, p=p, E=E, X=X), info


def _names():
    d = np.load(os.path.join(GOLD, "runs_1d_lag.npz"))
    return sorted({k.split("/")[0] for k in d.files})


@pytest.mark.gpu
@pytest.mark.parametrize("name", _names())
def test_lag_matches_reference_golden(gpu_lib, name):
    hg = gpu_lib
    d = np.load(os.path.join(GOLD, "runs_1d_lag.npz"))
    rho, u, p = d[f"{name}/in"]
    meta = d[f"{name}/meta"]
    got, info = _run(hg, rho, u, p, d[f"{name}/cfg"], int(meta[2]))
    assert info.k_out == int(meta[0]) and info.time == meta[1], name
    for f in ("rho", "u", "p", "E", "X"):
        assert rel_l1(got[f], d[f"{name}/{f}"]) <= TOL, (name, f, rel_l1(got[f], d[f"{name}/{f}"]))
    # the device rounds every operation, pow included, as the reference does
    for f in ("rho", "u", "p", "E", "X"):
        assert np.array_equal(got[f], d[f"{name}/{f}"]), (name, f)


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("m", [37, 600, 5000])
def test_lag_random_tube_matches_oracle(gpu_lib, order, m):
    """Sizes below, at and beyond one thread per interface of a 16-CTA cluster,
    against the oracle."""
    hg = gpu_lib
    import oracle as orc

    port = orc.Oracle("port")

    rng = np.random.default_rng(m + order)
    x = (np.arange(m) + 0.5) / m
    rho = 1.0 + 0.4 * np.sin(2 * np.pi * x) + 0.5 * (x > rng.uniform(0.3, 0.7))
    u = 0.2 * np.cos(4 * np.pi * x)
    p = 1.0 + 0.3 * (x < 0.5) + 0.05 * rng.uniform(size=m)
    steps = 40 if m > 1000 else 200
    cfg = orc.default_config_1d(t_all=-1, steps=steps, hx=1 / m, bx=-7, cfl=0.45)
    cfg[1] = np.inf
    want = port.run_1d_lag(rho, u, p, cfg, order)
    got, info = _run(hg, rho, u, p, cfg, order)
    assert info.k_out == want["steps"]
    for f in ("rho", "u", "p", "E", "X"):
        assert rel_l1(got[f], want[f]) <= TOL, (f, rel_l1(got[f], want[f]))


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_lag_dropin_entry_with_snapshots(gpu_lib, order):
    """The reference's entry points with two plot times: the stored CV/X slots
    hold the state at the first step past each plot time, the last slot the
    final state; config[5] and time_plot come back as the reference writes
    them (checked against the oracle)."""
    hg = gpu_lib
    from hydro_gb300 import cases
    from hydro_gb300.dropin import call_1d_lag
    import oracle as orc

    port = orc.Oracle("port")

    rho, u, p = cases.sod(200)
    cfg = orc.default_config_1d(t_all=0.2, steps=100000, hx=1 / 200, bx=-4, cfl=0.45)
    data, X, nplot, time_plot, k_out = call_1d_lag(hg.lib(), rho, u, p, 1.4, cfg.copy(), order,
                                                   plot_times=[0.05, 0.1])
    assert nplot == 4
    want = port.run_1d_lag(rho, u, p, cfg, order)
    assert k_out == want["steps"] and time_plot[-1] == want["time"]
    for f, key in enumerate(("rho", "u", "p", "E")):
        assert rel_l1(data[f, nplot - 1], want[key]) <= TOL, key
    assert rel_l1(X[nplot - 1], want["X"]) <= TOL
    # slot k is the state (and nodes) at the start of the first step whose time has reached
    # time_plot[k]: the oracle after K steps with no end time, K the first count reaching it
    K = 1
    for k in (1, 2):
        while True:
            c = orc.default_config_1d(t_all=-1, steps=K, hx=1 / 200, bx=-4, cfl=0.45)
            ref = port.run_1d_lag(rho, u, p, c, order)
            if ref["time"] >= time_plot[k]:
                break
            K += 1
        for f, key in enumerate(("rho", "u", "p", "E")):
            assert rel_l1(data[f, k], ref[key]) <= TOL, (k, key)
        assert rel_l1(X[k], ref["X"]) <= TOL, k


@pytest.mark.gpu
def test_lag_unknown_boundary_is_reported(gpu_lib):
    hg = gpu_lib
    import oracle as orc
    from hydro_gb300 import cases

    rho, u, p = cases.sod(50)
    cfg = orc.default_config_1d(t_all=0.1, steps=100, hx=1 / 50, bx=-3, cfl=0.45)
    L = hg.lib()
    P = ctypes.POINTER(ctypes.c_double)
    info = hg.RunInfo()
    cfg = np.ascontiguousarray(cfg)
    rc = L.hydro1d_run_lag(50, rho.ctypes.data_as(P), u.ctypes.data_as(P), p.ctypes.data_as(P), None, None,
                           cfg.ctypes.data_as(P), len(cfg), 2, ctypes.byref(info))
    assert rc == -2
