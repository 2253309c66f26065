"""GPU parity of the 1D Godunov and GRP schemes (FP64) with the oracle and
with the reference's golden runs (Sod tube and every boundary code)."""
import ctypes
import os

import numpy as np
import pytest

from helpers import rel_l1

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


def _run(hg, rho, u, p, cfg, order):
    L = hg.lib()
    L.hydro1d_run.restype = ctypes.c_int
    rho, u, p = (np.array(a, np.float64) for a in (rho, u, p))
    g = float(cfg[6])
    E = 0.5 * u * u + p / (g - 1.0) / rho  # the 1D driver's energy (src/hydrocode_1D/hydrocode.c:235)
    info = hg.RunInfo()
    cfg = np.ascontiguousarray(cfg, np.float64)
    P = ctypes.POINTER(ctypes.c_double)
    rc = L.hydro1d_run(len(rho), rho.ctypes.data_as(P), u.ctypes.data_as(P), p.ctypes.data_as(P),
                       E.ctypes.data_as(P), cfg.ctypes.data_as(P), len(cfg), order, ctypes.byref(info))
    assert rc == 0, hg.last_error()
    return dict(rho=rho, u=u, p=p, E=E), info


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_sod_matches_reference_golden(gpu_lib, order):
    hg = gpu_lib
    from hydro_gb300 import cases

    d = np.load(os.path.join(GOLD, "runs_1d.npz"))
    rho, u, p = cases.sod(400)
    got, info = _run(hg, rho, u, p, d[f"sod{order}/cfg"], order)
    assert info.k_out == int(d[f"sod{order}/meta"][0])
    assert info.time == d[f"sod{order}/meta"][1]
    for f in ("rho", "u", "p", "E"):
        assert rel_l1(got[f], d[f"sod{order}/{f}"]) <= TOL, f


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["bc7o2", "bc2o2", "bc24o1", "bc1o2"])
def test_boundaries_match_reference_golden(gpu_lib, name):
    hg = gpu_lib
    d = np.load(os.path.join(GOLD, "runs_1d.npz"))
    rho, u, p = d[f"{name}/in"]
    meta = d[f"{name}/meta"]
    got, info = _run(hg, rho, u, p, d[f"{name}/cfg"], int(meta[2]))
    assert info.k_out == int(meta[0]) and info.time == meta[1]
    for f in ("rho", "u", "p", "E"):
        assert rel_l1(got[f], d[f"{name}/{f}"]) <= TOL, (name, f)


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_random_tube_matches_oracle(gpu_lib, port, order):
    hg = gpu_lib
    rng = np.random.default_rng(order)
    m = 1500  # more cells than threads of the persistent CTA
    rho = rng.uniform(0.2, 2.0, m)
    u = rng.uniform(-1, 1, m)
    p = rng.uniform(0.2, 2.0, m)
    import oracle as orc

    cfg = orc.default_config_1d(t_all=0.01, steps=100000, hx=1.0 / m, bx=-7, cfl=0.5)
    want = port.run_1d(rho, u, p, cfg, order)
    got, info = _run(hg, rho, u, p, cfg, order)
    assert info.k_out == int(want["steps"]) and info.time == want["time"]
    for f in ("rho", "u", "p", "E"):
        assert rel_l1(got[f], want[f]) <= TOL, f
