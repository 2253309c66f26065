"""The reference's scheme entry points, called the way its drivers call them
(global config[], caller-owned struct cell_var_stru arrays), against the
reference's golden output (plot snapshots included)."""
import os

import numpy as np
import pytest

from hydro_gb300.dropin import call_1d, call_2d
from helpers import rel_l1

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


@pytest.mark.gpu
def test_2d_entry_with_plot_snapshots(gpu_lib, host_path):
    hg = gpu_lib
    d = np.load(os.path.join(GOLD, "runs_2d.npz"))
    rho, u, v, p = d["snap/in"]
    cfg = d["snap/cfg"].copy()
    data, nplot, time_plot, k_out = call_2d(hg.lib(), rho, u, v, p, 1.4, cfg, plot_times=[0.02, 0.05])
    snaps = d["snap/snaps"]
    assert nplot == snaps.shape[0]
    assert k_out == d["snap/meta"][0] and time_plot[nplot - 1] == d["snap/meta"][1]
    for k in range(nplot):
        for f in range(5):
            assert rel_l1(data[k, f], snaps[k, f]) <= TOL, (k, f)


@pytest.fixture(params=["direct", "default", "staged"])
def host_path(request, monkeypatch):
    """The ways the scheme call moves the caller's rows: read and written by
    the GPU itself (HYDRO_DIRECT_HOST_ROWS=1, where it accesses pageable host
    memory coherently), the default (read by the GPU where it walks the host's
    page tables, written back staged), and packed into one host buffer and
    copied both ways (HYDRO_DIRECT_HOST_ROWS=0)."""
    if request.param == "direct":
        monkeypatch.setenv("HYDRO_DIRECT_HOST_ROWS", "1")
    elif request.param == "staged":
        monkeypatch.setenv("HYDRO_DIRECT_HOST_ROWS", "0")
    else:
        monkeypatch.delenv("HYDRO_DIRECT_HOST_ROWS", raising=False)
    return request.param


@pytest.mark.gpu
@pytest.mark.parametrize("split", [0, 1])
def test_2d_entry_matches_oracle(gpu_lib, port, split, host_path):
    hg = gpu_lib
    from hydro_gb300 import cases

    m, n = 23, 19
    rho, u, v, p = cases.four_quadrant(m, n, 4)
    cfg = hg.config_2d(t_all=0.04, steps=1000, hx=1 / m, hy=1 / n, bx=-4, by=-2, split=split)
    data, nplot, time_plot, k_out = call_2d(hg.lib(), rho, u, v, p, 1.4, cfg, split=split)
    want = port.run_2d(rho, u, v, p, cfg, split=split)
    assert k_out == want["steps"] and time_plot[nplot - 1] == want["time"]
    for f, key in enumerate(("rho", "u", "v", "p", "E")):
        assert rel_l1(data[nplot - 1, f], want[key]) <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_1d_entry_sod(gpu_lib, order):
    hg = gpu_lib
    from hydro_gb300 import cases

    d = np.load(os.path.join(GOLD, "runs_1d.npz"))
    rho, u, p = cases.sod(400)
    data, nplot, time_plot, k_out = call_1d(hg.lib(), rho, u, p, 1.4, d[f"sod{order}/cfg"].copy(), order)
    assert nplot == 2 and k_out == d[f"sod{order}/meta"][0] and time_plot[1] == d[f"sod{order}/meta"][1]
    for f, key in enumerate(("rho", "u", "p", "E")):
        assert rel_l1(data[f, 1], d[f"sod{order}/{key}"]) <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("rows", ["0", "in"])
@pytest.mark.parametrize("form", [0, 1, 2])
def test_entry_row_copies_match_plane_api(gpu_lib, form, rows, monkeypatch):
    """The scheme call's row copies, staged (host threads pack the caller's
    rows, converted to the form's precision, through a pair of host buffers)
    or read by the GPU itself, and the plane API (the device converts) leave
    the same state bit for bit, values at and below the float subnormal range
    included."""
    monkeypatch.setenv("HYDRO_DIRECT_HOST_ROWS", rows)
    hg = gpu_lib
    from hydro_gb300 import cases

    m, n = 40, 33
    rho, u, v, p = (a.copy() for a in cases.four_quadrant(m, n, 6))
    u[3, 4], u[5, 6], v[7, 8], v[9, 10] = 1e-40, -3e-39, 1.1754942e-38, 5e-324
    cfg = hg.config_2d(t_all=-1, steps=15, hx=1 / m, hy=1 / n, bx=-4, by=-4, form=form)
    data, nplot, _, _ = call_2d(hg.lib(), rho, u, v, p, 1.4, cfg.copy())
    E = 0.5 * u * u + p / (1.4 - 1.0) / rho
    E += 0.5 * v * v  # the driver's energy, as the scheme call receives it
    s = hg.Solver2D(m, n, form)
    try:
        if form == hg.FORM_FP32_LEARNED:
            s.set_mlp(hg.load_weights())
        s.upload(rho, u, v, p, E)
        s.run(cfg)
        want = s.download()
    finally:
        s.close()
    for f, key in enumerate(("rho", "u", "v", "p", "E")):
        assert np.array_equal(data[nplot - 1, f], want[key]), key


@pytest.mark.gpu
@pytest.mark.parametrize("form", [None, 2])
def test_2d_entry_kept_solver(gpu_lib, monkeypatch, form):
    """The 2D entry keeps the last call's solver for the next call of the same
    grid and form: repeated calls (the kept solver) give the same bits as a call
    with the cache off (HYDRO_SOLVER_CACHE=0, a solver of its own), also after
    a call of another size in between, and after hydro_gb300_release_cache."""
    hg = gpu_lib
    from hydro_gb300 import cases

    m, n = 40, 36
    rho, u, v, p = cases.four_quadrant(m, n, 6)
    cfg = hg.config_2d(t_all=-1, steps=12, hx=1 / m, hy=1 / n, bx=-4, by=-4,
                       **({} if form is None else {"form": form}))
    other = cases.four_quadrant(24, 28, 7)
    cfg_other = hg.config_2d(t_all=-1, steps=5, hx=1 / 24, hy=1 / 28, bx=-4, by=-4,
                             **({} if form is None else {"form": form}))
    monkeypatch.setenv("HYDRO_SOLVER_CACHE", "0")
    ref = call_2d(hg.lib(), rho, u, v, p, 1.4, cfg, N_MAX=2)[0]
    monkeypatch.delenv("HYDRO_SOLVER_CACHE")
    runs = [call_2d(hg.lib(), rho, u, v, p, 1.4, cfg, N_MAX=2)[0] for _ in range(2)]
    call_2d(hg.lib(), *other, 1.4, cfg_other, N_MAX=2)
    runs.append(call_2d(hg.lib(), rho, u, v, p, 1.4, cfg, N_MAX=2)[0])
    hg.lib().hydro_gb300_release_cache()
    runs.append(call_2d(hg.lib(), rho, u, v, p, 1.4, cfg, N_MAX=2)[0])
    for got in runs:
        assert np.array_equal(got[1], ref[1])
    hg.lib().hydro_gb300_release_cache()
