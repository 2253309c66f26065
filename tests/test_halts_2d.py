"""The reference's halting semantics on the single-grid FP64 path, driven by
bad states made on the host and compared with the oracle.

GRP_solver_2D_EUL_source stops a run in two ways
(src/finite_volume/grp_solver_2D_EUL_source.c):
  * stop_t -- the step is finished and kept, then the loop ends: a time step
    below eps (:193-197), a face whose star state or derivatives fail their
    check (flux_generator_x/_y returning 2, :219-225, flux_generator_x.c:
    132-152), a non-positive pressure or density after the update (:249-253);
  * return_NULL -- the loop ends at once and the step is discarded: a
    non-finite time step (:200-204), a face whose states fail ifvar_check
    (flux_generator_x/_y returning 1).
The device records the same keys per launch and resolves the outcome on the
host; here every case runs on the GPU and on the oracle (the reference's loop
restated in C, pinned to it bit for bit) from the same input, and the step
count config[5], the final time and the whole state must agree (NaN where the
reference leaves NaN).
"""
import numpy as np
import pytest

from helpers import rel_l1

M, N = 40, 36
FIELDS = ("rho", "u", "v", "p", "E")


def _base(hg):
    from hydro_gb300 import cases

    return [a.copy() for a in cases.four_quadrant(M, N, seed=7)]


def _cfg(hg, **kw):
    d = dict(t_all=-1, steps=6, hx=1.0 / M, hy=1.0 / N, bx=-4, by=-4)
    d.update(kw)
    return hg.config_2d(**d)


def _case(hg, name):
    r, u, v, p = _base(hg)
    cfg = _cfg(hg)
    if name == "negative_pressure":
        p[20, 17] = -0.5  # its faces' star states go non-finite: stop after the step
    elif name == "nan_density":
        r[10, 30] = np.nan  # ifvar_check fails: the step is discarded
    elif name == "tiny_time_step":
        cfg = _cfg(hg, t_all=1.0, hx=1e-12, hy=1e-12)  # CFL tau ~ 1e-13 < eps = 1e-9: stop
    elif name == "vacuum":
        r[:] = 1.0
        p[:] = 0.1
        u[: M // 2] = -3.0
        u[M // 2:] = 3.0
        v[:] = 0.0
        cfg = _cfg(hg, steps=30)
    elif name == "fixed_tiny_tau":
        cfg[16] = 1e-13  # a fixed time step is not checked against eps: no halt
    return (r, u, v, p), cfg


# case -> the device's halt kind (1 = discarded step, 2 = kept step, 0 = none).
# The time step is computed on the host (the CFL minimum of the initial data,
# as the reference's loop computes it), so a time step below eps ends the
# host's plan of launches after that step: no device halt, the same outcome.
KINDS = {"negative_pressure": 2, "nan_density": 1, "tiny_time_step": 0, "vacuum": 2, "fixed_tiny_tau": 0}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(KINDS))
def test_halt_matches_oracle(gpu_lib, port, name):
    hg = gpu_lib
    (r, u, v, p), cfg = _case(hg, name)
    want = port.run_2d(r, u, v, p, cfg)
    got, info = hg.run_2d(r, u, v, p, cfg)
    assert info.halted == KINDS[name], (name, info.halted)
    assert info.k_out == int(want["steps"]), (name, info.k_out, want["steps"])
    assert info.time == want["time"], (name, info.time, want["time"])
    for f in FIELDS:
        a, b = got[f], want[f]
        assert np.array_equal(np.isnan(a), np.isnan(b)), (name, f)
        ok = ~np.isnan(b)
        assert rel_l1(a[ok], b[ok]) <= 1e-12, (name, f, rel_l1(a[ok], b[ok]))


@pytest.mark.gpu
def test_halt_through_the_scheme_entry(gpu_lib, port):
    """The reference's entry point with a discarded step: config[5] and the
    stored snapshot are the reference's."""
    hg = gpu_lib
    from hydro_gb300.dropin import call_2d

    (r, u, v, p), cfg = _case(hg, "nan_density")
    want = port.run_2d(r, u, v, p, cfg)
    data, nplot, time_plot, k_out = call_2d(hg.lib(), r, u, v, p, 1.4, cfg.copy(), N_MAX=2)
    assert k_out == int(want["steps"])
    for i, f in enumerate(("rho", "u", "v", "p")):
        a, b = data[nplot - 1, i], want[f]
        assert np.array_equal(np.isnan(a), np.isnan(b)), f
        ok = ~np.isnan(b)
        assert rel_l1(a[ok], b[ok]) <= 1e-12, f
