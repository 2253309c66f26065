"""Conservation: with periodic boundaries the conservative update telescopes,
so the domain integrals of mass, momentum and energy change only by
round-off from step to step.  Checked through hydro2d_conservation (FP64,
fixed-order reduction), which is itself checked against the downloaded state."""
import numpy as np
import pytest

STEPS = 60


def _integrals(st, hx, hy):
    rho, u, v, E = st["rho"], st["u"], st["v"], st["E"]
    return np.array([rho.sum(), (rho * u).sum(), (rho * v).sum(), (rho * E).sum()]) * hx * hy


@pytest.mark.gpu
@pytest.mark.parametrize("form,tol", [(0, 1e-13), (1, 2e-6), (2, 2e-6)])
@pytest.mark.parametrize("split", [0, 1])
def test_periodic_drift_is_round_off(gpu_lib, form, tol, split):
    hg = gpu_lib
    from hydro_gb300 import cases

    m, n = 96, 80
    rho, u, v, p = cases.shear_layer(m, n, seed=3)
    hx, hy = 1.0 / m, 1.0 / n
    s = hg.Solver2D(m, n, form)
    try:
        if form == hg.FORM_FP32_LEARNED:
            s.set_mlp(hg.load_weights())
        s.upload(rho, u, v, p)
        c0 = s.conservation(hx, hy)
        st0 = s.download()
        info = s.run(hg.config_2d(t_all=-1, steps=STEPS, hx=hx, hy=hy, bx=-7, by=-7, split=split))
        assert info.halted == 0
        c1 = s.conservation(hx, hy)
        st1 = s.download()
    finally:
        s.close()
    # the API's integrals are the state's
    for c, st in ((c0, st0), (c1, st1)):
        got = np.array([c["mass"], c["mom_x"], c["mom_y"], c["energy"]])
        want = _integrals(st, hx, hy)
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-15)
    # drift of each integral, relative to the mass (momentum can integrate to ~0)
    scale = abs(c0["mass"])
    for key in ("mass", "mom_x", "mom_y", "energy"):
        assert abs(c1[key] - c0[key]) <= tol * max(scale, abs(c0[key])), (key, c0[key], c1[key])
    # and the run did something: the state moved
    assert np.abs(st1["rho"] - st0["rho"]).max() > 1e-3
