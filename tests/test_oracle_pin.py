"""Pin the oracle (C restatement) to the reference: bit-for-bit against the
golden fixtures generated from the reference's own sources
(tests/golden/make_golden.py), against the reference library itself where the
reference tree exists, and against analytic known answers.

Every test runs twice: with the oracle as built ("port", which calls this
host's C library pow, as the reference does) and with its twin whose pow is
the FP64 device path's (``lpow``: a host build of csrc/libm_pow.cuh).  The
twin passing every pin bit for bit shows, without a GPU, that the device's pow
rounds as the reference's does on every argument these runs produce."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", params=["port", "lpow"])
def port(request):
    import oracle as orc

    if not (os.path.exists(orc.PORT_SO) and os.path.exists(orc.LPOW_SO)):
        orc.build()
    return orc.Oracle(request.param)


def load(name):
    return np.load(os.path.join(GOLD, name))


def test_riemann_exact_golden(port):
    d = load("riemann_exact.npz")
    assert np.array_equal(port.riemann_exact(d["inp"], 1e-9, 1e-9, 500), d["out"], equal_nan=True)
    assert np.array_equal(port.riemann_exact_ben(d["inp"][:, [0, 2, 3, 4, 5, 6, 7]], 1e-9, 1e-9, 50), d["out50"],
                          equal_nan=True)


def test_grp2d_flux_golden(port):
    d = load("grp2d_flux.npz")
    got = port.grp2d_flux(d["inp"], float(d["tau"]))
    want = d["out"]
    assert np.array_equal(got[:, 8], want[:, 8])
    ok = want[:, 8] == 0  # the reference leaves the flux of a rejected interface unwritten
    assert ok.mean() > 0.9
    assert np.array_equal(got[ok], want[ok], equal_nan=True)


def test_q1d_golden(port):
    d = load("q1d.npz")
    got, want = port.q1d(d["inp"]), d["out"]
    fin = np.isfinite(want).all(axis=1)
    assert np.array_equal(got[fin], want[fin])


def test_g2d_golden(port):
    """The genuinely-2D GRP solver, both atc modes, against the reference's
    linear_GRP_solver_Edir_G2D: bit for bit, and different from the quasi-1D
    solver on most of these rows (the cases reach its own branches)."""
    d = load("g2d.npz")
    assert np.array_equal(port.g2d(d["inp"], 1e-9, 1e-9), d["out"], equal_nan=True)
    assert np.array_equal(port.g2d(d["inp"], 1e-9, np.inf), d["out_acoustic"], equal_nan=True)
    q = port.q1d(d["inp"], 1e-9, 1e-9)
    differ = ~np.all((q == d["out"]) | (np.isnan(q) & np.isnan(d["out"])), axis=1)
    assert differ.mean() > 0.3


def test_runs_2d_g2d_golden(port):
    """Whole runs with config[301] = 1 against the reference built with
    GRP_2D_flux calling the genuinely-2D solver (unsplit and split, every
    boundary kind in the set)."""
    d = load("runs_2d_g2d.npz")
    names = _runs(d)
    assert len(names) >= 5
    for name in names:
        meta = d[f"{name}/meta"]
        cfg = d[f"{name}/cfg"]
        assert cfg[301] == 1
        out = port.run_2d(d[f"{name}/in_rho"], d[f"{name}/in_u"], d[f"{name}/in_v"], d[f"{name}/in_p"],
                          cfg, split=int(meta[2]))
        assert out["steps"] == meta[0] and out["time"] == meta[1], name
        for f in ("rho", "u", "v", "p", "E"):
            assert np.array_equal(out[f], d[f"{name}/{f}"]), (name, f)
        if meta[2] == 0:
            # the switch matters: the quasi-1D solver gives another result.  (The
            # split sweeps pass no tangential derivatives, and without them the
            # two solvers differ only in their uniform-pair test.)
            q = cfg.copy()
            q[301] = np.inf
            other = port.run_2d(d[f"{name}/in_rho"], d[f"{name}/in_u"], d[f"{name}/in_v"], d[f"{name}/in_p"], q)
            assert not np.array_equal(other["rho"], out["rho"]), name


def test_grp1d_golden(port):
    d = load("grp1d.npz")
    assert np.array_equal(port.grp1d(d["inp"], 1e-9, 1e-9), d["out_grp"], equal_nan=True)
    assert np.array_equal(port.grp1d(d["inp"], 1e-9, np.inf), d["out_acoustic"], equal_nan=True)


def _runs(d):
    names = sorted({k.split("/")[0] for k in d.files if k.split("/")[1] == "meta" and k.split("/")[0] != "snap"})
    return names


def test_runs_2d_golden(port):
    d = load("runs_2d.npz")
    names = _runs(d)
    assert len(names) >= 6
    for name in names:
        meta = d[f"{name}/meta"]
        out = port.run_2d(d[f"{name}/in_rho"], d[f"{name}/in_u"], d[f"{name}/in_v"], d[f"{name}/in_p"],
                          d[f"{name}/cfg"], split=int(meta[2]))
        assert out["steps"] == meta[0] and out["time"] == meta[1], name
        for f in ("rho", "u", "v", "p", "E"):
            assert np.array_equal(out[f], d[f"{name}/{f}"]), (name, f)


def test_plot_snapshots_golden(port):
    d = load("runs_2d.npz")
    rho, u, v, p = d["snap/in"]
    out = port.run_2d(rho, u, v, p, d["snap/cfg"], plot_times=[0.02, 0.05], want_snaps=True)
    assert np.array_equal(out["snaps"], d["snap/snaps"])
    assert out["steps"] == d["snap/meta"][0] and out["time"] == d["snap/meta"][1]


def test_runs_1d_golden(port):
    d = load("runs_1d.npz")
    for order in (1, 2):
        from hydro_gb300 import cases

        rho, u, p = cases.sod(400)
        out = port.run_1d(rho, u, p, d[f"sod{order}/cfg"], order)
        assert out["steps"] == d[f"sod{order}/meta"][0] and out["time"] == d[f"sod{order}/meta"][1]
        for f in ("rho", "u", "p", "E"):
            assert np.array_equal(out[f], d[f"sod{order}/{f}"]), (order, f)
    for name in ("bc7o2", "bc2o2", "bc24o1", "bc1o2"):
        rho, u, p = d[f"{name}/in"]
        meta = d[f"{name}/meta"]
        out = port.run_1d(rho, u, p, d[f"{name}/cfg"], int(meta[2]))
        assert out["steps"] == meta[0] and out["time"] == meta[1], name
        for f in ("rho", "u", "p", "E"):
            assert np.array_equal(out[f], d[f"{name}/{f}"]), (name, f)


def test_sod_exact_star_state(port):
    """Known answer: Sod's star state p* = 0.30313, u* = 0.92745 (Toro, table 4.3)."""
    g = 1.4
    inp = np.array([[g, g, 0.0, 0.0, 1.0, 0.1, np.sqrt(g * 1.0 / 1.0), np.sqrt(g * 0.1 / 0.125)]])
    out = port.riemann_exact(inp)
    assert abs(out[0, 1] - 0.30313) < 5e-5 and abs(out[0, 0] - 0.92745) < 5e-5
    assert out[0, 2] == 1 and out[0, 3] == 0  # left rarefaction, right shock


def test_sod_scheme_plateau(port):
    """The 1D schemes reproduce the star state on the plateau (x ~ 0.6 at t = 0.2)."""
    d = load("runs_1d.npz")
    for order in (1, 2):
        p = d[f"sod{order}/p"]
        u = d[f"sod{order}/u"]
        assert abs(p[240] - 0.30313) < 2e-3 and abs(u[240] - 0.92745) < 2e-3


def test_port_matches_reference_random(port, ref):
    """Fresh random inputs, both libraries (only where the reference tree exists)."""
    rng = np.random.default_rng(99)
    n = 4000
    rho = np.exp(rng.uniform(-4, 4, (n, 2))); p = np.exp(rng.uniform(-4, 4, (n, 2))); u = rng.uniform(-3, 3, (n, 2))
    c = np.sqrt(1.4 * p / rho)
    inp = np.column_stack([np.full(n, 1.4), np.full(n, 1.4), u[:, 0], u[:, 1], p[:, 0], p[:, 1], c[:, 0], c[:, 1]])
    assert np.array_equal(port.riemann_exact(inp), ref.riemann_exact(inp), equal_nan=True)
    from hydro_gb300 import cases
    import oracle as orc

    rho, u, v, p = cases.shear_layer(24, 20, 5)
    cfg = orc.default_config_2d(t_all=-1, steps=25, hx=1 / 24, hy=1 / 20, bx=-7, by=-4)
    a, b = port.run_2d(rho, u, v, p, cfg), ref.run_2d(rho, u, v, p, cfg)
    for f in ("rho", "u", "v", "p", "E"):
        assert np.array_equal(a[f], b[f])


def test_g2d_port_matches_reference_random(port, ref_g2d):
    """Fresh random faces and a fresh run against the reference's G2D build."""
    import oracle as orc
    from hydro_gb300 import cases

    rng = np.random.default_rng(123)
    n = 1500
    L = np.column_stack([np.exp(rng.uniform(-3, 3, n)), rng.uniform(-3, 3, (n, 2)), np.exp(rng.uniform(-3, 3, n)),
                         rng.normal(0, 2, (n, 8))])
    R = np.column_stack([np.exp(rng.uniform(-3, 3, n)), rng.uniform(-3, 3, (n, 2)), np.exp(rng.uniform(-3, 3, n)),
                         rng.normal(0, 2, (n, 8))])
    inp = np.column_stack([np.full(n, 1.4), L, R])
    assert np.array_equal(port.g2d(inp), ref_g2d.g2d(inp), equal_nan=True)
    rho, u, v, p = cases.four_quadrant(22, 18, 31)
    cfg = orc.default_config_2d(t_all=-1, steps=20, hx=1 / 22, hy=1 / 18, bx=-7, by=-2)
    cfg[301] = 1
    a, b = port.run_2d(rho, u, v, p, cfg), ref_g2d.run_2d(rho, u, v, p, cfg)
    for f in ("rho", "u", "v", "p", "E"):
        assert np.array_equal(a[f], b[f])


def test_lag_golden(port):
    """linear_GRP_solver_LAG, nonlinear and acoustic modes, bit for bit."""
    d = load("lag.npz")
    assert np.array_equal(port.lag(d["inp"], 1e-9, 1e-9), d["out"], equal_nan=True)
    assert np.array_equal(port.lag(d["inp"], 1e-9, np.inf), d["out_acoustic"], equal_nan=True)


def test_runs_1d_lag_golden(port):
    """Godunov_solver_LAG_source / GRP_solver_LAG_source: Sod and every
    boundary code, state and moving node coordinates bit for bit."""
    d = load("runs_1d_lag.npz")
    names = _runs(d)
    assert len(names) >= 9
    for name in names:
        rho, u, p = d[f"{name}/in"]
        meta = d[f"{name}/meta"]
        out = port.run_1d_lag(rho, u, p, d[f"{name}/cfg"], int(meta[2]))
        assert out["steps"] == meta[0] and out["time"] == meta[1], name
        for f in ("rho", "u", "p", "E", "X"):
            assert np.array_equal(out[f], d[f"{name}/{f}"]), (name, f)


def test_lag_sod_known_answer(port):
    """Sod in Lagrangian coordinates: the contact moves at u* = 0.92745, so the
    node that starts at x = 0.5 ends at 0.5 + 0.2 u*; the plateau pressure is
    p* = 0.30313 (Toro, table 4.3)."""
    d = load("runs_1d_lag.npz")
    for order in (1, 2):
        X = d[f"sod{order}/X"]
        assert abs(X[200] - (0.5 + 0.2 * 0.92745)) < 2e-3
        p = d[f"sod{order}/p"]
        assert abs(p[200] - 0.30313) < 5e-3


def test_lag_port_matches_reference_random(port, ref):
    rng = np.random.default_rng(77)
    n = 800
    side = lambda: np.column_stack([np.exp(rng.uniform(-3, 3, n)), rng.uniform(-3, 3, n), np.exp(rng.uniform(-3, 3, n)),
                                    rng.normal(0, 2, (n, 3))])
    inp = np.column_stack([np.full(n, 1.4), side(), side()])
    assert np.array_equal(port.lag(inp), ref.lag(inp), equal_nan=True)
    import oracle as orc

    m = 90
    x = (np.arange(m) + 0.5) / m
    rho, u, p = 1 + 0.3 * np.cos(4 * np.pi * x), 0.2 * np.sin(2 * np.pi * x), 1 + 0.5 * (x > 0.45)
    for order in (1, 2):
        cfg = orc.default_config_1d(t_all=0.08, steps=100000, hx=1 / m, bx=-7, cfl=0.4)
        a, b = port.run_1d_lag(rho, u, p, cfg, order), ref.run_1d_lag(rho, u, p, cfg, order)
        for f in ("rho", "u", "p", "E", "X"):
            assert np.array_equal(a[f], b[f])


# -- two-component (MULTIFLUID_BASICS) interface flux --------------------------

def _mf_rows_equal(got, want):
    """Same return code everywhere; outputs bit for bit where the reference
    returned 0 (on a failed check it returns before writing them)."""
    assert np.array_equal(got[:, 18], want[:, 18])
    ok = want[:, 18] == 0
    assert np.array_equal(got[ok], want[ok])


def test_mf_flux_golden(port):
    """The two-component GRP_2D_flux against the reference's MULTIFLUID build:
    per-side gamma, volume/mass fractions, mixture gamma, F_gamma on and off."""
    d = load("grp2d_flux_mf.npz")
    tau, ga, gb = float(d["tau"]), float(d["gamma_a"]), float(d["gamma_b"])
    _mf_rows_equal(port.grp2d_flux_mf(d["inp"], tau, 1e-9, ga, gb, True), d["out"])
    _mf_rows_equal(port.grp2d_flux_mf(d["inp"], tau, 1e-9, ga, gb, False), d["out_nogamma"])
    out = d["out"]
    assert (out[:, 18] == 0).mean() > 0.9
    assert np.all(d["out_nogamma"][out[:, 18] == 0, 9] == 0.0)


def test_mf_flux_reduces_to_single_fluid(port):
    """One gamma on both sides equal to config[6] and z = 1 with flat z: the
    mixture gamma is config[6] and the gas-dynamic outputs are those of the
    single-fluid GRP_2D_flux, bit for bit; the component fluxes follow from
    them (F_phi = F_rho phi_mid with phi_mid = PHI at tau/2)."""
    d = load("grp2d_flux_mf.npz")
    inp = d["inp"].copy()
    g = 1.4
    inp[:, 2] = g
    inp[:, 21] = g
    inp[:, 15] = inp[:, 34] = 1.0
    inp[:, [16, 17, 35, 36]] = 0.0
    mf = port.grp2d_flux_mf(inp, 1e-3, 1e-9, g, 3.0, True)
    single = np.column_stack([inp[:, 0], inp[:, 1], np.full(len(inp), g), inp[:, 3:15], inp[:, 22:34]])
    sf = port.grp2d_flux(single, 1e-3)
    ok = sf[:, 8] == 0
    assert np.array_equal(mf[:, 18], sf[:, 8])
    assert np.array_equal(mf[ok, :8], sf[ok, :8])
    assert np.array_equal(mf[ok, 12], np.ones(ok.sum()))           # Z_a stays 1
    np.testing.assert_allclose(mf[ok, 9], mf[ok, 0] * g, rtol=1e-15)  # F_gamma = F_rho gamma_mid


def test_mf_port_matches_reference_random(port, ref_mf):
    """Fresh random two-component faces (wide state ranges, any normal)
    against the reference's MULTIFLUID build."""
    rng = np.random.default_rng(321)
    n = 3000

    def side():
        return np.column_stack([rng.uniform(1.05, 4.0, n), np.exp(rng.uniform(-3, 3, n)), rng.uniform(-3, 3, (n, 2)),
                                np.exp(rng.uniform(-3, 3, n)), rng.normal(0, 2, (n, 8)), rng.uniform(0, 1, n),
                                rng.normal(0, 1, (n, 2)), rng.uniform(0, 1, n), rng.normal(0, 1, (n, 2))])
    th = rng.uniform(0, 2 * np.pi, n)
    inp = np.column_stack([np.cos(th), np.sin(th), side(), side()])
    for ga, gb, sg in ((1.4, 3.0, True), (1.67, 1.2, False)):
        _mf_rows_equal(port.grp2d_flux_mf(inp, 2e-3, 1e-9, ga, gb, sg), ref_mf.grp2d_flux_mf(inp, 2e-3, 1e-9, ga, gb, sg))
