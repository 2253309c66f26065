"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own hot-path sources, compiled unmodified by
``make -C oracle ref`` (oracle/_ref/libhydro_ref.so), on seeded inputs and
stores inputs and float64 outputs as .npz files.  Only this script needs the
reference tree; the fixtures travel with the repository.

    python tests/golden/make_golden.py            # all fixtures
    python tests/golden/make_golden.py --large    # also the 1024^2 x 100 / x 500 run summaries
    python tests/golden/make_golden.py --only large  # only those two summaries
    python tests/golden/make_golden.py --only g2d # only the genuinely-2D solver's fixtures
    python tests/golden/make_golden.py --only lag # only the 1D Lagrangian schemes' fixtures
    python tests/golden/make_golden.py --only mf  # only the two-component interface flux

The genuinely-2D GRP fixtures come from oracle/_ref/libhydro_ref_g2d.so, the
same sources with GRP_2D_flux calling linear_GRP_solver_Edir_G2D (the
alternative the reference keeps commented out at flux_solver.c:189).  The
two-component interface-flux fixture comes from oracle/_ref/libhydro_ref_mf.so
(GRP_2D_flux compiled with MULTIFLUID_BASICS).
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "hydrocode-fusion_gb300"))

import oracle as orc  # noqa: E402
from hydro_gb300 import cases  # noqa: E402

G = 1.4


def riemann_inputs(rng, n):
    """Random pairs plus edge cases: equal states, strong shocks, strong
    rarefactions towards vacuum, transonic rarefactions."""
    rho = np.exp(rng.uniform(np.log(1e-3), np.log(1e3), (n, 2)))
    p = np.exp(rng.uniform(np.log(1e-4), np.log(1e4), (n, 2)))
    u = rng.uniform(-5, 5, (n, 2))
    k = n // 8
    p[:k, 1] = p[:k, 0]; u[:k, 1] = u[:k, 0]                       # trivial
    u[k:2 * k, 0] = 3.0; u[k:2 * k, 1] = -3.0                        # colliding: two shocks
    u[2 * k:3 * k, 0] = -2.0; u[2 * k:3 * k, 1] = 2.0                # receding: two rarefactions
    p[3 * k:4 * k, 1] = p[3 * k:4 * k, 0] * 1e-4                     # strong pressure ratio
    c = np.sqrt(G * p / rho)
    return np.column_stack([np.full(n, G), np.full(n, G), u[:, 0], u[:, 1], p[:, 0], p[:, 1], c[:, 0], c[:, 1]])


def side_block(rng, n, scale=1.0):
    return np.column_stack([np.exp(rng.uniform(-2, 2, n)), rng.uniform(-2, 2, n), rng.uniform(-2, 2, n),
                            np.exp(rng.uniform(-2, 2, n)), rng.normal(0, scale, (n, 8))])


def flux_inputs(rng, n):
    """Interface pairs for x- and y-normals: random, uniform pairs (dist < eps),
    supersonic and sonic cases, with random normal/tangential slopes."""
    L = side_block(rng, n)
    R = side_block(rng, n)
    k = n // 6
    R[:k, :4] = L[:k, :4]                                            # uniform pairs -> acoustic GRP
    R[k:2 * k, :4] = L[k:2 * k, :4] * (1 + 1e-12)                   # near-uniform but above eps
    L[2 * k:3 * k, 1] = 3.0; R[2 * k:3 * k, 1] = 3.2                 # supersonic to the right
    L[3 * k:4 * k, 1] = -3.0; R[3 * k:4 * k, 1] = -3.2               # supersonic to the left
    L[4 * k:5 * k, 1] = -1.5; R[4 * k:5 * k, 1] = 1.5                # rarefactions, sonic points
    normals = np.zeros((n, 2))
    normals[: n // 2, 0] = 1.0
    normals[n // 2:, 1] = 1.0
    return np.column_stack([normals, np.full(n, G), L, R])


def grp1d_inputs(rng, n):
    L = np.column_stack([np.exp(rng.uniform(-2, 2, n)), rng.uniform(-2, 2, n), np.exp(rng.uniform(-2, 2, n)),
                         rng.normal(0, 1, (n, 3))])
    R = np.column_stack([np.exp(rng.uniform(-2, 2, n)), rng.uniform(-2, 2, n), np.exp(rng.uniform(-2, 2, n)),
                         rng.normal(0, 1, (n, 3))])
    k = n // 6
    R[:k, :3] = L[:k, :3]
    L[k:2 * k, 1] = 3.0; R[k:2 * k, 1] = 3.3
    L[2 * k:3 * k, 1] = -1.8; R[2 * k:3 * k, 1] = 1.8
    return np.column_stack([np.full(n, G), L, R])


RUNS_2D = [
    # name, m, n, kind, bx, by, steps, split, seed
    ("fq_free", 17, 13, "fq", -4, -4, 40, 0, 7),
    ("shear_periodic", 16, 16, "sh", -7, -7, 40, 0, 7),
    ("fq_reflect_mixed", 20, 12, "fq", -2, -24, 40, 0, 5),
    ("fq_fixed", 15, 11, "fq", -1, -1, 30, 0, 3),
    ("fq_split", 17, 13, "fq", -4, -4, 30, 1, 7),
    ("shear_split", 16, 12, "sh", -7, -2, 30, 1, 2),
]


def g2d_inputs(rng, n):
    """Normal-frame pairs for the genuinely-2D solver: the flux mix above plus
    rarefaction/shock combinations on both sides of the contact (both
    rarefactions, t-axis right of the contact, sonic points) and tangential
    velocity jumps, which only this solver's uniform test sees."""
    q = flux_inputs(rng, n)[:, 2:]
    L, R = q[:, 1:13], q[:, 13:25]
    k = n // 8
    L[:k, 1] = -1.2; R[:k, 1] = 1.0                                  # two rarefactions, u* > 0 or < 0
    L[k:2 * k, 1] = -0.4; R[k:2 * k, 1] = -2.0                       # shocks and rarefactions, u* < 0
    L[2 * k:3 * k, 1] = 2.5; R[2 * k:3 * k, 1] = 0.5                 # left rarefaction sonic / shocks
    R[3 * k:4 * k, :4] = L[3 * k:4 * k, :4]
    R[3 * k:4 * k, 2] = L[3 * k:4 * k, 2] + 0.3                      # equal but for v: not uniform here
    return q


RUNS_2D_G2D = [
    # name, m, n, kind, bx, by, steps, split, seed
    ("fq_free", 17, 13, "fq", -4, -4, 30, 0, 7),
    ("shear_periodic", 16, 16, "sh", -7, -7, 30, 0, 7),
    ("fq_reflect_mixed", 20, 12, "fq", -2, -24, 30, 0, 5),
    ("fq_split", 17, 13, "fq", -4, -4, 25, 1, 7),
    ("shear_split", 16, 12, "sh", -7, -2, 25, 1, 2),
]


def make_g2d():
    R = orc.Oracle("reference_g2d")
    rng = np.random.default_rng(20261203)
    qin = g2d_inputs(rng, 1024)
    np.savez_compressed(os.path.join(HERE, "g2d.npz"), inp=qin, out=R.g2d(qin, 1e-9, 1e-9),
                        out_acoustic=R.g2d(qin, 1e-9, np.inf))
    runs = {}
    for name, m, n, kind, bx, by, steps, split, seed in RUNS_2D_G2D:
        gen = cases.four_quadrant if kind == "fq" else cases.shear_layer
        rho, u, v, p = gen(m, n, seed)
        cfg = orc.default_config_2d(t_all=-1, steps=steps, hx=1.0 / m, hy=1.0 / n, bx=bx, by=by, split=split)
        cfg[301] = 1  # the port's switch for the same solver; the reference ignores config[301]
        out = R.run_2d(rho, u, v, p, cfg, split=split)
        for key, val in (("in_rho", rho), ("in_u", u), ("in_v", v), ("in_p", p), ("cfg", cfg)):
            runs[f"{name}/{key}"] = val
        for f in ("rho", "u", "v", "p", "E"):
            runs[f"{name}/{f}"] = out[f]
        runs[f"{name}/meta"] = np.array([out["steps"], out["time"], split])
    np.savez_compressed(os.path.join(HERE, "runs_2d_g2d.npz"), **runs)


def lag_inputs(rng, n):
    """Lagrangian GRP pairs: rho, u, p and material derivatives per side;
    shocks, rarefactions and near-uniform (acoustic) pairs."""
    def side(k):
        return np.column_stack([np.exp(rng.uniform(-2, 2, k)), rng.uniform(-2, 2, k), np.exp(rng.uniform(-2, 2, k)),
                                rng.normal(0, 1, (k, 3))])
    L, R = side(n), side(n)
    k = n // 6
    R[:k, :3] = L[:k, :3]                                            # equal states: acoustic
    L[k:2 * k, 1] = 2.0; R[k:2 * k, 1] = -2.0                        # colliding: two shocks
    L[2 * k:3 * k, 1] = -1.5; R[2 * k:3 * k, 1] = 1.5                # receding: two rarefactions
    return np.column_stack([np.full(n, G), L, R])


def lag_runs():
    """Sod (400 cells, t = 0.2) with both Lagrangian schemes, and a smooth
    profile with a jump under every boundary code."""
    runs = []
    for order in (1, 2):
        rho, u, p = cases.sod(400)
        cfg = orc.default_config_1d(t_all=0.2, steps=100000, hx=1 / 400, bx=-4, cfl=0.45)
        runs.append((f"sod{order}", rho, u, p, cfg, order))
    m = 120
    x = (np.arange(m) + 0.5) / m
    rho = 1.0 + 0.5 * np.sin(2 * np.pi * x) + (x > 0.3) * 0.4
    u = 0.3 * np.cos(2 * np.pi * x)
    p = 1.0 + 0.2 * (x < 0.6)
    for bnd, order in ((-7, 2), (-2, 2), (-24, 1), (-1, 2), (-2, 1), (-24, 2)):
        cfg = orc.default_config_1d(t_all=0.1, steps=100000, hx=1 / m, bx=bnd, cfl=0.45)
        runs.append((f"bc{-bnd}o{order}", rho, u, p, cfg, order))
    # a fixed time step (config[16]) with a step count and no end time
    cfg = orc.default_config_1d(t_all=-1, steps=60, hx=1 / m, bx=-4, cfl=0.45)
    cfg[16] = 4e-4
    runs.append(("fixed_tau", rho, u, p, cfg, 2))
    return runs


def mf_inputs(rng, n):
    """Two-component interface pairs (rows of 40, the layout of the oracle's
    grp2d_flux_mf): the wave mix of g2d_inputs with a gamma per side, volume
    and mass fractions with random slopes, axis and oblique normals."""
    q = g2d_inputs(rng, n)
    L, R = q[:, 1:13], q[:, 13:25]

    def scal(k):
        return np.column_stack([rng.uniform(0, 1, k), rng.normal(0, 1, k), rng.normal(0, 1, k),
                                rng.uniform(0, 1, k), rng.normal(0, 1, k), rng.normal(0, 1, k)])
    gL = rng.uniform(1.1, 3.0, n)
    gR = rng.uniform(1.1, 3.0, n)
    k = n // 8
    gR[4 * k:5 * k] = gL[4 * k:5 * k]                                # one gamma on both sides
    th = rng.uniform(0, 2 * np.pi, n)
    normals = np.column_stack([np.cos(th), np.sin(th)])
    normals[: n // 4] = [1.0, 0.0]
    normals[n // 4: n // 2] = [0.0, 1.0]
    return np.column_stack([normals, gL, L, scal(n), gR, R, scal(n)])


MF_GAMMA_A, MF_GAMMA_B = 1.4, 3.0   # config[6], config[106]


def make_mf():
    R = orc.Oracle("reference_mf")
    rng = np.random.default_rng(20261205)
    inp = mf_inputs(rng, 1024)
    tau = 1e-3
    np.savez_compressed(os.path.join(HERE, "grp2d_flux_mf.npz"), inp=inp, tau=tau,
                        gamma_a=MF_GAMMA_A, gamma_b=MF_GAMMA_B,
                        out=R.grp2d_flux_mf(inp, tau, 1e-9, MF_GAMMA_A, MF_GAMMA_B, True),
                        out_nogamma=R.grp2d_flux_mf(inp, tau, 1e-9, MF_GAMMA_A, MF_GAMMA_B, False))


def make_lag():
    R = orc.Oracle("reference")
    rng = np.random.default_rng(20261204)
    lin = lag_inputs(rng, 1200)
    np.savez_compressed(os.path.join(HERE, "lag.npz"), inp=lin, out=R.lag(lin, 1e-9, 1e-9),
                        out_acoustic=R.lag(lin, 1e-9, np.inf))
    r1 = {}
    for name, rho, u, p, cfg, order in lag_runs():
        out = R.run_1d_lag(rho, u, p, cfg, order)
        r1[f"{name}/in"] = np.stack([rho, u, p])
        r1[f"{name}/cfg"] = cfg
        for f in ("rho", "u", "p", "E", "X"):
            r1[f"{name}/{f}"] = out[f]
        r1[f"{name}/meta"] = np.array([out["steps"], out["time"], order])
    np.savez_compressed(os.path.join(HERE, "runs_1d_lag.npz"), **r1)


def field_sha256(a: np.ndarray) -> str:
    """SHA-256 of a field's float64 values, little-endian, x-major (C order):
    the full-field identity of a run, checkable on any host."""
    return hashlib.sha256(np.ascontiguousarray(a, "<f8").tobytes()).hexdigest()


def make_large():
    """Summaries of the 1024^2 four-quadrant run (transmissive, CFL 0.45) after
    100 and 500 steps: step count and time, per field its SHA-256, sums, a 64 x 64
    subsample, one row and one column."""
    R = orc.Oracle("reference")
    m = n = 1024
    rho, u, v, p = cases.four_quadrant(m, n, seed=2024)
    for steps in (100, 500):
        cfg = orc.default_config_2d(t_all=-1, steps=steps, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4)
        out = R.run_2d(rho, u, v, p, cfg)
        summ = {"meta": np.array([out["steps"], out["time"], out["wall"]]), "cfg": cfg}
        for f in ("rho", "u", "v", "p", "E"):
            summ[f"sha256/{f}"] = np.array(field_sha256(out[f]))
            summ[f"abs_sum/{f}"] = np.abs(out[f]).sum()
            summ[f"sum/{f}"] = out[f].sum()
            summ[f"sub/{f}"] = out[f][::16, ::16].copy()
            summ[f"row/{f}"] = out[f][m // 2 + 3, :].copy()
            summ[f"col/{f}"] = out[f][:, n // 2 - 5].copy()
        np.savez_compressed(os.path.join(HERE, f"fq1024_{steps}.npz"), **summ)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--large", action="store_true")
    ap.add_argument("--only", choices=["all", "g2d", "lag", "mf", "large"], default="all")
    args = ap.parse_args()
    orc.build(ref=True)
    if args.only in ("all", "g2d"):
        make_g2d()
    if args.only in ("all", "lag"):
        make_lag()
    if args.only in ("all", "mf"):
        make_mf()
    if args.only == "large":
        make_large()
    if args.only != "all":
        print("fixtures written to", HERE)
        return
    R = orc.Oracle("reference")
    rng = np.random.default_rng(20241203)

    inp = riemann_inputs(rng, 2048)
    np.savez_compressed(os.path.join(HERE, "riemann_exact.npz"), inp=inp, out=R.riemann_exact(inp, 1e-9, 1e-9, 500),
                        out50=R.riemann_exact_ben(inp[:, [0, 2, 3, 4, 5, 6, 7]], 1e-9, 1e-9, 50))
    fin = flux_inputs(rng, 3072)
    np.savez_compressed(os.path.join(HERE, "grp2d_flux.npz"), inp=fin, tau=1e-3, out=R.grp2d_flux(fin, 1e-3))
    qin = fin[:, 2:]
    np.savez_compressed(os.path.join(HERE, "q1d.npz"), inp=qin, out=R.q1d(qin, 1e-9, 1e-9))
    gin = grp1d_inputs(rng, 2048)
    np.savez_compressed(os.path.join(HERE, "grp1d.npz"), inp=gin, out_grp=R.grp1d(gin, 1e-9, 1e-9),
                        out_acoustic=R.grp1d(gin, 1e-9, np.inf))

    runs = {}
    for name, m, n, kind, bx, by, steps, split, seed in RUNS_2D:
        gen = cases.four_quadrant if kind == "fq" else cases.shear_layer
        rho, u, v, p = gen(m, n, seed)
        cfg = orc.default_config_2d(t_all=-1, steps=steps, hx=1.0 / m, hy=1.0 / n, bx=bx, by=by, split=split)
        out = R.run_2d(rho, u, v, p, cfg, split=split)
        for key, val in (("in_rho", rho), ("in_u", u), ("in_v", v), ("in_p", p), ("cfg", cfg)):
            runs[f"{name}/{key}"] = val
        for f in ("rho", "u", "v", "p", "E"):
            runs[f"{name}/{f}"] = out[f]
        runs[f"{name}/meta"] = np.array([out["steps"], out["time"], split])
    # plot snapshots: time_plot with two plot times, 2D
    rho, u, v, p = cases.four_quadrant(18, 14, 9)
    cfg = orc.default_config_2d(t_all=0.08, steps=100000, hx=1 / 18, hy=1 / 14, bx=-4, by=-4)
    out = R.run_2d(rho, u, v, p, cfg, plot_times=[0.02, 0.05], want_snaps=True)
    runs["snap/in"] = np.stack([rho, u, v, p])
    runs["snap/cfg"] = cfg
    runs["snap/snaps"] = out["snaps"]
    runs["snap/meta"] = np.array([out["steps"], out["time"]])
    np.savez_compressed(os.path.join(HERE, "runs_2d.npz"), **runs)

    r1 = {}
    for order in (1, 2):
        rho, u, p = cases.sod(400)
        cfg = orc.default_config_1d(t_all=0.2, steps=100000, hx=1 / 400, bx=-4, cfl=0.45)
        out = R.run_1d(rho, u, p, cfg, order)
        for f in ("rho", "u", "p", "E"):
            r1[f"sod{order}/{f}"] = out[f]
        r1[f"sod{order}/meta"] = np.array([out["steps"], out["time"]])
        r1[f"sod{order}/cfg"] = cfg
    for bnd, order in ((-7, 2), (-2, 2), (-24, 1), (-1, 2)):
        m = 96
        x = (np.arange(m) + 0.5) / m
        rho = 1.0 + 0.5 * np.sin(2 * np.pi * x) + (x > 0.3) * 0.4
        u = 0.3 * np.cos(2 * np.pi * x)
        p = 1.0 + 0.2 * (x < 0.6)
        cfg = orc.default_config_1d(t_all=0.1, steps=100000, hx=1 / m, bx=bnd, cfl=0.5)
        out = R.run_1d(rho, u, p, cfg, order)
        name = f"bc{-bnd}o{order}"
        r1[f"{name}/in"] = np.stack([rho, u, p])
        r1[f"{name}/cfg"] = cfg
        for f in ("rho", "u", "p", "E"):
            r1[f"{name}/{f}"] = out[f]
        r1[f"{name}/meta"] = np.array([out["steps"], out["time"], order])
    np.savez_compressed(os.path.join(HERE, "runs_1d.npz"), **r1)

    if args.large:
        make_large()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
