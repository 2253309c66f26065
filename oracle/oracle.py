"""TEST INFRASTRUCTURE ONLY: ctypes access to the oracle.

Two interchangeable back ends with identical entry points:

* ``port``      -- oracle/_build/libhydro_oracle.so, the C restatement in
                   hydro_oracle.c (built by ``make -C oracle port`` on any host);
* ``reference`` -- oracle/_ref/libhydro_ref.so, the reference's own sources
                   compiled by ``make -C oracle ref`` where the reference tree
                   exists (this is what pins the port).

Only tests/, the smoke test and bench.py's CPU-baseline leg use
this module; the product never imports it.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libhydro_oracle.so")
CRPOW_SO = os.path.join(HERE, "_build", "libhydro_oracle_crpow.so")
# the same with the FP64 device path's pow (the C library's method, libm_pow.cuh)
LPOW_SO = os.path.join(HERE, "_build", "libhydro_oracle_lpow.so")
REF_SO = os.path.join(HERE, "_ref", "libhydro_ref.so")
# the reference with GRP_2D_flux calling the genuinely-2D solver (oracle/Makefile)
REF_G2D_SO = os.path.join(HERE, "_ref", "libhydro_ref_g2d.so")
# GRP_2D_flux of the reference's two-component build (MULTIFLUID_BASICS)
REF_MF_SO = os.path.join(HERE, "_ref", "libhydro_ref_mf.so")
# The reference project's tree, from the HYDRO_REFERENCE environment variable;
# only needed to build REF_SO (and its variants).  Without it the tests that
# need the reference build skip, and the committed golden fixtures pin the port.
REF_TREE = os.environ.get("HYDRO_REFERENCE", "")
NCONF = 400

_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_int = ctypes.c_int
_dbl = ctypes.c_double


def reference_available() -> bool:
    return bool(REF_TREE) and os.path.isdir(os.path.join(REF_TREE, "src", "finite_volume"))


def build(ref: bool = False) -> None:
    """Compile the port (and the reference lib if asked and possible)."""
    targets = ["port"] + (["ref"] if ref and reference_available() else [])
    subprocess.run(["make", "-s", "-C", HERE, f"REF={REF_TREE}"] + targets, check=True)


def default_config_2d(**kw) -> np.ndarray:
    """config[] as the reference's config_check leaves it for a 2D Eulerian run
    (src/file_io/config_handle.c:39-152), with keyword overrides by name."""
    c = np.full(NCONF, np.inf)
    c[0] = 2
    c[2] = 1; c[8] = 0; c[30] = 0; c[31] = 0; c[32] = 1; c[33] = 0; c[40] = 0
    c[41] = 1.9; c[42] = 1; c[53] = 0; c[60] = 0; c[61] = 0; c[70] = 0
    c[110] = 0.72; c[210] = 0.0; c[211] = 0.0; c[212] = 0.0
    c[4] = 1e-9; c[6] = 1.4; c[7] = 0.45
    names = {"t_all": 1, "eps": 4, "steps": 5, "gamma": 6, "cfl": 7, "hx": 10, "hy": 11,
             "tau": 16, "bx": 17, "by": 18, "split": 33, "alpha": 41}
    for k, v in kw.items():
        c[names[k]] = v
    # config_check: a negative/absent total time with a step count means "run N steps"
    if not (math.isfinite(c[1]) and c[1] >= 0.0):
        c[1] = np.inf
    c[20] = c[10]
    return c


def default_config_1d(**kw) -> np.ndarray:
    c = default_config_2d(**kw)
    c[0] = 1
    if "cfl" not in kw:
        c[7] = 0.9
    return c


class Oracle:
    def __init__(self, which: str = "port"):
        """which: "port" (the C restatement), "crpow" (the same with a correctly
        rounded pow), "lpow" (the same with the device path's pow), "reference" (the reference's own sources) or
        "reference_g2d" (the same with GRP_2D_flux calling the genuinely-2D
        solver; the port selects it per run with config[301] = 1) or
        "reference_mf" (only the two-component interface flux, grp2d_flux_mf)."""
        path = {"port": PORT_SO, "crpow": CRPOW_SO, "lpow": LPOW_SO, "reference_g2d": REF_G2D_SO,
                "reference_mf": REF_MF_SO}.get(which, REF_SO)
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library missing: {path} (run make -C oracle)")
        self.which = which
        self.lib = ctypes.CDLL(path)
        p = "ref_" if which.startswith("reference") else "orc_"
        L = self.lib
        self._fluxmf = getattr(L, p + "grp2d_flux_mf", None)
        if self._fluxmf is not None:
            self._fluxmf.argtypes = [_int, _dp, _dbl, _dbl, _dbl, _dbl, _int, _dp]
        if which == "reference_mf":
            return
        self._run2d = getattr(L, p + "run_2d")
        self._run2d.argtypes = [_int, _int, _dp, _dp, _dp, _dp, _dp, _dp, _int, _int, _int,
                                ctypes.c_void_p, _int, ctypes.c_void_p, ctypes.POINTER(_int), _dp]
        self._run1d = getattr(L, p + "run_1d")
        self._run1d.argtypes = [_int, _dp, _dp, _dp, _dp, _dp, _int, _int, _dp]
        self._rex = getattr(L, p + "riemann_exact")
        self._rex.argtypes = [_int, _dp, _dbl, _dbl, _int, _dp]
        self._rexb = getattr(L, p + "riemann_exact_ben")
        self._rexb.argtypes = [_int, _dp, _dbl, _dbl, _int, _dp]
        self._flux = getattr(L, p + "grp2d_flux")
        self._flux.argtypes = [_int, _dp, _dbl, _dbl, _dp]
        self._q1d = getattr(L, p + "q1d")
        self._q1d.argtypes = [_int, _dp, _dbl, _dbl, _dp]
        self._run1dl = getattr(L, p + "run_1d_lag")
        self._run1dl.argtypes = [_int, _dp, _dp, _dp, _dp, _dp, _dp, _int, _int, _dp]
        self._lag = getattr(L, p + "lag")
        self._lag.argtypes = [_int, _dp, _dbl, _dbl, _dp]
        self._g2d = getattr(L, p + "g2d")
        self._g2d.argtypes = [_int, _dp, _dbl, _dbl, _dp]
        self._g1d = getattr(L, p + "grp1d")
        self._g1d.argtypes = [_int, _dp, _dbl, _dbl, _dp]
        if not which.startswith("reference"):
            self._rexi = L.orc_riemann_exact_iters
            self._rexi.argtypes = [_int, _dp, _dbl, _dbl, _int, _dp]

    # -- full runs -----------------------------------------------------------
    def run_2d(self, rho, u, v, p, cfg, split=False, threads=0, plot_times=None, want_snaps=False):
        """Run the 2D scheme. Arrays are x-major (m, n): value of cell (x=j, y=i) at [j, i].
        Returns dict(rho,u,v,p,E, steps=config[5] written back, time, cpu_time, wall[, snaps])."""
        rho = np.ascontiguousarray(rho, np.float64).copy()
        u = np.ascontiguousarray(u, np.float64).copy()
        v = np.ascontiguousarray(v, np.float64).copy()
        p = np.ascontiguousarray(p, np.float64).copy()
        m, n = rho.shape
        E = np.zeros_like(rho)
        info = np.zeros(4)
        cfg = np.ascontiguousarray(cfg, np.float64)
        pt = None if plot_times is None else np.ascontiguousarray(plot_times, np.float64)
        npt = 0 if pt is None else len(pt)
        nsnap = _int(0)
        snaps = np.zeros(((npt + 2) * 5, m, n)) if want_snaps else None
        self._run2d(m, n, rho, u, v, p, E, cfg, len(cfg), int(bool(split)), int(threads),
                    None if pt is None else pt.ctypes.data, npt,
                    None if snaps is None else snaps.ctypes.data, ctypes.byref(nsnap), info)
        out = dict(rho=rho, u=u, v=v, p=p, E=E, steps=info[0], time=info[1], cpu_time=info[2], wall=info[3])
        if want_snaps:
            out["snaps"] = snaps[: nsnap.value * 5].reshape(nsnap.value, 5, m, n)
        return out

    def run_1d(self, rho, u, p, cfg, order):
        rho = np.ascontiguousarray(rho, np.float64).copy()
        u = np.ascontiguousarray(u, np.float64).copy()
        p = np.ascontiguousarray(p, np.float64).copy()
        E = np.zeros_like(rho)
        info = np.zeros(4)
        cfg = np.ascontiguousarray(cfg, np.float64)
        self._run1d(len(rho), rho, u, p, E, cfg, len(cfg), int(order), info)
        return dict(rho=rho, u=u, p=p, E=E, steps=info[0], time=info[1], cpu_time=info[2], wall=info[3])

    # -- point solvers ---------------------------------------------------------
    def riemann_exact(self, inp, eps=1e-9, tol=1e-9, N=500):
        inp = np.ascontiguousarray(inp, np.float64)
        out = np.zeros((len(inp), 5))
        self._rex(len(inp), inp, eps, tol, N, out)
        return out

    def riemann_exact_iters(self, inp, eps=1e-9, tol=1e-9, N=500):
        inp = np.ascontiguousarray(inp, np.float64)
        out = np.zeros((len(inp), 6))
        self._rexi(len(inp), inp, eps, tol, N, out)
        return out

    def riemann_exact_ben(self, inp, eps=1e-9, tol=1e-9, N=50):
        inp = np.ascontiguousarray(inp, np.float64)
        out = np.zeros((len(inp), 5))
        self._rexb(len(inp), inp, eps, tol, N, out)
        return out

    def grp2d_flux(self, inp, tau, eps=1e-9):
        inp = np.ascontiguousarray(inp, np.float64)
        out = np.zeros((len(inp), 9))
        self._flux(len(inp), inp, tau, eps, out)
        return out

    def grp2d_flux_mf(self, inp, tau, eps=1e-9, gamma_a=1.4, gamma_b=1.4, store_gamma=True):
        """Two-component GRP_2D_flux on rows of 40 (n_x, n_y, then per side gamma,
        rho,u,v,p, d_rho,d_u,d_v,d_p, t_rho,t_u,t_v,t_p, z,d_z,t_z, phi,d_phi,t_phi);
        returns rows of 19 (F_rho,F_u,F_v,F_e, RHO_int,U_int,V_int,P_int, F_phi,
        F_gamma, F_e_a, PHI, Z_a, U_qt_add_c,V_qt_add_c, U_qt_star,V_qt_star,
        P_star, return code).  gamma_a/gamma_b/store_gamma: config[6]/[106]/[60]."""
        inp = np.ascontiguousarray(inp, np.float64)
        out = np.zeros((len(inp), 19))
        self._fluxmf(len(inp), inp, tau, eps, gamma_a, gamma_b, int(bool(store_gamma)), out)
        return out

    def q1d(self, inp, eps=1e-9, atc=1e-9):
        inp = np.ascontiguousarray(inp, np.float64)
        out = np.zeros((len(inp), 14))
        self._q1d(len(inp), inp, eps, atc, out)
        return out

    def run_1d_lag(self, rho, u, p, cfg, order):
        """1D Lagrangian run (order 1 Godunov, 2 GRP); returns the final state,
        the m+1 node coordinates and the step/time summary."""
        m = len(rho)
        r, uu, pp = (np.ascontiguousarray(a, np.float64).copy() for a in (rho, u, p))
        E = np.zeros(m)
        X = np.zeros(m + 1)
        info = np.zeros(4)
        cfg = np.ascontiguousarray(cfg, np.float64)
        self._run1dl(m, r, uu, pp, E, X, cfg, len(cfg), int(order), info)
        return {"rho": r, "u": uu, "p": pp, "E": E, "X": X, "steps": info[0], "time": info[1], "wall": info[3]}

    def lag(self, inp, eps=1e-9, atc=1e-9):
        """linear_GRP_solver_LAG on rows (gamma, left rho,u,p,t_rho,t_u,t_p, right the same)."""
        inp = np.ascontiguousarray(inp, np.float64)
        out = np.zeros((len(inp), 8))
        self._lag(len(inp), inp, eps, atc, out)
        return out

    def g2d(self, inp, eps=1e-9, atc=1e-9):
        """linear_GRP_solver_Edir_G2D on rows laid out as for q1d."""
        inp = np.ascontiguousarray(inp, np.float64)
        out = np.zeros((len(inp), 14))
        self._g2d(len(inp), inp, eps, atc, out)
        return out

    def grp1d(self, inp, eps=1e-9, atc=1e-9):
        inp = np.ascontiguousarray(inp, np.float64)
        out = np.zeros((len(inp), 6))
        self._g1d(len(inp), inp, eps, atc, out)
        return out
