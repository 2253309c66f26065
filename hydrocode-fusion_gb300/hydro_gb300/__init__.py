"""Python access to libhydro_gb300.so (ctypes over the C ABI in include/hydro_gb300.h).

The library is the product: GB300 (sm_103a) kernels behind the reference's
scheme entry points.  This module only loads it and moves numpy arrays across
the C ABI; there is no Python or CPU fallback -- a missing or unloadable
library raises immediately.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libhydro_gb300.so")
NCONF = 400

FORM_FP64 = 0
FORM_FP32 = 1
FORM_FP32_LEARNED = 2
# interface GRP solver of the 2D schemes (config[301], HYDRO_SOLVER_*)
SOLVER_Q1D = 0
SOLVER_G2D = 1

_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
MLP_NPARAM = 4673
WEIGHTS_PATH = os.path.join(PKG_DIR, "weights", "riemann_guess_6_64_64_1.f32")


class RunInfo(ctypes.Structure):
    _fields_ = [
        ("k_out", ctypes.c_int),
        ("steps_done", ctypes.c_int),
        ("sweeps_launched", ctypes.c_int),
        ("halted", ctypes.c_int),
        ("error_code_x", ctypes.c_int),
        ("error_code_y", ctypes.c_int),
        ("time", ctypes.c_double),
        ("tau", ctypes.c_double),
        ("gpu_ms", ctypes.c_double),
        ("newton_faces", ctypes.c_ulonglong),
        ("newton_iters", ctypes.c_ulonglong),
        ("newton_fallbacks", ctypes.c_ulonglong),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class BatchInfo(ctypes.Structure):
    _fields_ = [
        ("gpu_ms", ctypes.c_double),
        ("shape", ctypes.c_int),
        ("schedule", ctypes.c_int),
        ("graphed", ctypes.c_int),
        ("steps", ctypes.c_int),
        ("tiles", ctypes.c_int),
        ("halted_problems", ctypes.c_int),
        ("newton_faces", ctypes.c_ulonglong),
        ("newton_iters", ctypes.c_ulonglong),
        ("newton_fallbacks", ctypes.c_ulonglong),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class FaceInfo(ctypes.Structure):
    """hydro_face_info: outcome of one hydro_grp2d_flux_mf call."""
    _fields_ = [
        ("n_bad", ctypes.c_int),
        ("first_bad", ctypes.c_int),
        ("first_code", ctypes.c_int),
        ("resumed", ctypes.c_int * 4),
        ("kernel_ms", ctypes.c_double),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


SCHEDULES = ("persistent-static", "persistent-static-largest-first", "persistent-dynamic",
             "persistent-dynamic-largest-first", "graph-per-step")


def build(jobs: int = 4) -> str:
    """Compile the library in-tree (nvcc, sm_103a) and return its path."""
    subprocess.run(["make", "-s", "-j", str(jobs), "-C", PKG_DIR], check=True)
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    """Load the library once; raise if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libhydro_gb300.so not built: {LIB_PATH} (run make -C {PKG_DIR})")
    L = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
    L.hydro2d_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.hydro2d_create.restype = ctypes.c_int
    L.hydro2d_create_ex.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int]
    L.hydro2d_create_ex.restype = ctypes.c_int
    L.hydro2d_destroy.argtypes = [ctypes.c_void_p]
    L.hydro2d_destroy.restype = None
    L.hydro2d_upload.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, ctypes.c_void_p, ctypes.c_double]
    L.hydro2d_upload.restype = ctypes.c_int
    L.hydro2d_download.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp]
    L.hydro2d_download.restype = ctypes.c_int
    L.hydro2d_run.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(RunInfo)]
    L.hydro2d_run.restype = ctypes.c_int
    L.hydro2d_num_variants.argtypes = [ctypes.c_void_p]
    L.hydro2d_set_variant.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.hydro2d_get_variant.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
    L.hydro2d_autotune.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
    L.hydro2d_set_mlp.argtypes = [ctypes.c_void_p, _fp]
    L.hydro2d_conservation.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _dp]
    vp = ctypes.c_void_p
    L.hydro_mlp_create.argtypes = [ctypes.POINTER(vp), ctypes.c_ulonglong]
    L.hydro_mlp_destroy.argtypes = [vp]
    L.hydro_mlp_destroy.restype = None
    L.hydro_mlp_get_params.argtypes = [vp, _fp]
    L.hydro_mlp_set_params.argtypes = [vp, _fp]
    L.hydro_mlp_generate.argtypes = [vp, ctypes.c_longlong, ctypes.c_ulonglong, ctypes.c_double, ctypes.c_void_p]
    L.hydro_mlp_get_data.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]
    L.hydro_mlp_train.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_longlong, ctypes.c_void_p]
    L.hydro_mlp_gradient.argtypes = [vp, _fp, _fp, ctypes.c_int, _fp, ctypes.POINTER(ctypes.c_float)]
    L.hydro_mlp_predict.argtypes = [vp, _fp, ctypes.c_int, _fp]
    L.hydro_mlp_features.argtypes = [_dp, ctypes.c_int, ctypes.c_double, _fp]
    L.hydro_batch_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.hydro_batch_destroy.argtypes = [vp]
    L.hydro_batch_destroy.restype = None
    L.hydro_batch_upload.argtypes = [vp, ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_void_p, ctypes.c_double]
    L.hydro_batch_download.argtypes = [vp, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]
    L.hydro_batch_run.argtypes = [vp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(BatchInfo)]
    L.hydro_batch_shape.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.hydro_batch_set_schedule.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.hydro_batch_set_wait_limit.argtypes = [vp, ctypes.c_double]
    L.hydro_batch_autotune.argtypes = [vp, _dp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
    L.hydro_batch_problem_info.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    L.hydro_grp2d_flux_mf.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double,
                                      ctypes.POINTER(FaceInfo)]
    L.hydro_grp2d_flux_mf.restype = ctypes.c_int
    L.hydro_gb300_last_error.restype = ctypes.c_char_p
    L.hydro_gb300_kernel_launches.restype = ctypes.c_ulonglong
    _lib = L
    return L


def last_error() -> str:
    return lib().hydro_gb300_last_error().decode()


def kernel_launches() -> int:
    return int(lib().hydro_gb300_kernel_launches())


def config_2d(**kw) -> np.ndarray:
    """config[] for a 2D Eulerian run as the reference's config_check leaves it
    (src/file_io/config_handle.c:39-152); keyword overrides by name."""
    c = np.full(NCONF, np.inf)
    c[0] = 2
    c[2] = 1; c[8] = 0; c[30] = 0; c[31] = 0; c[32] = 1; c[33] = 0; c[40] = 0
    c[41] = 1.9; c[42] = 1; c[53] = 0; c[60] = 0; c[61] = 0; c[70] = 0
    c[110] = 0.72; c[210] = 0.0; c[211] = 0.0; c[212] = 0.0
    c[4] = 1e-9; c[6] = 1.4; c[7] = 0.45
    names = {"t_all": 1, "eps": 4, "steps": 5, "gamma": 6, "cfl": 7, "hx": 10, "hy": 11,
             "tau": 16, "bx": 17, "by": 18, "split": 33, "alpha": 41, "form": 300, "solver": 301}
    for k, v in kw.items():
        c[names[k]] = v
    if not (math.isfinite(c[1]) and c[1] >= 0.0):
        c[1] = np.inf
    c[20] = c[10]
    return c


def config_1d(**kw) -> np.ndarray:
    c = config_2d(**kw)
    c[0] = 1
    if "cfl" not in kw:
        c[7] = 0.9
    return c


class Solver2D:
    """Device-resident 2D solver (hydro2d_* in the C ABI).

    Arrays are x-major numpy arrays of shape (m, n): value of cell (x=j, y=i) at [j, i].
    """

    def __init__(self, m: int, n: int, form: int = FORM_FP64, solver: int = SOLVER_Q1D):
        self.m, self.n, self.form, self.solver = m, n, form, solver
        h = ctypes.c_void_p()
        if lib().hydro2d_create_ex(ctypes.byref(h), m, n, form, solver) != 0:
            raise RuntimeError("hydro2d_create failed: " + last_error())
        self._h = h

    def close(self):
        if self._h:
            lib().hydro2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, rho, u, v, p, E=None, gamma=1.4):
        arrs = [np.ascontiguousarray(a, np.float64) for a in (rho, u, v, p)]
        for a in arrs:
            assert a.shape == (self.m, self.n)
        e = None if E is None else np.ascontiguousarray(E, np.float64)
        rc = lib().hydro2d_upload(self._h, *arrs, None if e is None else e.ctypes.data, gamma)
        if rc != 0:
            raise RuntimeError("upload failed: " + last_error())

    def download(self):
        out = [np.empty((self.m, self.n)) for _ in range(5)]
        if lib().hydro2d_download(self._h, *out) != 0:
            raise RuntimeError("download failed: " + last_error())
        return dict(zip(("rho", "u", "v", "p", "E"), out))

    def num_variants(self) -> int:
        return int(lib().hydro2d_num_variants(self._h))

    def set_variant(self, v: int):
        if lib().hydro2d_set_variant(self._h, int(v)) != 0:
            raise RuntimeError(last_error())

    def variant(self):
        shape = (ctypes.c_int * 5)()
        v = lib().hydro2d_get_variant(self._h, shape)
        kind = {0: "tile", 1: "tma", 2: "tma", 3: "strip"}[int(shape[4])]
        return int(v), {"tile_x": shape[0], "tile_y": shape[1], "threads": shape[2], "min_ctas_per_sm": shape[3],
                        "kernel": kind, "tma": kind == "tma", "tma_stages": int(shape[4]) if kind == "tma" else 0}

    def autotune(self, cfg, steps=3):
        """Time every kernel variant on `steps` steps of the uploaded state (restored
        afterwards); keep the fastest. Returns (best index, per-variant ms)."""
        cfg = np.ascontiguousarray(cfg, np.float64)
        nv = self.num_variants()
        times = (ctypes.c_float * nv)()
        best = lib().hydro2d_autotune(self._h, cfg, len(cfg), int(steps), times)
        if best < 0:
            raise RuntimeError("autotune failed: " + last_error())
        return int(best), [float(t) for t in times]

    def set_mlp(self, params):
        if lib().hydro2d_set_mlp(self._h, np.ascontiguousarray(params, np.float32)) != 0:
            raise RuntimeError(last_error())

    def conservation(self, hx=None, hy=None):
        """FP64 integrals of mass, x/y momentum and energy of the current state."""
        hx = 1.0 / self.m if hx is None else hx
        hy = 1.0 / self.n if hy is None else hy
        out = np.zeros(4)
        if lib().hydro2d_conservation(self._h, hx, hy, out) != 0:
            raise RuntimeError(last_error())
        return dict(zip(("mass", "mom_x", "mom_y", "energy"), out.tolist()))

    def run(self, cfg, split=False, stats=False) -> RunInfo:
        cfg = np.ascontiguousarray(cfg, np.float64)
        info = RunInfo()
        if lib().hydro2d_run(self._h, cfg, len(cfg), int(bool(split)), int(bool(stats)), ctypes.byref(info)) != 0:
            raise RuntimeError("run failed: " + last_error())
        return info


def run_2d(rho, u, v, p, cfg, split=False, form=FORM_FP64, stats=False, mlp=None, solver=SOLVER_Q1D):
    """Upload, run, download; returns (state dict, RunInfo).  The learned form
    uses `mlp` (a parameter vector) or the shipped trained weights; `solver`
    picks the interface GRP solver (SOLVER_Q1D or SOLVER_G2D)."""
    m, n = np.shape(rho)
    s = Solver2D(m, n, form, solver)
    try:
        if form == FORM_FP32_LEARNED:
            s.set_mlp(load_weights() if mlp is None else mlp)
        s.upload(rho, u, v, p, None, float(cfg[6]))
        info = s.run(cfg, split=split, stats=stats)
        return s.download(), info
    finally:
        s.close()


# Field order of the two-component face batch (hydro_grp2d_flux_mf).
MF_SIDE_FIELDS = ("gamma", "rho", "u", "v", "p", "d_rho", "d_u", "d_v", "d_p", "t_rho", "t_u", "t_v", "t_p",
                  "z", "d_z", "t_z", "phi", "d_phi", "t_phi")
MF_OUT_FIELDS = ("F_rho", "F_u", "F_v", "F_e", "RHO_int", "U_int", "V_int", "P_int", "F_phi", "F_gamma", "F_e_a",
                 "PHI", "Z_a", "U_qt_add_c", "V_qt_add_c", "U_qt_star", "V_qt_star", "P_star")


def grp2d_flux_mf(fields, tau, cfg, out=None, status=None):
    """Two-component GRP_2D_flux for a batch of faces on the GPU.
    fields: (40, nface) float64 -- n_x, n_y, then MF_SIDE_FIELDS for the left
    and the right side.  cfg: config[] (4 eps, 6 / 106 the two gammas, 60
    store F_gamma).  out (18, nface) float64 and status (nface,) int32 may be
    given to be filled (a caller that flushes batches repeatedly keeps them).
    Returns (out in MF_OUT_FIELDS order, status, FaceInfo)."""
    fields = np.ascontiguousarray(fields, np.float64)
    if fields.ndim != 2 or fields.shape[0] != 40:
        raise ValueError("fields must have shape (40, nface)")
    nface = fields.shape[1]
    if out is None:
        out = np.zeros((18, nface))
    if status is None:
        status = np.zeros(nface, np.int32)
    if out.shape != (18, nface) or out.dtype != np.float64 or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous float64 array of shape (18, nface)")
    if status.shape != (nface,) or status.dtype != np.int32 or not status.flags.c_contiguous:
        raise ValueError("status must be a C-contiguous int32 array of shape (nface,)")
    cfg = np.ascontiguousarray(cfg, np.float64)
    info = FaceInfo()
    rc = lib().hydro_grp2d_flux_mf(nface, fields, out, status.ctypes.data_as(ctypes.c_void_p), cfg, len(cfg),
                                   float(tau), ctypes.byref(info))
    if rc != 0:
        raise RuntimeError("hydro_grp2d_flux_mf failed: " + last_error())
    return out, status, info


class Mlp:
    """The learned Newton starting pressure network (hydro_mlp_* in the C ABI)."""

    def __init__(self, seed: int = 1):
        h = ctypes.c_void_p()
        if lib().hydro_mlp_create(ctypes.byref(h), seed) != 0:
            raise RuntimeError("hydro_mlp_create failed: " + last_error())
        self._h = h

    def close(self):
        if self._h:
            lib().hydro_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.zeros(MLP_NPARAM, np.float32)
        if lib().hydro_mlp_get_params(self._h, p) != 0:
            raise RuntimeError(last_error())
        return p

    def set_params(self, p):
        if lib().hydro_mlp_set_params(self._h, np.ascontiguousarray(p, np.float32)) != 0:
            raise RuntimeError(last_error())

    def generate(self, n: int, seed: int = 7, gamma: float = 1.4, want_raw: bool = False):
        raw = np.zeros((n, 6)) if want_raw else None
        if lib().hydro_mlp_generate(self._h, n, seed, gamma, None if raw is None else raw.ctypes.data) != 0:
            raise RuntimeError(last_error())
        return raw

    def data(self, n: int):
        X = np.zeros((n, 6), np.float32)
        Y = np.zeros(n, np.float32)
        if lib().hydro_mlp_get_data(self._h, X.ctypes.data, Y.ctypes.data, n) != 0:
            raise RuntimeError(last_error())
        return X, Y

    def train(self, epochs: int, batch: int = 8192, lr: float = 3e-3, holdout: int = 0):
        losses = np.zeros(epochs, np.float32)
        if lib().hydro_mlp_train(self._h, epochs, batch, lr, holdout, losses.ctypes.data) != 0:
            raise RuntimeError(last_error())
        return losses

    def gradient(self, X, Y):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        g = np.zeros(MLP_NPARAM, np.float32)
        loss = ctypes.c_float()
        if lib().hydro_mlp_gradient(self._h, X, Y, len(Y), g, ctypes.byref(loss)) != 0:
            raise RuntimeError(last_error())
        return g, float(loss.value)

    def predict(self, X):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros(len(X), np.float32)
        if lib().hydro_mlp_predict(self._h, X, len(X), Y) != 0:
            raise RuntimeError(last_error())
        return Y


def features(states, gamma=1.4):
    """Device feature map of rows (rhoL, uL, pL, rhoR, uR, pR)."""
    states = np.ascontiguousarray(states, np.float64)
    X = np.zeros((len(states), 6), np.float32)
    if lib().hydro_mlp_features(states, len(states), gamma, X) != 0:
        raise RuntimeError(last_error())
    return X


def fp64_peak() -> float:
    """Measured FP64 fused multiply-add rate of the current GPU (DFMA/s)."""
    v = ctypes.c_double()
    L = lib()
    L.hydro_fp64_peak.restype = ctypes.c_int
    if L.hydro_fp64_peak(ctypes.byref(v)) != 0:
        raise RuntimeError("hydro_fp64_peak failed: " + last_error())
    return float(v.value)


LEARNED_COST_KEYS = ("network_ns_per_face", "solve_ns_per_face_reference_start", "iters_reference_start",
                     "solve_ns_per_face_learned_start", "iters_learned_start", "ns_per_newton_iteration",
                     "grp_derivatives_ns_per_face", "exact_face_ns_per_face", "solve_ns_per_face_fp32_start",
                     "iters_fp32_start")


def learned_costs(params=None, nfaces: int = 1 << 20, seed: int = 7, gamma: float = 1.4) -> dict:
    """What the learned start costs and saves per face in the FP32 form's device
    code (hydro_learned_costs): the network pass, the exact solve from the
    reference's, the network's and the FP32 form's own start with their
    iterations, one Newton iteration, the GRP derivatives."""
    prm = np.ascontiguousarray(load_weights() if params is None else params, np.float32)
    out = (ctypes.c_double * len(LEARNED_COST_KEYS))()
    L = lib()
    L.hydro_learned_costs.restype = ctypes.c_int
    L.hydro_learned_costs.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_ulonglong,
                                      ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    if L.hydro_learned_costs(prm.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), int(nfaces), int(seed),
                             float(gamma), out) != 0:
        raise RuntimeError("hydro_learned_costs failed: " + last_error())
    return dict(zip(LEARNED_COST_KEYS, (float(v) for v in out)))


def load_weights(path: str = WEIGHTS_PATH) -> np.ndarray:
    w = np.fromfile(path, dtype="<f4")
    if w.size != MLP_NPARAM:
        raise ValueError(f"{path}: {w.size} values, expected {MLP_NPARAM}")
    return w


class Batch:
    """Many independent 2D problems of uneven size, advanced together in the
    FP32 form (hydro_batch_* in the C ABI).  sizes: list of (m, n)."""

    def __init__(self, sizes):
        self.sizes = [(int(m), int(n)) for m, n in sizes]
        ms = (ctypes.c_int * len(self.sizes))(*[m for m, _ in self.sizes])
        ns = (ctypes.c_int * len(self.sizes))(*[n for _, n in self.sizes])
        h = ctypes.c_void_p()
        if lib().hydro_batch_create(ctypes.byref(h), len(self.sizes), ms, ns) != 0:
            raise RuntimeError("hydro_batch_create failed: " + last_error())
        self._h = h

    def close(self):
        if self._h:
            lib().hydro_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, p, rho, u, v, pr, gamma=1.4):
        arrs = [np.ascontiguousarray(a, np.float64) for a in (rho, u, v, pr)]
        for a in arrs:
            assert a.shape == self.sizes[p]
        if lib().hydro_batch_upload(self._h, p, *arrs, None, gamma) != 0:
            raise RuntimeError("batch upload failed: " + last_error())

    def download(self, p):
        out = [np.empty(self.sizes[p]) for _ in range(5)]
        if lib().hydro_batch_download(self._h, p, *out) != 0:
            raise RuntimeError("batch download failed: " + last_error())
        return dict(zip(("rho", "u", "v", "p", "E"), out))

    def set_schedule(self, shape, schedule):
        if lib().hydro_batch_set_schedule(self._h, int(shape), int(schedule)) != 0:
            raise RuntimeError(last_error())

    def set_wait_limit(self, seconds):
        if lib().hydro_batch_set_wait_limit(self._h, float(seconds)) != 0:
            raise RuntimeError(last_error())

    @staticmethod
    def shapes():
        out = []
        for k in range(lib().hydro_batch_num_shapes()):
            s = (ctypes.c_int * 4)()
            lib().hydro_batch_shape(k, s)
            out.append({"tile_x": s[0], "tile_y": s[1], "threads": s[2], "min_ctas_per_sm": s[3],
                        "kind": "strip" if lib().hydro_batch_shape_kind(k) == 1 else "tile"})
        return out

    def autotune(self, cfg, steps=3):
        cfg = np.ascontiguousarray(cfg, np.float64)
        nsh, nsc = lib().hydro_batch_num_shapes(), lib().hydro_batch_num_schedules()
        times = (ctypes.c_float * (nsh * nsc))()
        best = lib().hydro_batch_autotune(self._h, cfg, len(cfg), int(steps), times)
        if best < 0:
            raise RuntimeError("batch autotune failed: " + last_error())
        return int(best), np.array(list(times), np.float64).reshape(nsh, nsc)

    def run(self, cfg, steps, stats=False) -> BatchInfo:
        cfg = np.ascontiguousarray(cfg, np.float64)
        info = BatchInfo()
        rc = lib().hydro_batch_run(self._h, cfg, len(cfg), int(steps), int(bool(stats)), ctypes.byref(info))
        if rc != 0:
            raise RuntimeError(f"batch run failed ({rc}): " + last_error())
        return info

    def problem_info(self, p):
        k, s, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        if lib().hydro_batch_problem_info(self._h, p, ctypes.byref(k), ctypes.byref(s), ctypes.byref(t)) != 0:
            raise RuntimeError(last_error())
        return {"halted": k.value, "halted_step": s.value, "tau": t.value}
