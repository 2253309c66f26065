"""The C-ABI library loads and exports every function include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_declared_symbols():
    import hydro_gb300 as hg

    if not os.path.exists(hg.LIB_PATH):
        hg.build()
    lib = ctypes.CDLL(hg.LIB_PATH)
    names = declared_functions()
    for must in ("GRP_solver_2D_EUL_source", "GRP_solver_2D_split_EUL_source", "GRP_solver_EUL_source",
                 "Godunov_solver_EUL_source", "hydro2d_run"):
        assert must in names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # the configuration array the reference's drivers define is resolvable too
    ctypes.c_double.in_dll(lib, "config")


def test_face_flux_argument_checks_need_no_gpu():
    """hydro_grp2d_flux_mf validates its arguments before any CUDA call: a
    negative count is rejected (-2), an empty batch succeeds with nothing to
    report, missing arrays for a non-empty batch are rejected."""
    import numpy as np

    import hydro_gb300 as hg

    if not os.path.exists(hg.LIB_PATH):
        hg.build()
    # a private handle (RTLD_LOCAL): hg.lib() loads the library globally, and its
    # config[] would then stand in for the reference harness's own in later tests
    L = ctypes.CDLL(hg.LIB_PATH)
    L.hydro_grp2d_flux_mf.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int, ctypes.c_double, ctypes.POINTER(hg.FaceInfo)]
    L.hydro_grp2d_flux_mf.restype = ctypes.c_int
    cfg = np.full(400, np.inf)
    info = hg.FaceInfo()
    dummy = np.zeros(40)
    d, c = dummy.ctypes.data, cfg.ctypes.data
    assert L.hydro_grp2d_flux_mf(-1, d, d, None, c, len(cfg), 1e-3, ctypes.byref(info)) == -2
    assert L.hydro_grp2d_flux_mf(0, d, d, None, c, len(cfg), 1e-3, ctypes.byref(info)) == 0
    assert info.n_bad == 0 and info.first_bad == -1
    assert L.hydro_grp2d_flux_mf(5, d, d, None, c, len(cfg), 1e-3, ctypes.byref(info)) == -2
