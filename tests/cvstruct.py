"""ctypes mirror of the reference's struct cell_var_stru (src/include/var_struc.h:61-74)
and helpers that call the library's scheme entry points the way the reference's
drivers do (global config[], caller-owned x-major pointer arrays)."""
import ctypes

import numpy as np

PP = ctypes.POINTER(ctypes.POINTER(ctypes.c_double))
P = ctypes.POINTER(ctypes.c_double)

_FIELDS = [("E", PP), ("RHO", PP), ("U", PP), ("V", PP), ("P", PP),
           ("d_rho", P), ("d_u", P), ("d_v", P), ("d_p", P)]
for grp in ("s", "t"):
    _FIELDS += [(f"{grp}_{v}", PP) for v in ("rho", "u", "v", "p")]
_FIELDS += [(f"{v}I{ax}", PP) for ax in ("x", "y") for v in ("rho", "u", "v", "p")]
_FIELDS += [("F_rho", PP), ("F_e", PP), ("F_u", PP), ("F_v", PP), ("G_rho", PP), ("G_e", PP), ("G_u", PP), ("G_v", PP)]


class CellVarStru(ctypes.Structure):
    _fields_ = _FIELDS


def config_view(lib):
    """numpy view of the library's (weak) global config[400]."""
    addr = ctypes.addressof(ctypes.c_double.in_dll(lib, "config"))
    return np.ctypeslib.as_array((ctypes.c_double * 400).from_address(addr))


def _rows(arr2d, keep):
    """double** over the rows of a C-contiguous 2D array."""
    rows = (P * arr2d.shape[0])(*[arr2d[j].ctypes.data_as(P) for j in range(arr2d.shape[0])])
    keep.append(rows)
    return ctypes.cast(rows, PP)


def call_2d(lib, rho, u, v, p, gamma, cfg, split=False, plot_times=None, N_MAX=5):
    """Run GRP_solver_2D_[split_]EUL_source on x-major (m, n) arrays with the
    2D driver's set-up (src/hydrocode_2D/hydrocode.c:164-274).  Returns
    (slots[N_T, 5(rho,u,v,p,E), m, n], N_plot, time_plot, config[5])."""
    m, n = rho.shape
    ntp = 0 if plot_times is None else len(plot_times)
    N_plot = ntp + 2
    N_T = min(N_MAX, N_plot)
    time_plot = np.zeros(N_plot)
    time_plot[0] = 0.0
    time_plot[-1] = cfg[1]
    if ntp:
        time_plot[1:-1] = plot_times
    data = np.zeros((N_T, 5, m, n))
    data[0, 0], data[0, 1], data[0, 2], data[0, 3] = rho, u, v, p
    E = 0.5 * u * u + p / (gamma - 1.0) / rho
    E += 0.5 * v * v
    data[0, 4] = E
    keep = []
    cvs = (CellVarStru * N_T)()
    for k in range(N_T):
        cvs[k].RHO = _rows(data[k, 0], keep)
        cvs[k].U = _rows(data[k, 1], keep)
        cvs[k].V = _rows(data[k, 2], keep)
        cvs[k].P = _rows(data[k, 3], keep)
        cvs[k].E = _rows(data[k, 4], keep)
    conf = config_view(lib)
    conf[:] = cfg
    cpu_time = np.zeros(N_T)
    nplot = ctypes.c_int(N_plot)
    fn = lib.GRP_solver_2D_split_EUL_source if split else lib.GRP_solver_2D_EUL_source
    fn.restype = None
    fn(ctypes.c_int(m), ctypes.c_int(n), cvs, None, None, cpu_time.ctypes.data_as(P), ctypes.c_char_p(b"test"),
       ctypes.c_int(N_T), ctypes.byref(nplot), time_plot.ctypes.data_as(P))
    return data, nplot.value, time_plot, conf[5]


def call_1d(lib, rho, u, p, gamma, cfg, order, plot_times=None, N_MAX=1000):
    """Run Godunov_solver_EUL_source / GRP_solver_EUL_source with the 1D driver's
    set-up (src/hydrocode_1D/hydrocode.c:150-273)."""
    m = len(rho)
    ntp = 0 if plot_times is None else len(plot_times)
    N_plot = ntp + 2
    N = min(N_MAX, N_plot)
    time_plot = np.zeros(N_plot)
    time_plot[-1] = cfg[1]
    if ntp:
        time_plot[1:-1] = plot_times
    data = np.zeros((4, N, m))  # RHO, U, P, E slots
    data[0, 0], data[1, 0], data[2, 0] = rho, u, p
    data[3, 0] = 0.5 * u * u + p / (gamma - 1.0) / rho
    keep = []
    cv = CellVarStru()
    cv.RHO = _rows(data[0], keep)
    cv.U = _rows(data[1], keep)
    cv.P = _rows(data[2], keep)
    cv.E = _rows(data[3], keep)
    conf = config_view(lib)
    conf[:] = cfg
    cpu_time = np.zeros(N)
    nplot = ctypes.c_int(N)
    fn = lib.Godunov_solver_EUL_source if order == 1 else lib.GRP_solver_EUL_source
    fn.restype = None
    fn.argtypes = [ctypes.c_int, CellVarStru, P, ctypes.POINTER(ctypes.c_int), P]
    fn(m, cv, cpu_time.ctypes.data_as(P), ctypes.byref(nplot), time_plot.ctypes.data_as(P))
    return data, nplot.value, time_plot, conf[5]
