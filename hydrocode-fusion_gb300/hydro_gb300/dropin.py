"""The reference-facing call from Python: a ctypes mirror of the reference's
struct cell_var_stru (src/include/var_struc.h:61-74) and helpers that call the
library's scheme entry points the way the reference's drivers do (global
config[], caller-owned x-major pointer arrays of host memory)."""
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


class Call2D:
    """Host arrays and arguments of one GRP_solver_2D_[split_]EUL_source call,
    set up as the 2D driver does (src/hydrocode_2D/hydrocode.c:164-274);
    call() runs the scheme (host buffers in and out, as a C caller has them)."""

    def __init__(self, lib, rho, u, v, p, gamma, cfg, split=False, plot_times=None, N_MAX=5):
        m, n = rho.shape
        self.lib, self.m, self.n, self.split = lib, m, n, split
        self.cfg = np.array(cfg, np.float64)
        ntp = 0 if plot_times is None else len(plot_times)
        self.N_plot0 = ntp + 2
        self.N_T = min(N_MAX, self.N_plot0)
        self.time_plot = np.zeros(self.N_plot0)
        self.time_plot[-1] = cfg[1]
        if ntp:
            self.time_plot[1:-1] = plot_times
        self._time_plot0 = self.time_plot.copy()
        self.data = np.zeros((self.N_T, 5, m, n))
        d0 = self.data[0]
        d0[0], d0[1], d0[2], d0[3] = rho, u, v, p
        E = 0.5 * u * u + p / (gamma - 1.0) / rho
        E += 0.5 * v * v
        d0[4] = E
        self._keep = []
        self.cvs = (CellVarStru * self.N_T)()
        for k in range(self.N_T):
            for idx, name in enumerate(("RHO", "U", "V", "P", "E")):
                setattr(self.cvs[k], name, _rows(self.data[k, idx], self._keep))
        self.cpu_time = np.zeros(self.N_T)

    def call(self):
        """Runs the scheme from the initial data in CV[0]; repeatable (the plot
        times, which the call overwrites with the times reached, are reset)."""
        conf = config_view(self.lib)
        conf[:] = self.cfg
        self.time_plot[:] = self._time_plot0
        nplot = ctypes.c_int(self.N_plot0)
        fn = self.lib.GRP_solver_2D_split_EUL_source if self.split else self.lib.GRP_solver_2D_EUL_source
        fn.restype = None
        fn(ctypes.c_int(self.m), ctypes.c_int(self.n), self.cvs, None, None, self.cpu_time.ctypes.data_as(P),
           ctypes.c_char_p(b"run"), ctypes.c_int(self.N_T), ctypes.byref(nplot), self.time_plot.ctypes.data_as(P))
        return nplot.value, conf[5]


def call_2d(lib, rho, u, v, p, gamma, cfg, split=False, plot_times=None, N_MAX=5):
    """Run GRP_solver_2D_[split_]EUL_source on x-major (m, n) arrays.  Returns
    (slots[N_T, 5(rho,u,v,p,E), m, n], N_plot, time_plot, config[5])."""
    c = Call2D(lib, rho, u, v, p, gamma, cfg, split, plot_times, N_MAX)
    nplot, k_out = c.call()
    return c.data, nplot, c.time_plot, k_out


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


def call_1d_lag(lib, rho, u, p, gamma, cfg, order, plot_times=None, N_MAX=1000):
    """Run Godunov_solver_LAG_source / GRP_solver_LAG_source with the 1D driver's
    set-up for "LAG" (src/hydrocode_1D/hydrocode.c:196-247: X[0][j] = j h,
    config[8] = 1).  Returns (CV data [4][N][m], node slots X [N][m+1], N_plot,
    time_plot, config[5])."""
    m = len(rho)
    ntp = 0 if plot_times is None else len(plot_times)
    N_plot = ntp + 2
    N = min(N_MAX, N_plot)
    time_plot = np.zeros(N_plot)
    time_plot[-1] = cfg[1]
    if ntp:
        time_plot[1:-1] = plot_times
    data = np.zeros((4, N, m))
    data[0, 0], data[1, 0], data[2, 0] = rho, u, p
    data[3, 0] = 0.5 * u * u + p / (gamma - 1.0) / rho
    X = np.zeros((N, m + 1))
    X[0] = cfg[10] * np.arange(m + 1)
    keep = []
    cv = CellVarStru()
    cv.RHO = _rows(data[0], keep)
    cv.U = _rows(data[1], keep)
    cv.P = _rows(data[2], keep)
    cv.E = _rows(data[3], keep)
    xrows = _rows(X, keep)
    conf = config_view(lib)
    conf[:] = cfg
    conf[8] = 1.0
    cpu_time = np.zeros(N)
    nplot = ctypes.c_int(N)
    fn = lib.Godunov_solver_LAG_source if order == 1 else lib.GRP_solver_LAG_source
    fn.restype = None
    fn.argtypes = [ctypes.c_int, CellVarStru, ctypes.c_void_p, P, ctypes.POINTER(ctypes.c_int), P]
    fn(m, cv, ctypes.cast(xrows, ctypes.c_void_p), cpu_time.ctypes.data_as(P), ctypes.byref(nplot),
       time_plot.ctypes.data_as(P))
    return data, X, nplot.value, time_plot, conf[5]

