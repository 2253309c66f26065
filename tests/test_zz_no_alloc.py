"""The allocation-free 1D entry point (hydro1d_run_noalloc).

It serves callers that cannot allocate device memory (a framework whose own
allocator owns the device pool, a driver with a fixed memory budget): its
scratch is a fixed static device array.  The test plays such a caller -- the state buffers
are allocated here, by the test, and only their device addresses cross the C
ABI -- and checks that two calls in a row give the same results as the
allocating entry point hydro1d_run, at the parity tolerance of the other tests,
then that an over-size grid is rejected with an error instead of running.
This file is named so that pytest collects it last."""
import ctypes

import numpy as np
import pytest

TOL = 1e-12
P = ctypes.POINTER(ctypes.c_double)


def _rel_l1(a, b):
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def _reference_entry(hg, rho, u, p, E, cfg, order):
    L = hg.lib()
    L.hydro1d_run.restype = ctypes.c_int
    out = [np.array(a, np.float64) for a in (rho, u, p, E)]
    info = hg.RunInfo()
    c = np.ascontiguousarray(cfg, np.float64)
    rc = L.hydro1d_run(len(rho), *[a.ctypes.data_as(P) for a in out], c.ctypes.data_as(P), len(c), order,
                       ctypes.byref(info))
    assert rc == 0, hg.last_error()
    return out, info


def _noalloc_entry(hg, torch, rho, u, p, E, cfg, order):
    L = hg.lib()
    L.hydro1d_run_noalloc.restype = ctypes.c_int
    L.hydro1d_run_noalloc.argtypes = [ctypes.c_int, ctypes.c_void_p, P, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.POINTER(hg.RunInfo)]
    state = torch.tensor(np.stack([rho, u, p, E]), dtype=torch.float64, device="cuda")
    c = np.ascontiguousarray(cfg, np.float64)
    info = hg.RunInfo()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.hydro1d_run_noalloc(len(rho), state.data_ptr(), c.ctypes.data_as(P), len(c), order, stream,
                               ctypes.byref(info))
    assert rc == 0, hg.last_error()
    torch.cuda.synchronize()
    return [x for x in state.cpu().numpy()], info


def _case(kind, m):
    rng = np.random.default_rng(m)
    if kind == "sod":
        x = (np.arange(m) + 0.5) / m
        rho, u, p = np.where(x < 0.5, 1.0, 0.125), np.zeros(m), np.where(x < 0.5, 1.0, 0.1)
    else:
        rho, u, p = rng.uniform(0.2, 2, m), rng.uniform(-1, 1, m), rng.uniform(0.2, 2, m)
    E = 0.5 * u * u + p / 0.4 / rho
    return rho, u, p, E


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_twice(gpu_lib):
    import torch

    hg = gpu_lib
    # two different problems in a row: the second call reuses the scratch the first one left behind
    runs = [("sod", 400, 2, -4, 0.2), ("random", 3000, 1, -7, 0.02)]
    for kind, m, order, bnd, t_all in runs:
        rho, u, p, E = _case(kind, m)
        cfg = hg.config_1d(t_all=t_all, steps=100000, hx=1.0 / m, bx=bnd, cfl=0.45)
        want, iw = _reference_entry(hg, rho, u, p, E, cfg, order)
        got, ig = _noalloc_entry(hg, torch, rho, u, p, E, cfg, order)
        assert ig.k_out == iw.k_out and ig.time == iw.time and ig.halted == iw.halted
        for a, b in zip(got, want):
            assert _rel_l1(a, b) <= TOL


@pytest.mark.gpu
def test_noalloc_rejects_oversize_grid(gpu_lib):
    import torch

    hg = gpu_lib
    m = 16385
    L = hg.lib()
    L.hydro1d_run_noalloc.restype = ctypes.c_int
    L.hydro1d_run_noalloc.argtypes = [ctypes.c_int, ctypes.c_void_p, P, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.POINTER(hg.RunInfo)]
    state = torch.ones((4, m), dtype=torch.float64, device="cuda")
    c = np.ascontiguousarray(hg.config_1d(t_all=0.1, steps=10, hx=1.0 / m, bx=-4), np.float64)
    info = hg.RunInfo()
    rc = L.hydro1d_run_noalloc(m, state.data_ptr(), c.ctypes.data_as(P), len(c), 2, None, ctypes.byref(info))
    assert rc == -3
    assert "16384" in hg.last_error()
