"""Benchmark: 2D GRP cell-updates/s at 4096^2 on one GB300.

Workload: the 2D unsplit GRP scheme (the reference's GRP_solver_2D_EUL_source)
on a 4096 x 4096 grid over [0,1]^2, seeded four-quadrant Riemann data
(rho, p ~ U[0.1,2], u, v ~ U[-1,1], seed 2024), transmissive boundaries,
gamma 1.4, CFL 0.45.  A "step" is one time step over the whole grid.

value       FP32 form with the learned Newton starting pressure (the headline
            form), state resident in HBM, CUDA-event time of K steps on the
            solver's stream (inputs of 13 planes x 4 B x 16.8 M cells, far
            larger than L2, so no flush is needed between steps).
e2e         the same form through the reference's scheme call
            GRP_solver_2D_EUL_source (config[300] = 2) from host arrays:
            upload, K steps and download inside the timed region (wall clock
            around the call; the second call on the same host arrays, which
            reuses the solver the entry point kept from the first; the first
            call is reported beside it).
forms       plain FP32 and the FP64 parity form on the same grid and steps,
            relative L1 of every FP32 result against the FP64 result, FP64
            conservation integrals, Newton statistics.
roofline    HBM roofline of the step kernel: 96 algorithmic bytes per FP32
            cell-update (the carried state, 4 primitives + 8 limiter slopes,
            read once and written once; 192 B in FP64).
batch       512 independent four-quadrant problems, N x N with N uniform in
            {64, 96, ..., 512}, 300 steps, captured in a CUDA graph with the
            autotuned tile shape and schedule (one persistent kernel, or one
            launch per step).
cpu_baseline the oracle's C restatement of the reference's CPU path (OpenMP,
            all host cores) on a bounded number of steps of the same grid.

--impl reference times that CPU path alone on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "hydrocode-fusion_gb300")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402

METRIC = "2D GRP cell-updates/s at 4096^2"
UNIT = "cell-updates/s"
BYTES_PER_CELL_F32 = 96.0    # 4 primitives + 8 slopes, read once and written once, 4 B
BYTES_PER_CELL_F64 = 192.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def fp64_inst_per_cell():
    """FP64-pipe thread instructions per cell-update of the FP64 step kernel
    (ncu capture summarised in profiles/traffic.json), and that kernel."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            d = json.load(f)["fp64"]
        return float(d["fp64_thread_inst_per_cell"]), d["kernel"]
    except Exception:
        return None, None


def traffic_per_cell(form_key):
    """DRAM bytes per cell-update of a form's step kernel from the committed
    ncu summary, and the kernel configuration it was captured on."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            d = json.load(f)[form_key]
        return float(d["dram_bytes_per_cell"]), d["kernel"]
    except Exception:
        return None, None


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or "0"
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", dev, f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [v for v in (num(s[0]) for s in self.samples) if v is not None]
        mx = [v for v in (num(s[1]) for s in self.samples) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_rate(m, n, steps, threads, warmup=1):
    """The oracle's C restatement of the reference's 2D unsplit GRP loop on the
    host cores: `warmup` untimed steps (page the code and data in), then
    `steps` steps timed by the loop's own wall clock, as the reference's
    cpu_time_sum (grp_solver_2D_EUL_source.c:284,289); returns (cell-updates/s,
    seconds of the timed loop)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from hydro_gb300 import cases

    if not os.path.exists(orc.PORT_SO):
        orc.build()
    port = orc.Oracle("port")
    rho, u, v, p = cases.four_quadrant(m, n, seed=2024)
    if warmup > 0:
        cfgw = orc.default_config_2d(t_all=-1, steps=warmup, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4)
        port.run_2d(rho, u, v, p, cfgw, threads=threads)
    cfg = orc.default_config_2d(t_all=-1, steps=steps, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4)
    out = port.run_2d(rho, u, v, p, cfg, threads=threads)
    return m * n * steps / out["wall"], out["wall"]


def host_info():
    """The host the CPU legs ran on: logical cores, CPU model, OMP_NUM_THREADS."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                key = ln.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "processor model") and ":" in ln:
                    model = ln.split(":", 1)[1].strip()
                    break
        if model is None:
            import platform
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for ln in out.splitlines():
                if ln.strip().lower().startswith("model name"):
                    model = ln.split(":", 1)[1].strip()
                    break
            model = model or platform.processor() or platform.machine()
    except Exception:
        pass
    return {"nproc": os.cpu_count() or 1, "cpu_model": model, "omp_num_threads": os.environ.get("OMP_NUM_THREADS")}


def cpu_baseline(m, n, steps, warmup):
    """The CPU baseline: all host threads on `steps` steps of the workload, and
    one thread on one step of it (the reference's loop restated in C)."""
    threads = os.cpu_count() or 1
    rate, loop = cpu_rate(m, n, steps, threads, warmup)
    rate1, loop1 = cpu_rate(m, n, 1, 1, 0)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{m}x{n}, {steps} timed steps after {warmup} untimed (the reference's loop restated in C, "
                      f"OpenMP, all host threads)",
            "ms_per_step": loop * 1e3 / steps,
            "one_thread": {"value": rate1, "unit": UNIT, "ms_per_step": loop1 * 1e3, "sample": f"{m}x{n}, 1 step"},
            "host": host_info()}


def slowest_rank_ms(ms, dist, device):
    """The job's time over ranks: the maximum (every rank advances its own
    grid, and the job ends when the slowest replica does); ms itself with one
    rank."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_value(cells, steps, ms, world):
    """Whole-job cell-updates/s of `world` replicas that each advance `cells`
    cells `steps` steps, the slowest taking ms milliseconds."""
    return world * cells * steps / (ms * 1e-3)


def rel_l1(a, b):
    d = np.abs(b).sum()
    return float(np.abs(a - b).sum() / d) if d > 0 else float(np.abs(a - b).sum())


def timed_form(hg, form, state, m, n, K, W, tune, stats_steps, clocks=False, dist=None, bnd=-4, solver=0):
    """Tune, warm up, then time K steps of one form from the initial state
    (boundary code bnd on all sides; solver = the interface GRP solver,
    config[301]).  Returns a dict with the rate, the final state and
    statistics."""
    rho, u, v, p = state
    cfgK = hg.config_2d(t_all=-1, steps=K, hx=1.0 / m, hy=1.0 / n, bx=bnd, by=bnd, solver=solver)
    cfgW = hg.config_2d(t_all=-1, steps=W, hx=1.0 / m, hy=1.0 / n, bx=bnd, by=bnd, solver=solver)
    s = hg.Solver2D(m, n, form, solver)
    res = {}
    try:
        if form == hg.FORM_FP32_LEARNED:
            s.set_mlp(hg.load_weights())
        s.upload(rho, u, v, p)
        if tune:
            best, times = s.autotune(cfgW, steps=3)
            res["autotune"] = {"best": best, "ms_per_3_steps": [round(t, 3) for t in times]}
        res["kernel_variant"] = s.variant()[1]
        s.run(cfgW)
        s.upload(rho, u, v, p)
        res["conservation_initial"] = s.conservation()
        import torch

        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        l0 = hg.kernel_launches()
        sampler = ClockSampler() if clocks else None
        if sampler:
            sampler.__enter__()
        info = s.run(cfgK)
        if sampler:
            sampler.__exit__(None, None, None)
        torch.cuda.synchronize()
        res["launches"] = hg.kernel_launches() - l0
        ms = slowest_rank_ms(info.gpu_ms, dist, "cuda")
        res["gpu_ms"] = ms
        res["ms_per_step"] = ms / K
        res["value"] = m * n * K / (ms * 1e-3)
        res["steps_done"] = info.steps_done
        res["halted"] = info.halted
        res["clocks"] = sampler.summary() if sampler else None
        res["conservation_final"] = s.conservation()
        res["state"] = s.download()
        if stats_steps > 0:
            s.upload(rho, u, v, p)
            i2 = s.run(hg.config_2d(t_all=-1, steps=stats_steps, hx=1.0 / m, hy=1.0 / n, bx=bnd, by=bnd,
                                    solver=solver), stats=True)
            faces = 2.0 * m * n * stats_steps
            res["newton"] = {"steps": stats_steps, "exact_solves_per_face": i2.newton_faces / faces,
                             "iters_per_exact_solve": (i2.newton_iters / i2.newton_faces) if i2.newton_faces else 0.0,
                             "fp64_fallbacks_per_exact_solve": (i2.newton_fallbacks / i2.newton_faces)
                             if i2.newton_faces else 0.0}
    finally:
        s.close()
    return res


def e2e_run(hg, state, m, n, K):
    """The learned form through GRP_solver_2D_EUL_source with host arrays."""
    from hydro_gb300.dropin import Call2D

    rho, u, v, p = state
    cfg = hg.config_2d(t_all=-1, steps=K, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4, form=hg.FORM_FP32_LEARNED)
    c = Call2D(hg.lib(), rho, u, v, p, 1.4, cfg, N_MAX=2)
    warm = Call2D(hg.lib(), rho, u, v, p, 1.4,
                  hg.config_2d(t_all=-1, steps=3, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4, form=hg.FORM_FP32_LEARNED),
                  N_MAX=2)
    # the scheme call reports on stdout as the reference's does: keep that
    # text out of this program's one JSON line
    import ctypes

    sys.stdout.flush()
    saved, devnull = os.dup(1), os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    try:
        # an untimed 3-step call first (the process's one-time costs: network
        # file, driver entry points, kernel attributes), then the K-step call
        # twice on the same host arrays: the first takes the page faults of the
        # caller's freshly allocated output rows (reported as first_call), the
        # second is timed.  Each call creates its solver, packs and copies the
        # host arrays both ways.
        warm.call()
        t0 = time.perf_counter()
        c.call()
        first = time.perf_counter() - t0
        l0 = hg.kernel_launches()
        t0 = time.perf_counter()
        nplot, k_out = c.call()
        wall = time.perf_counter() - t0
        launches = hg.kernel_launches() - l0
        ctypes.CDLL(None).fflush(None)
    finally:
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)
    plane_bytes = 8 * m * n
    return {"value": m * n * K / wall, "unit": UNIT, "h2d_bytes_per_step": 5 * plane_bytes / K,
            "d2h_bytes_per_step": 5 * plane_bytes / K, "wall_s": wall, "k_out": int(k_out), "launches": int(launches),
            "first_call": {"value": m * n * K / first, "wall_s": first,
                           "note": "the same call into freshly allocated host rows (their first-touch page faults)"},
            "call": "GRP_solver_2D_EUL_source, config[300]=2, host x-major row arrays (CV[0] in, CV[1] out)"}


def batch_run(hg, count, steps, tune_steps, l1_sample, fixed=None):
    """fixed: (shape, schedule) to run instead of the autotuner's pick."""
    from hydro_gb300 import cases

    sizes = cases.batch_sizes(count, seed=4)
    probs = cases.batch_problems(sizes, seed=4)
    cfg = hg.config_2d(t_all=-1, steps=steps, bx=-4, by=-4)
    b = hg.Batch(sizes)
    try:
        for k, pr in enumerate(probs):
            b.upload(k, *pr)
        if fixed is None:
            best, times = b.autotune(cfg, steps=tune_steps)
        else:
            b.set_schedule(*fixed)
            times = np.zeros((0, 0))
        l0 = hg.kernel_launches()
        info = b.run(cfg, steps)
        launches = hg.kernel_launches() - l0
        cells = sum(mm * nn for mm, nn in sizes)
        rate = cells * steps / (info.gpu_ms * 1e-3)
        halted = [k for k in range(count) if b.problem_info(k)["halted"]]
        sample = sorted(set(list(range(0, count, max(1, count // l1_sample)))[:l1_sample] + halted[:4]))
        l1 = []
        for k in sample:
            mm, nn = sizes[k]
            got = b.download(k)
            pi = b.problem_info(k)
            c64 = hg.config_2d(t_all=-1, steps=steps, hx=1.0 / mm, hy=1.0 / nn, bx=-4, by=-4)
            want, i64 = hg.run_2d(*probs[k], c64)
            rec = {"problem": k, "N": mm, "halted_fp32": pi["halted"], "halted_step_fp32": pi["halted_step"],
                   "halted_fp64": i64.halted, "steps_fp64": i64.steps_done}
            if not pi["halted"] and not i64.halted:
                rec.update({f: rel_l1(got[f], want[f]) for f in ("rho", "u", "v", "p")})
            l1.append(rec)
    finally:
        b.close()
    shapes = hg.Batch.shapes()
    peak, _ = peaks()
    return {"problems": count, "sizes": "N x N, N uniform in {64, 96, ..., 512} (seed 4)", "cells": cells,
            "steps": steps, "value": rate, "unit": UNIT, "gpu_ms": info.gpu_ms,
            "hbm_frac": BYTES_PER_CELL_F32 * rate / 1e9 / peak,
            "shape": shapes[info.shape], "schedule": hg.SCHEDULES[info.schedule], "graphed": bool(info.graphed),
            "autotune_ms_per_%d_steps" % tune_steps: np.round(times, 3).tolist(), "gpu_launches": int(launches),
            "halted_problems": info.halted_problems, "per_problem_l1_vs_fp64": l1}


def shear_suite(hg, m, n, K, W, tune, stats_steps):
    """Periodic shear layer (rho = 2, u = +0.5 inside |y - 1/2| < 1/4, else
    rho = 1, u = -0.5; p = 2.5; v = 0.01 sin(4 pi x) + seeded noise 1e-3):
    Newton-heavy data, where most faces need the exact Riemann solver.  The
    FP32 forms are timed and compared with the FP64 form."""
    from hydro_gb300 import cases

    state = cases.shear_layer(m, n, seed=1)
    res = {}
    for key, form in (("fp32_learned", hg.FORM_FP32_LEARNED), ("fp32", hg.FORM_FP32), ("fp64", hg.FORM_FP64)):
        res[key] = timed_form(hg, form, state, m, n, K, W, tune, stats_steps, bnd=-7)
    out = {"workload": f"2D unsplit GRP, {m}x{n} periodic shear layer (seed 1), gamma 1.4, CFL 0.45", "steps": K}
    for key in ("fp32_learned", "fp32", "fp64"):
        r = res[key]
        out[key] = {"value": r["value"], "ms_per_step": r["ms_per_step"], "kernel_variant": r["kernel_variant"],
                    "newton": r.get("newton"), "halted": r["halted"]}
        if key != "fp64":
            out[key]["l1_vs_fp64"] = {f: rel_l1(r["state"][f], res["fp64"]["state"][f]) for f in ("rho", "u", "v", "p")}
    out["speedup_learned_over_fp32"] = res["fp32_learned"]["value"] / res["fp32"]["value"]
    out["speedup_learned_over_fp64"] = res["fp32_learned"]["value"] / res["fp64"]["value"]
    return out


def g2d_suite(hg, state, m, n, K, K64, W, tune, stats_steps):
    """The same four-quadrant workload with the genuinely-2D interface solver
    (config[301] = 1, the alternative GRP_2D_flux keeps commented out): FP32
    and FP64 forms timed, FP32 compared with FP64."""
    res = {}
    for key, form, steps in (("fp32", hg.FORM_FP32, K), ("fp64", hg.FORM_FP64, K64)):
        if steps > 0:
            res[key] = timed_form(hg, form, state, m, n, steps, W, tune, stats_steps, solver=hg.SOLVER_G2D)
    out = {"workload": workload_name(m, n) + ", genuinely-2D GRP interface solver (config[301] = 1)"}
    for key, r in res.items():
        out[key] = {"value": r["value"], "ms_per_step": r["ms_per_step"], "steps": r["steps_done"],
                    "kernel_variant": r["kernel_variant"], "newton": r.get("newton"), "halted": r["halted"]}
    if "fp64" in res and res["fp64"]["steps_done"] == res["fp32"]["steps_done"]:
        out["fp32"]["l1_vs_fp64"] = {f: rel_l1(res["fp32"]["state"][f], res["fp64"]["state"][f])
                                     for f in ("rho", "u", "v", "p")}
    return out


MF_BYTES_PER_FACE = 40 * 8 + 18 * 8 + 4   # fields in, fluxes out, status


def mf_faces(rng, n):
    """Two-component faces (field-major, 40 x n): a gamma per side in
    [1.1, 3], densities and pressures log-uniform over e^-2..e^2, velocities
    uniform, unit-normal slopes, volume/mass fractions in [0, 1], any normal;
    a fifth of the faces are uniform pairs (the acoustic case)."""
    f = np.empty((40, n))
    th = rng.uniform(0, 2 * np.pi, n)
    f[0], f[1] = np.cos(th), np.sin(th)
    for b in (2, 21):
        f[b] = rng.uniform(1.1, 3.0, n)
        f[b + 1] = np.exp(rng.uniform(-2, 2, n))
        f[b + 2:b + 4] = rng.uniform(-2, 2, (2, n))
        f[b + 4] = np.exp(rng.uniform(-2, 2, n))
        f[b + 5:b + 13] = rng.normal(0, 1, (8, n))
        f[b + 13] = rng.uniform(0, 1, n)
        f[b + 14:b + 16] = rng.normal(0, 1, (2, n))
        f[b + 16] = rng.uniform(0, 1, n)
        f[b + 17:b + 19] = rng.normal(0, 1, (2, n))
    k = n // 5
    f[22:26, :k] = f[3:7, :k]
    return f


def mf_suite(hg, peak, nface=8 << 20, reps=5, cpu=True):
    """The two-component interface flux (GRP_2D_flux, MULTIFLUID_BASICS) on a
    batch of nface faces through hydro_grp2d_flux_mf: kernel time (inputs in
    HBM), the call's wall time with the host copies, and the oracle's serial
    loop on a sample."""
    rng = np.random.default_rng(2025)
    base = mf_faces(rng, 1 << 20)
    f = np.tile(base, (1, nface >> 20))
    cfg = np.full(400, np.inf)
    cfg[4], cfg[6], cfg[60], cfg[106] = 1e-9, 1.4, 1.0, 3.0
    tau = 1e-4
    # the caller's output arrays, filled by every call (the warm-up call also
    # takes their first-touch page faults, and the device buffers, module load)
    out = np.empty((18, nface))
    status = np.empty(nface, np.int32)
    hg.grp2d_flux_mf(f, tau, cfg, out, status)
    kern, wall = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        out, status, info = hg.grp2d_flux_mf(f, tau, cfg, out, status)
        wall.append(time.perf_counter() - t0)
        kern.append(info.kernel_ms)
    k_ms = float(np.median(kern))
    w_s = float(np.median(wall))
    res = {"workload": f"{nface} two-component faces (seeded, a fifth uniform pairs), gamma_a 1.4, gamma_b 3.0",
           "value": nface / (k_ms * 1e-3), "unit": "faces/s", "kernel_ms": k_ms,
           "e2e": {"value": nface / w_s, "unit": "faces/s", "wall_ms": w_s * 1e3,
                   "h2d_bytes": 40 * 8 * nface, "d2h_bytes": (18 * 8 + 4) * nface},
           "hbm": {"bytes_per_face": MF_BYTES_PER_FACE,
                   "achieved_gbs": MF_BYTES_PER_FACE * nface / (k_ms * 1e-3) / 1e9, "peak_gbs": peak},
           "bad_faces": int(info.n_bad), "resumed_faces": [int(r) for r in info.resumed]}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        sample = 1 << 19
        idx = np.arange(sample) * (nface // sample)      # spread over the batch's mix of cases
        rows = np.ascontiguousarray(f[:, idx].T)
        port = orc.Oracle("port")
        t0 = time.perf_counter()
        want = port.grp2d_flux_mf(rows, tau, 1e-9, 1.4, 3.0, True)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": sample / dt, "unit": "faces/s", "cores": os.cpu_count() or 1,
                               "kind": "port",
                               "sample": f"{sample} faces spread over the batch, the oracle's face loop on all "
                                         f"host threads (OpenMP)"}
        ok = want[:, 18] == 0
        res["rel_l1_vs_oracle_sample"] = float(np.abs(out[:, idx].T[ok] - want[ok, :18]).sum() /
                                               np.abs(want[ok, :18]).sum())
    return res


def reference_arm(args, m, n, rank):
    """The reference's CPU path (the oracle's restatement, all host threads) on
    the same workload: W untimed steps, then every one of the K steps timed
    (capped at --cpu-max-steps so the run stays within minutes; the line says
    how many were timed)."""
    if rank != 0:
        return
    S = max(1, min(args.steps, args.cpu_max_steps))
    cpu = cpu_baseline(m, n, S, min(args.warmup, 3))
    rate = cpu["value"]
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
            "steps": S, "warmup": min(args.warmup, 3), "ms_per_step": cpu["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(m, n), "steps_requested": args.steps},
            "cpu_baseline": cpu,
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_name(m, n):
    return f"2D unsplit GRP, {m}x{n} four-quadrant Riemann data (seed 2024), transmissive, gamma 1.4, CFL 0.45"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--fp64-steps", type=int, default=-1, help="FP64 form steps (default: --steps; 0 skips)")
    ap.add_argument("--stats-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=12, help="timed steps of the CPU baseline beside our arm")
    ap.add_argument("--cpu-max-steps", type=int, default=200, help="most steps the reference arm times")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the kernel-variant autotuners")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-shear", action="store_true")
    ap.add_argument("--no-g2d", action="store_true")
    ap.add_argument("--no-mf", action="store_true")
    ap.add_argument("--no-costs", action="store_true", help="skip the learned start's per-face cost parts")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=300)
    ap.add_argument("--batch-schedule", default=None,
                    help="SHAPE,SCHEDULE: run the batch with this pair instead of the autotuner's pick")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    m = n = args.size
    if args.impl == "reference":
        reference_arm(args, m, n, rank)
        return

    import torch

    import hydro_gb300 as hg
    from hydro_gb300 import cases

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist = None
    if world > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl")
        dist = tdist
    state = cases.four_quadrant(m, n, seed=2024)
    K, W = args.steps, max(3, args.warmup)
    tune = not args.no_tune
    k64 = K if args.fp64_steps < 0 else args.fp64_steps

    head = timed_form(hg, hg.FORM_FP32_LEARNED, state, m, n, K, W, tune, args.stats_steps, clocks=True, dist=dist)
    if dist is not None:
        dist.barrier()
    value = replicas_value(m * n, K, head["gpu_ms"], world)  # replicas: every rank advances its own grid
    if rank != 0:
        return
    plain = timed_form(hg, hg.FORM_FP32, state, m, n, K, W, tune, args.stats_steps)
    fp64 = timed_form(hg, hg.FORM_FP64, state, m, n, k64, 3, tune, args.stats_steps) if k64 > 0 else None

    def accuracy(res):
        if fp64 is None or k64 != K:
            return None
        return {f: rel_l1(res["state"][f], fp64["state"][f]) for f in ("rho", "u", "v", "p")}

    def summary(res, dtype):
        return {k: v for k, v in res.items() if k not in ("state",)} | {"dtype": dtype}

    peak, peak_kind = peaks()
    ms = head["ms_per_step"]
    achieved = BYTES_PER_CELL_F32 * m * n / (ms * 1e-3) / 1e9
    kv = head["kernel_variant"]
    kname = "%s<float,%dx%d,%d,learned>" % ({"tma": "k_step_tma", "strip": "k_step_strip"}.get(kv.get("kernel"),
                                                                                           "k_step_unsplit"),
                                             kv["tile_x"], kv["tile_y"], kv["threads"])
    tpc, tkern = traffic_per_cell("fp32_learned")
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": tpc * m * n if tpc else None, "peak_source": peak_kind,
            "kernel": kname + " (one launch per step)", "algorithmic_bytes_per_launch": BYTES_PER_CELL_F32 * m * n,
            "traffic_source": f"ncu capture of {tkern} at 2048^2, scaled by cells (profiles/traffic.json)"
            if tpc else None}

    forms = {
        "fp32_learned": summary(head, "f32") | {"l1_vs_fp64": accuracy(head)},
        "fp32": summary(plain, "f32") | {"l1_vs_fp64": accuracy(plain)},
        "fp64": (summary(fp64, "f64") | {
            "hbm_frac": BYTES_PER_CELL_F64 * fp64["value"] / 1e9 / peak}) if fp64 else None,
        "speedup_learned_over_fp64": head["value"] / fp64["value"] if fp64 else None,
    }
    if fp64:
        for key in ("fp32_learned", "fp32"):
            forms[key]["mass_drift_vs_fp64"] = (
                forms[key]["conservation_final"]["mass"] - fp64["conservation_final"]["mass"]) / fp64[
                "conservation_final"]["mass"]

    e2e = None if args.no_e2e else e2e_run(hg, state, m, n, K)
    fixed = tuple(int(x) for x in args.batch_schedule.split(",")) if args.batch_schedule else None
    batch = None if args.no_batch else batch_run(hg, args.batch_count, args.batch_steps, 5, 8, fixed)
    shear = None if args.no_shear else shear_suite(hg, m, n, K, W, tune, args.stats_steps)
    g2d = None if args.no_g2d else g2d_suite(hg, state, m, n, K, k64, W, tune, args.stats_steps)
    mf = None if args.no_mf else mf_suite(hg, peak, cpu=not args.no_cpu)

    cpu = None if args.no_cpu else cpu_baseline(m, n, max(1, args.cpu_steps), 1)

    # short keys first: a reader that keeps only the head of the line still
    # sees every form's rate, the accuracy of the FP32 forms and the learned start
    fp64_short = None
    if fp64:
        fp64_short = {"value": fp64["value"], "ms_per_step": fp64["ms_per_step"], "steps": k64,
                      "kernel_variant": fp64["kernel_variant"], "hbm_frac": forms["fp64"]["hbm_frac"]}
        # the FP64 form is bound by the FP64 pipe: its roofline is the FP64
        # instructions per cell (ncu) times the cell rate against the measured DFMA rate
        try:
            pk = hg.fp64_peak()
        except Exception:
            pk = None
        ipc, ik = fp64_inst_per_cell()
        fp64_short["fp64_pipe_roofline"] = {
            "bound": "fp64 pipe", "peak": pk, "unit": "FP64 thread-instructions/s",
            "peak_source": "measured (hydro_fp64_peak: DFMA chains on every SM)",
            "inst_per_cell": ipc, "inst_source": f"ncu capture of {ik} at 2048^2 (profiles/traffic.json)" if ipc else None,
            "achieved": ipc * fp64["value"] if ipc else None,
            "frac": ipc * fp64["value"] / pk if (ipc and pk) else None}
    learned = {"ms_per_step": head["ms_per_step"], "plain_fp32_ms_per_step": plain["ms_per_step"],
               "speedup_over_plain_fp32": plain["ms_per_step"] / head["ms_per_step"],
               "speedup_over_fp64": forms["speedup_learned_over_fp64"],
               "newton_learned": head.get("newton"), "newton_plain": plain.get("newton")}
    # the learned start's parts per face, in the FP32 form's code (1 M seeded exact-path faces)
    if rank == 0 and not args.no_costs:
        try:
            c = hg.learned_costs(nfaces=1 << 20)
            c["faces"] = "1048576 seeded pairs, four-quadrant ranges, all through the exact path"
            c["network_vs_iteration"] = (c["network_ns_per_face"] / c["ns_per_newton_iteration"]
                                         if c["ns_per_newton_iteration"] > 0 else None)
            learned["costs"] = c
        except Exception as exc:  # reported, not fatal: the timed forms above are the headline
            learned["costs"] = {"error": str(exc)}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_name(m, n), "form": "fp32 state + learned Newton start",
                       "grid": [m, n], "parallelism": "replicas" if world > 1 else "single",
                       "l2": "no flush: 13 planes x 4 B x 16.8M cells = 872 MB per state >> 129 MB L2"},
            "e2e": e2e, "roofline": roof, "gpu_launches": int(head["launches"]), "clocks": head["clocks"],
            "fp64": fp64_short,
            "l1_vs_fp64": {"fp32_learned": forms["fp32_learned"]["l1_vs_fp64"], "fp32": forms["fp32"]["l1_vs_fp64"]},
            "learned": learned, "cpu_baseline": cpu,
            "forms": forms, "shear": shear, "g2d": g2d, "mf_flux": mf, "batch": batch}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
