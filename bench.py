"""Benchmark: 2D GRP cell-updates/s at 4096^2 on one GB300.

A "step" is one time step of the 2D unsplit GRP scheme over the whole grid
(seeded four-quadrant Riemann data, transmissive boundaries, CFL 0.45).
value      : FP32 form (learned starting pressure when available), device
             resident state, CUDA-event time of the K timed steps.
e2e        : the same metric through the reference's C entry point
             GRP_solver_2D_EUL_source with host arrays (upload, K steps,
             download inside the timed region).
fp64       : the plain FP64 parity form on the same grid (fewer steps).
roofline   : HBM roofline of the step kernel from its algorithmic bytes
             (96 B per cell-update in FP32: rho,u,v,p + 8 slopes read and written).
cpu_baseline: the oracle port of the reference's CPU path (OpenMP, all host
             threads) on a bounded sample of the same grid.

--impl reference times that CPU path alone on the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "hydrocode-fusion_gb300")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
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
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_baseline(m, n, steps, threads):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from hydro_gb300 import cases

    if not os.path.exists(orc.PORT_SO):
        orc.build()
    port = orc.Oracle("port")
    rho, u, v, p = cases.four_quadrant(m, n, seed=2024)
    cfg = orc.default_config_2d(t_all=-1, steps=steps, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4)
    t0 = time.perf_counter()
    out = port.run_2d(rho, u, v, p, cfg, threads=threads)
    wall = time.perf_counter() - t0
    loop = out["wall"]  # time of the scheme call itself (allocation + loop)
    return m * n * steps / loop, loop, wall


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--fp64-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the kernel-variant autotuner")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    m = n = args.size
    workload = f"2D GRP unsplit, {m}x{n} four-quadrant (seeded), transmissive, CFL 0.45"
    metric = "2D GRP cell-updates/s at 4096^2"
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        rate, loop, wall = cpu_baseline(m, n, max(1, args.cpu_steps), threads)
        line = {"impl": "reference", "metric": metric, "value": rate, "unit": "cell-updates/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": loop * 1e3 / max(1, args.cpu_steps),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": workload, "sample_steps": max(1, args.cpu_steps)},
                "cpu_baseline": {"value": rate, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                                 "sample": f"{m}x{n}, {max(1, args.cpu_steps)} steps"},
                "e2e": {"value": rate, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch

    import hydro_gb300 as hg
    from hydro_gb300 import cases

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rho, u, v, p = cases.four_quadrant(m, n, seed=2024)
    K, W = args.steps, max(3, args.warmup)
    form = hg.FORM_FP32
    cfg_w = hg.config_2d(t_all=-1, steps=W, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4)
    cfg_k = hg.config_2d(t_all=-1, steps=K, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4)

    s = hg.Solver2D(m, n, form)
    s.upload(rho, u, v, p)
    tune = None
    if not args.no_tune:
        best, times = s.autotune(cfg_w, steps=3)
        tune = {"best": best, "ms_per_3_steps": times}
    variant = s.variant()
    s.run(cfg_w)                      # warm-up steps
    s.upload(rho, u, v, p)
    torch.cuda.synchronize()
    l0 = hg.kernel_launches()
    with ClockSampler() as cs:
        info = s.run(cfg_k, stats=False)
    launches = hg.kernel_launches() - l0
    torch.cuda.synchronize()
    ms_step = info.gpu_ms / K
    value = m * n * K / (info.gpu_ms * 1e-3)
    s.close()

    # FP64 parity form, same grid
    fp64 = None
    if args.fp64_steps > 0:
        fp64 = fp64_run(hg, m, n, rho, u, v, p, args)
    line_fp64 = fp64

    peak, peak_kind = peaks()
    alg_bytes = 96.0 * m * n  # per launch: 12 FP32 fields read + written
    achieved = alg_bytes / (ms_step * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "peak_source": peak_kind}

    cpu = None
    if not args.no_cpu:
        rate, loop, wall = cpu_baseline(m, n, max(1, args.cpu_steps), threads)
        cpu = {"value": rate, "unit": "cell-updates/s", "cores": threads, "kind": "port",
               "sample": f"{m}x{n}, {max(1, args.cpu_steps)} steps of the FP64 reference arithmetic (OpenMP)"}

    line = {"metric": metric, "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload, "form": "fp32", "grid": [m, n], "l2": "inputs larger than L2 (13 planes x 4 B x 16.8M cells)",
                       "kernel_variant": variant, "autotune": tune},
            "roofline": roof, "cpu_baseline": cpu, "gpu_launches": int(launches),
            "fp64": line_fp64, "clocks": cs.summary()}
    if rank == 0:
        print(json.dumps(line))


def fp64_run(hg, m, n, rho, u, v, p, args):
    s64 = hg.Solver2D(m, n, hg.FORM_FP64)
    s64.upload(rho, u, v, p)
    tune64 = None
    if not args.no_tune and args.fp64_steps > 0:
        best64, times64 = s64.autotune(hg.config_2d(t_all=-1, steps=2, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4), steps=2)
        tune64 = {"best": best64, "ms_per_2_steps": times64}
    s64.run(hg.config_2d(t_all=-1, steps=3, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4))
    s64.upload(rho, u, v, p)
    i64 = s64.run(hg.config_2d(t_all=-1, steps=args.fp64_steps, hx=1.0 / m, hy=1.0 / n, bx=-4, by=-4), stats=True)
    fp64_rate = m * n * args.fp64_steps / (i64.gpu_ms * 1e-3)
    s64.close()
    return {"value": fp64_rate, "unit": "cell-updates/s", "steps": args.fp64_steps,
            "ms_per_step": i64.gpu_ms / args.fp64_steps,
            "newton_faces_per_step": i64.newton_faces / args.fp64_steps,
            "newton_iters_per_face": (i64.newton_iters / i64.newton_faces) if i64.newton_faces else 0.0,
            "autotune": tune64}


if __name__ == "__main__":
    main()
