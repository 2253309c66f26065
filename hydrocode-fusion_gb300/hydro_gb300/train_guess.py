"""Train the learned Newton starting pressure on the GPU and write its weights.

    python -m hydro_gb300.train_guess [--n 10000000] [--epochs 12] [--out PATH]

Problems are generated and labelled on the device (FP64 exact solver), the
network is trained by the library's own forward/backward/Adam kernels, and the
flat FP32 parameter vector (4673 values, little-endian) is written to
hydrocode-fusion_gb300/weights/riemann_guess_6_64_64_1.f32.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import WEIGHTS_PATH, Mlp


def train(n=10_000_000, epochs=12, batch=8192, lr=3e-3, seed=2024, holdout=200_000, out=WEIGHTS_PATH):
    net = Mlp(seed=seed)
    t0 = time.time()
    net.generate(n, seed=seed)
    t1 = time.time()
    losses = net.train(epochs, batch=batch, lr=lr, holdout=holdout)
    t2 = time.time()
    X, Y = net.data(n)
    Xh, Yh = X[-holdout:], Y[-holdout:]
    pred = net.predict(Xh)
    err = pred - Yh
    report = {"samples": n, "epochs": epochs, "batch": batch, "lr": lr, "generate_s": t1 - t0, "train_s": t2 - t1,
              "loss_per_epoch": [float(x) for x in losses], "holdout_rmse_log_p": float(np.sqrt(np.mean(err ** 2))),
              "holdout_p90_abs_log_p": float(np.quantile(np.abs(err), 0.9))}
    os.makedirs(os.path.dirname(out), exist_ok=True)
    net.params().astype("<f4").tofile(out)
    return report


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=10_000_000)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--out", default=WEIGHTS_PATH)
    a = ap.parse_args()
    print(json.dumps(train(a.n, a.epochs, a.batch, a.lr, out=a.out)))


if __name__ == "__main__":
    main()
