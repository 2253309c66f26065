"""Seeded synthetic initial data with the shapes and value distributions of the
benchmark cases (the reference's data_in generators are Octave scripts; these
are restated in numpy).

All 2D arrays are returned x-major, shape (m, n): value of cell (x=j, y=i) at
[j, i], the layout of the reference's ``CV.RHO[j][i]`` and of the device planes.
Cell centres are at ((j+0.5)h_x, (i+0.5)h_y) on [0,1]^2.
"""
from __future__ import annotations

import numpy as np


def four_quadrant(m: int, n: int, seed: int = 0):
    """Four constant quadrants around (1/2, 1/2) with rho, p ~ U[0.1, 2] and
    u, v ~ U[-1, 1] drawn from ``default_rng(seed)``. Quadrant k = 0..3 is
    (x>=1/2, y>=1/2), (x<1/2, y>=1/2), (x<1/2, y<1/2), (x>=1/2, y<1/2)."""
    rng = np.random.default_rng(seed)
    rho_q = rng.uniform(0.1, 2.0, 4)
    p_q = rng.uniform(0.1, 2.0, 4)
    u_q = rng.uniform(-1.0, 1.0, 4)
    v_q = rng.uniform(-1.0, 1.0, 4)
    x = (np.arange(m) + 0.5) / m
    y = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, y, indexing="ij")
    q = np.where(X >= 0.5, np.where(Y >= 0.5, 0, 3), np.where(Y >= 0.5, 1, 2))
    return rho_q[q].copy(), u_q[q].copy(), v_q[q].copy(), p_q[q].copy()


def shear_layer(m: int, n: int, seed: int = 0, noise: float = 1e-3):
    """Periodic shear layer: rho = 2, u = +0.5 for |y-1/2| < 1/4, else rho = 1,
    u = -0.5; p = 2.5; v = 0.01 sin(4 pi x) + U[-noise, noise] (seeded)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(m) + 0.5) / m
    y = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, y, indexing="ij")
    inside = np.abs(Y - 0.5) < 0.25
    rho = np.where(inside, 2.0, 1.0)
    u = np.where(inside, 0.5, -0.5)
    p = np.full((m, n), 2.5)
    v = 0.01 * np.sin(4.0 * np.pi * X) + rng.uniform(-noise, noise, (m, n))
    return rho, u, v, p


def sod(m: int = 400):
    """Sod tube on [0,1]: (1, 0, 1) for x < 1/2, (0.125, 0, 0.1) otherwise."""
    x = (np.arange(m) + 0.5) / m
    rho = np.where(x < 0.5, 1.0, 0.125)
    u = np.zeros(m)
    p = np.where(x < 0.5, 1.0, 0.1)
    return rho, u, p


def batch_sizes(count: int = 512, seed: int = 4, lo: int = 64, hi: int = 512, step: int = 32):
    """Square grid sizes N x N with N drawn uniformly from {lo, lo+step, ..., hi}."""
    rng = np.random.default_rng(seed)
    choices = np.arange(lo, hi + 1, step)
    return [(int(N), int(N)) for N in rng.choice(choices, count)]


def batch_problems(sizes, seed: int = 4):
    """Seeded four-quadrant data for every grid of a batch (problem k uses seed*100003 + k)."""
    return [four_quadrant(m, n, seed * 100003 + k) for k, (m, n) in enumerate(sizes)]
