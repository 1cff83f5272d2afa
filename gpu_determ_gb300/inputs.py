"""Seeded synthetic distributions on the compact in-sphere nodes (host, numpy).

Maxwellian convention M(n, u, T) = n (pi T)^{-3/2} exp(-|xi - u|^2 / T), which
is the reference's exp(-c^2) initial state (determ.cu:116) at n = pi^{3/2},
T = 1.  All generators return float32 arrays [n_pnt][ncells].
"""
from __future__ import annotations

import numpy as np


def node_velocities(grid: dict):
    """(xi_x, xi_y, xi_z) per compact node, float64, from GridSpec.fill()."""
    return (grid["u"][grid["ui"]].astype(np.float64), grid["v"][grid["vi"]].astype(np.float64),
            grid["w"][grid["wi"]].astype(np.float64))


def maxwellian(grid: dict, n=1.0, u=(0.0, 0.0, 0.0), T=1.0) -> np.ndarray:
    xu, xv, xw = node_velocities(grid)
    c2 = (xu - u[0]) ** 2 + (xv - u[1]) ** 2 + (xw - u[2]) ** 2
    return n * (np.pi * T) ** -1.5 * np.exp(-c2 / T)


def reference_initial_state(grid: dict, ncells: int) -> np.ndarray:
    """determ.cu:101-121: exp(-(u-1.75)^2 - (v-0.25)^2 - w^2) in float, every cell."""
    u = grid["u"][grid["ui"]]
    v = grid["v"][grid["vi"]]
    w = grid["w"][grid["wi"]]
    u1, v1 = np.float32(1.75), np.float32(0.25)
    t = (-(u - u1)) * (u - u1) - (v - v1) * (v - v1) - w * w
    f = np.exp(t.astype(np.float32)).astype(np.float32)
    return np.repeat(f[:, None], ncells, axis=1)


def two_beam(grid: dict, ncells: int = 1) -> np.ndarray:
    """Homogeneous relaxation start: M(0.5, (+1.5,0,0), 1) + M(0.5, (-1.5,0,0), 1)."""
    f = maxwellian(grid, 0.5, (1.5, 0, 0), 1.0) + maxwellian(grid, 0.5, (-1.5, 0, 0), 1.0)
    return np.repeat(f.astype(np.float32)[:, None], ncells, axis=1)


def mixtures(grid: dict, ncells: int, seed: int = 0, kmax: int = 3, u_sigma: float = 0.7,
             T_range=(0.6, 1.8), n_sigma: float = 0.3) -> np.ndarray:
    """Per cell a mixture of 1..kmax Maxwellians: n ~ lognormal(0, n_sigma),
    u ~ N(0, u_sigma^2) per axis, T ~ U[T_range] (seeded numpy default_rng)."""
    rng = np.random.default_rng(seed)
    out = np.zeros((len(grid["ui"]), ncells), np.float64)
    for c in range(ncells):
        k = int(rng.integers(1, kmax + 1))
        for _ in range(k):
            n = float(rng.lognormal(0.0, n_sigma))
            u = rng.normal(0.0, u_sigma, 3)
            T = float(rng.uniform(*T_range))
            out[:, c] += maxwellian(grid, n, u, T)
    return out.astype(np.float32)
