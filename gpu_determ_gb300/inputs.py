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


def dirichlet_mixture_params(ncells: int, seed: int = 0, kmax: int = 4, u_sigma: float = 1.0,
                             T_range=(0.5, 2.0)):
    """Per cell k ~ U{1..kmax} Maxwellians with weights ~ Dirichlet(1, .., 1)
    (total density 1), u ~ N(0, u_sigma^2 I), T ~ U[T_range] (seeded numpy
    default_rng): weights [ncells][kmax] (0 past k), u [ncells][kmax][3], T."""
    rng = np.random.default_rng(seed)
    k = rng.integers(1, kmax + 1, ncells)
    wts = rng.dirichlet(np.ones(kmax), ncells)
    wts = np.where(np.arange(kmax)[None, :] < k[:, None], wts, 0.0)
    wts /= wts.sum(axis=1, keepdims=True)
    u = rng.normal(0.0, u_sigma, (ncells, kmax, 3))
    T = rng.uniform(T_range[0], T_range[1], (ncells, kmax))
    return wts, u, T


def dirichlet_mixtures(grid: dict, ncells: int, seed: int = 0, kmax: int = 4, u_sigma: float = 1.0,
                       T_range=(0.5, 2.0), chunk: int = 2048, device=None):
    """Surrogate training distributions (dirichlet_mixture_params), evaluated
    in FP64 on the host, or on a torch device when one is given (same values
    up to the exponential's rounding); float32 [n_pnt][ncells]."""
    wts, u, T = dirichlet_mixture_params(ncells, seed, kmax, u_sigma, T_range)
    xu, xv, xw = node_velocities(grid)
    if device is not None:
        import torch
        X = torch.from_numpy(np.stack([xu, xv, xw])).to(device)
        W, U, TT = (torch.from_numpy(a).to(device) for a in (wts, u, T))
        out = torch.zeros((len(xu), ncells), dtype=torch.float32, device=device)
        for c0 in range(0, ncells, chunk):
            c1 = min(ncells, c0 + chunk)
            acc = torch.zeros((len(xu), c1 - c0), dtype=torch.float64, device=device)
            for j in range(kmax):
                uu, tt, w = U[c0:c1, j], TT[c0:c1, j], W[c0:c1, j]
                c2 = sum((X[a][:, None] - uu[None, :, a]) ** 2 for a in range(3))
                acc += w[None, :] * (np.pi * tt[None, :]) ** -1.5 * torch.exp(-c2 / tt[None, :])
            out[:, c0:c1] = acc.float()
        return out
    out = np.zeros((len(xu), ncells), np.float32)
    for c0 in range(0, ncells, chunk):
        c1 = min(ncells, c0 + chunk)
        acc = np.zeros((len(xu), c1 - c0))
        for j in range(kmax):
            w = wts[c0:c1, j]
            live = w > 0
            if not live.any():
                continue
            uu, tt = u[c0:c1, j], T[c0:c1, j]
            c2 = ((xu[:, None] - uu[None, :, 0]) ** 2 + (xv[:, None] - uu[None, :, 1]) ** 2
                  + (xw[:, None] - uu[None, :, 2]) ** 2)
            acc += np.where(live[None, :], w[None, :] * (np.pi * tt[None, :]) ** -1.5 * np.exp(-c2 / tt[None, :]), 0.0)
        out[:, c0:c1] = acc
    return out


def cavity_field_params(ncells: int, amp: float = 0.8, T_amp: float = 0.3, seed: int = 0):
    """Cell states of a 2-D lid-driven-style field on the unit square.

    Cells sit on an m x m grid, m = ceil(sqrt(ncells)), at the centres
    ((i + 1/2)/m, (j + 1/2)/m) in row order.  The flow is divergence free,
    from the stream function psi = sum_k a_k sin(p_k pi x) sin(q_k pi y) over
    the modes (p, q) in {1, 2}^2 with seeded amplitudes a_k ~ N(0, 1)
    (a_(1,1) kept positive): u = d psi / dy, v = -d psi / dx, scaled so that
    the largest |(u, v)| over the cells is amp (so u vanishes normal to the
    walls, as in a cavity).  The temperature is
    T = 1 + T_amp tau / max|tau| with tau = sum_k b_k cos(p_k pi x) cos(q_k pi y),
    b_k ~ N(0, 1).  Density 1.  Returns u [ncells][3] (w = 0) and T [ncells]."""
    rng = np.random.default_rng(seed)
    m = int(np.ceil(np.sqrt(max(1, ncells))))
    c = np.arange(ncells)
    x = (c % m + 0.5) / m
    y = (c // m + 0.5) / m
    modes = [(1, 1), (1, 2), (2, 1), (2, 2)]
    a = rng.normal(0.0, 1.0, len(modes))
    a[0] = abs(a[0]) + 1.0
    b = rng.normal(0.0, 1.0, len(modes))
    u = np.zeros(ncells)
    v = np.zeros(ncells)
    tau = np.zeros(ncells)
    for (p, q), ak, bk in zip(modes, a, b):
        u += ak * q * np.pi * np.sin(p * np.pi * x) * np.cos(q * np.pi * y)
        v -= ak * p * np.pi * np.cos(p * np.pi * x) * np.sin(q * np.pi * y)
        tau += bk * np.cos(p * np.pi * x) * np.cos(q * np.pi * y)
    speed = np.sqrt(u * u + v * v).max()
    scale = amp / speed if speed > 0 else 0.0
    vel = np.stack([u * scale, v * scale, np.zeros(ncells)], axis=1)
    tmax = np.abs(tau).max()
    T = 1.0 + (T_amp * tau / tmax if tmax > 0 else 0.0)
    return vel, T


def cavity_field(grid: dict, ncells: int, amp: float = 0.8, T_amp: float = 0.3, seed: int = 0,
                 chunk: int = 1024) -> np.ndarray:
    """One Maxwellian M(1, u_c, T_c) per cell of cavity_field_params, in FP64
    on the host; float32 [n_pnt][ncells]."""
    vel, T = cavity_field_params(ncells, amp, T_amp, seed)
    xu, xv, xw = node_velocities(grid)
    out = np.empty((len(xu), ncells), np.float32)
    for c0 in range(0, ncells, chunk):
        c1 = min(ncells, c0 + chunk)
        uu, tt = vel[c0:c1], T[c0:c1]
        c2 = ((xu[:, None] - uu[None, :, 0]) ** 2 + (xv[:, None] - uu[None, :, 1]) ** 2
              + (xw[:, None] - uu[None, :, 2]) ** 2)
        out[:, c0:c1] = (np.pi * tt[None, :]) ** -1.5 * np.exp(-c2 / tt[None, :])
    return out


def rankine_hugoniot(mach: float = 3.0, gamma: float = 5.0 / 3.0, n1: float = 1.0, T1: float = 1.0) -> dict:
    """Upstream/downstream states of a normal shock in the convention
    f ~ n (pi T)^{-3/2} exp(-|xi - u|^2 / T), where T = 2 k T_phys / m and the
    sound speed is sqrt(gamma T / 2).  Ratios (monatomic gamma = 5/3):
    n2/n1 = (g+1) M^2 / ((g-1) M^2 + 2), u2 = u1 n1/n2,
    T2/T1 = (2 g M^2 - (g-1)) ((g-1) M^2 + 2) / ((g+1)^2 M^2).
    Velocities are along x in the frame moving with (u1 + u2) / 2, so the
    upstream and downstream bulk speeds are +-(u1 - u2) / 2."""
    g, M2 = gamma, mach * mach
    u1 = mach * np.sqrt(g * T1 / 2.0)
    r = (g + 1) * M2 / ((g - 1) * M2 + 2)
    tr = (2 * g * M2 - (g - 1)) * ((g - 1) * M2 + 2) / ((g + 1) ** 2 * M2)
    u2 = u1 / r
    shift = 0.5 * (u1 + u2)
    return {"n1": n1, "T1": T1, "u1": u1 - shift, "n2": n1 * r, "T2": T1 * tr, "u2": u2 - shift,
            "lab_u1": u1, "lab_u2": u2, "density_ratio": r, "temperature_ratio": tr, "frame_shift": shift}


def shock_profile(grid: dict, ncells: int, mach: float = 3.0, gamma: float = 5.0 / 3.0, half_width: float = 8.0,
                  thickness: float = 1.0) -> np.ndarray:
    """Cells at x_c = -half_width + (c + 1/2) 2 half_width / ncells across a
    normal shock: f = (1 - w) M(n1, u1, T1) + w M(n2, u2, T2) with
    w = (1 + tanh(x / thickness)) / 2 (the bimodal Mott-Smith form); float32."""
    s = rankine_hugoniot(mach, gamma)
    x = -half_width + (np.arange(ncells) + 0.5) * (2 * half_width / ncells)
    w = 0.5 * (1 + np.tanh(x / thickness))
    m1 = maxwellian(grid, s["n1"], (s["u1"], 0, 0), s["T1"])
    m2 = maxwellian(grid, s["n2"], (s["u2"], 0, 0), s["T2"])
    return ((1 - w)[None, :] * m1[:, None] + w[None, :] * m2[:, None]).astype(np.float32)
