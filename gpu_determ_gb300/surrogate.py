"""Learned collision surrogate with plain-method fallback.

    python -m gpu_determ_gb300.surrogate [--grid 20] [--radius 4.8] [--pairs 65536]
                                         [--steps 4000] [--batch 1024] [--tol 1e-3] [--seed 0]

Pipeline (all compute in libgpu_determ.so; torch only holds device buffers):
  1. data: seeded Dirichlet mixtures of 1-4 Maxwellians (inputs.dirichlet_mixtures)
     and their projected Q from the plain method (gd_collision + gd_project,
     collision matrices in BF16x3 mode, rel-L2 ~4e-6 against FP64);
  2. the network Q ~ net(f) (gd_mlp: inputs scaled by the cell's mean, output by
     its square, global gains from the training set's RMS) trained by
     gd_mlp_train_step on the batch-relative loss sum (y - Q)^2 / mean sum Q^2
     (a per-cell relative loss is dominated by near-equilibrium cells whose Q
     is ~0), Adam with warm-up and cosine decay;
  3. the error network log10(err) ~ est(f) trained on cells the main network
     never saw, err being the cell's relative L2 error of the projected
     surrogate Q against the plain Q;
  4. a calibration margin: the 99th percentile of log10(err) - est(f) on a
     third set, so gd_surrogate_gain gets tol * 10^-margin;
  5. evaluation on a fourth set: fallback fraction, per-cell and batch
     relative L2 error of the projected Q, conservation error.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time
from dataclasses import dataclass, field

import numpy as np

from . import (GAIN_CMATRIX_BF16X3, MLP_LOSS_BATCH, MLP_LOSS_MSE, MLP_SCALE_INPUT, MLP_SCALE_OUTPUT, Context,
               GridSpec, Mlp, Surrogate, cell_rel_l2, inputs)


@dataclass
class Dataset:
    f: object          # torch float32 [n][N] (device)
    q: object          # torch float32 or float64 [n][N] (device): projected plain Q
    seed: int
    seconds: float = 0.0

    @property
    def ncells(self) -> int:
        return int(self.f.shape[1])


def plain_q(ctx: Context, f, ncells: int, ld: int, q64, nu, gain, stream=None):
    """Projected Q of the plain method (context's gain path) into q64 (FP64)."""
    ctx.collision(f, ncells, ld, nu, gain, stream=stream)
    ctx.project(f, nu, gain, ncells, ld, q=q64, stream=stream)


def generate(ctx: Context, grid: dict, ncells: int, seed: int, fp64: bool = False, chunk: int = 4096) -> Dataset:
    """f and its plain projected Q for ncells seeded mixtures."""
    import torch
    dev = torch.device("cuda", ctx.device)
    n = ctx.n_pnt
    t0 = time.perf_counter()
    f = inputs.dirichlet_mixtures(grid, ncells, seed=seed, device=dev)
    q = torch.empty((n, ncells), dtype=torch.float64 if fp64 else torch.float32, device=dev)
    nu = torch.empty((n, chunk), dtype=torch.float32, device=dev)
    gain = torch.empty_like(nu)
    q64 = torch.empty((n, chunk), dtype=torch.float64, device=dev)
    for c0 in range(0, ncells, chunk):
        m = min(chunk, ncells - c0)
        fc = f[:, c0:c0 + m].contiguous()
        plain_q(ctx, fc, m, m, q64, nu, gain)
        q[:, c0:c0 + m] = q64.view(-1)[:n * m].view(n, m).to(q.dtype)
    torch.cuda.synchronize(dev)
    return Dataset(f, q, seed, time.perf_counter() - t0)


def lr_at(step: int, steps: int, lr: float, lr_final: float, warmup: int) -> float:
    if step < warmup:
        return lr * (step + 1) / warmup
    p = (step - warmup) / max(1, steps - warmup)
    return lr_final + 0.5 * (lr - lr_final) * (1.0 + math.cos(math.pi * p))


def train(net: Mlp, data: Dataset, targets, steps: int, batch: int, lr: float, lr_final: float = 0.0,
          weight_decay: float = 0.0, warmup: int = 100, seed: int = 0, log_every: int = 200,
          log=None) -> list:
    """Adam on contiguous batches of the (i.i.d.) dataset in a seeded random
    order; returns [(step, mean batch loss)] at the logging points."""
    import torch
    N = data.ncells
    if not targets.is_contiguous() or targets.shape[1] != N:
        raise ValueError("targets must be a contiguous [features][ncells] array")
    nb = N // batch
    if nb < 1:
        raise ValueError("dataset smaller than one batch")
    rng = np.random.default_rng(seed)
    order = rng.permutation(nb)
    loss = torch.zeros(1, dtype=torch.float32, device=data.f.device)
    hist = []
    for s in range(steps):
        if s and s % nb == 0:
            order = rng.permutation(nb)
        b = int(order[s % nb]) * batch
        want = (s + 1) % log_every == 0 or s == steps - 1
        net.train_step(data.f[:, b:], N, targets[:, b:], targets.shape[1], batch,
                       lr_at(s, steps, lr, lr_final, warmup), weight_decay, loss=loss if want else None)
        if want:
            v = float(loss.item())
            hist.append((s + 1, v))
            if log:
                log(f"step {s + 1}: loss {v:.4e}")
    net.check()
    return hist


@dataclass
class Model:
    ctx: Context
    net: Mlp
    est: Mlp | None
    surrogate: Surrogate
    margin: float = 0.0          # log10 safety added to the error estimate
    report: dict = field(default_factory=dict)

    def tol_arg(self, tol: float) -> float:
        """Tolerance to pass to gd_surrogate_gain for a target tol."""
        return tol * 10.0 ** (-self.margin) if tol > 0 else tol


def surrogate_q(model: Model, f, ncells: int, ld: int, tol: float, q64, nu, gain, est_out=None) -> int:
    """Projected Q with the surrogate (fallback above tol); returns the number
    of cells that took the plain method."""
    nfb = model.surrogate.gain(f, ncells, ld, tol, nu, gain, est_out)
    model.ctx.project(f, nu, gain, ncells, ld, q=q64)
    return nfb


def cell_errors(model: Model, data: Dataset, tol: float, chunk: int) -> dict:
    """Per-cell relative L2 error of the projected Q (fallback above tol; tol
    = inf disables it) against the dataset's plain Q, with the estimates."""
    import torch
    dev = data.f.device
    n, N = data.f.shape
    err = torch.empty(N, dtype=torch.float64, device=dev)
    est = torch.empty(N, dtype=torch.float32, device=dev)
    nu = torch.empty((n, chunk), dtype=torch.float32, device=dev)
    gain = torch.empty_like(nu)
    q64 = torch.empty((n, chunk), dtype=torch.float64, device=dev)
    num = den = 0.0
    nfb = 0
    cons = 0.0
    phi = _basis(model.ctx, dev)
    for c0 in range(0, N, chunk):
        m = min(chunk, N - c0)
        fc = data.f[:, c0:c0 + m].contiguous()
        qs = q64.view(-1)[:n * m].view(n, m)
        nfb += surrogate_q(model, fc, m, m, tol, qs, nu, gain, est[c0:c0 + m])
        qr = data.q[:, c0:c0 + m].to(torch.float64).contiguous()
        cell_rel_l2(qs, m, qr, m, n, m, err[c0:c0 + m])
        num += float(((qs - qr) ** 2).sum())
        den += float((qr ** 2).sum())
        mom = phi @ qs                                   # [5][m]
        scale = (phi.abs() @ qs.abs()).clamp_min(1e-300)
        cons = max(cons, float((mom.abs() / scale).max()))
    torch.cuda.synchronize(dev)
    return {"err": err.cpu().numpy(), "est": est.cpu().numpy(), "fallback": nfb,
            "batch_rel_l2": math.sqrt(num / den) if den > 0 else float("inf"), "conservation": cons}


def _basis(ctx: Context, dev):
    """phi [5][n] = (1, xi_x, xi_y, xi_z, |xi|^2) at the compact nodes (FP64)."""
    import torch
    g = ctx.spec.fill()
    xu, xv, xw = inputs.node_velocities(g)
    return torch.from_numpy(np.stack([np.ones_like(xu), xu, xv, xw, xu * xu + xv * xv + xw * xw])).to(dev)


def io_gains(data: Dataset) -> tuple:
    """Global gains that bring the per-cell scaled inputs f / mean(f) and
    targets Q / mean(f)^2 to unit RMS over the dataset."""
    s = data.f.mean(dim=0, keepdim=True)
    xs = data.f / s
    ts = data.q.to(data.f.dtype) / (s * s)
    return 1.0 / float(xs.pow(2).mean().sqrt()), float(ts.pow(2).mean().sqrt())


def fit(ctx: Context, grid: dict, pairs: int = 65536, steps: int = 4000, batch: int = 1024, lr: float = 1e-3,
        est_pairs: int = 16384, est_steps: int = 1500, calib_pairs: int = 4096, max_cells: int = 4096,
        seed: int = 0, log=None) -> Model:
    """Generate data with the context's plain method, train both networks and
    calibrate the fallback margin."""
    n = ctx.n_pnt
    t0 = time.perf_counter()
    train_set = generate(ctx, grid, pairs, seed=1000 + seed)
    if log:
        log(f"training pairs: {pairs} in {train_set.seconds:.1f} s")
    in_gain, out_gain = io_gains(train_set)
    net = Mlp(n, n, batch_cap=max(batch, max_cells), flags=MLP_SCALE_INPUT | MLP_SCALE_OUTPUT | MLP_LOSS_BATCH,
              seed=seed)
    net.set_io_scale(in_gain, out_gain)
    t1 = time.perf_counter()
    hist = train(net, train_set, train_set.q, steps, batch, lr, lr_final=lr * 0.02, weight_decay=0.0,
                 warmup=min(200, steps // 10 + 1), seed=seed, log=log)
    t_train = time.perf_counter() - t1
    del train_set
    est = Mlp(n, 1, batch_cap=max(batch, max_cells), flags=MLP_SCALE_INPUT | MLP_LOSS_MSE, seed=seed + 1)
    est.set_io_scale(in_gain, 1.0)
    model = Model(ctx, net, est, Surrogate(ctx, net, est, max_cells))
    est_set = generate(ctx, grid, est_pairs, seed=2000 + seed)
    e = cell_errors(model, est_set, float("inf"), max_cells)
    import torch
    tgt = torch.from_numpy(np.ascontiguousarray(np.log10(np.maximum(e["err"], 1e-12)).astype(np.float32)[None, :]))
    tgt = tgt.contiguous().to(est_set.f.device)
    t2 = time.perf_counter()
    est_hist = train(est, est_set, tgt, est_steps, batch, lr, lr_final=lr * 0.02, weight_decay=1e-4,
                     warmup=min(100, est_steps // 10 + 1), seed=seed + 7, log=log)
    t_est = time.perf_counter() - t2
    del est_set
    cal = generate(ctx, grid, calib_pairs, seed=3000 + seed)
    c = cell_errors(model, cal, float("inf"), max_cells)
    gap = np.log10(np.maximum(c["err"], 1e-12)) - c["est"]
    model.margin = float(np.quantile(gap, 0.99))
    model.report = {"pairs": pairs, "steps": steps, "batch": batch, "lr": lr, "train_s": round(t_train, 2),
                    "in_gain": in_gain, "out_gain": out_gain,
                    "est_pairs": est_pairs, "est_steps": est_steps, "est_train_s": round(t_est, 2),
                    "loss_first": hist[0][1], "loss_last": hist[-1][1], "est_loss_last": est_hist[-1][1],
                    "surrogate_err_median_heldout": float(np.median(e["err"])),
                    "margin_log10": model.margin, "fit_s": round(time.perf_counter() - t0, 2)}
    return model


def evaluate(model: Model, data: Dataset, tol: float, chunk: int) -> dict:
    """Fallback fraction and errors of surrogate+fallback at tol on data."""
    r = cell_errors(model, data, model.tol_arg(tol), chunk)
    err = r["err"]
    N = len(err)
    fb = r["fallback"]
    pure = cell_errors(model, data, float("inf"), chunk)["err"]
    return {"cells": N, "tol": tol, "fallback_fraction": fb / N,
            "batch_rel_l2": r["batch_rel_l2"], "cell_rel_l2_median": float(np.median(err)),
            "cell_rel_l2_p99": float(np.quantile(err, 0.99)), "cell_rel_l2_max": float(err.max()),
            "cells_above_tol": int((err > tol).sum()), "conservation_max": r["conservation"],
            "surrogate_only_median": float(np.median(pure)), "surrogate_only_p99": float(np.quantile(pure, 0.99)),
            "surrogate_only_within_tol": float((pure <= tol).mean())}


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--grid", type=int, default=20)
    p.add_argument("--radius", type=float, default=4.8)
    p.add_argument("--pairs", type=int, default=65536)
    p.add_argument("--steps", type=int, default=4000)
    p.add_argument("--batch", type=int, default=1024)
    p.add_argument("--lr", type=float, default=1e-3)
    p.add_argument("--est-steps", type=int, default=1500)
    p.add_argument("--test", type=int, default=4096)
    p.add_argument("--tol", type=float, nargs="+", default=[1e-3, 1e-2, 3e-2])
    p.add_argument("--seed", type=int, default=0)
    a = p.parse_args(argv)
    spec = GridSpec(a.grid, R=a.radius)
    ctx = Context(spec)
    ctx.set_gain_path(GAIN_CMATRIX_BF16X3)
    grid = spec.fill()
    log = lambda s: print(s, file=sys.stderr, flush=True)
    model = fit(ctx, grid, a.pairs, a.steps, a.batch, a.lr, est_steps=a.est_steps, seed=a.seed, log=log)
    test = generate(ctx, grid, a.test, seed=4000 + a.seed)
    out = {"grid": a.grid, "n_pnt": ctx.n_pnt, "fit": model.report,
           "eval": [evaluate(model, test, t, 4096) for t in a.tol]}
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
