"""Large batched surrogate+fallback: 32^3 lattice cut to R = 5.5 (21 992 nodes).

    python -m gpu_determ_gb300.large [--grid 32] [--radius 5.5] [--cells 16384] [--steps 200]
                                     [--pairs 65536] [--train-steps 4000] [--tol 1e-3]
                                     [--gain pair_tc] [--check-gain pair] [--check-every 1] [--seed 0]

Cells carry one Maxwellian each from a 2-D lid-driven-style field
(inputs.cavity_field: divergence-free sinusoidal flow, |u| <= 0.8,
T = 1 +- 0.3).  The surrogate (network + error estimator, inference in BF16
with FP32 accumulation) is trained first on mixtures of 1-4 Maxwellians
labelled by the plain method of the same context (surrogate.fit).  Each step
is: loss nu, surrogate gain with plain fallback above the tolerance
(gd_surrogate_gain), FP64 conservation projection, Courant relaxation
(dt = courant / max nu' as relax_f).  The plain method (training labels,
fallback, plain-step timing) is the --gain path: at 32^3 the collision matrices
do not fit, and the pair products with the contraction on the tensor cores
(pair_tc) run twice as fast as the FP32 pair kernel (pair) at ~6e-7 from it.
On check steps the --check-gain path (by default the plain FP32 kernel, on a
second context) gives the plain Q of the same f, hence the step's relative L2
error of Q, and the conservation error of the projected Q is measured.

Reported: per checked step the fallback fraction, batch and per-cell relative
L2 of Q, conservation error; totals: surrogate-step cells*steps/s (CUDA
events around the step launches only, checks excluded), the plain step's
cells*steps/s on the same cells, and the moment drift over the run.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

from . import DT_COURANT, GAIN_PAIR, GAIN_PAIR_TC, Context, GridSpec, cell_rel_l2, inputs

GAINS = {"pair": GAIN_PAIR, "pair_tc": GAIN_PAIR_TC}


def run(grid: int = 32, radius: float = 5.5, cells: int = 16384, steps: int = 200, pairs: int = 65536,
        train_steps: int = 4000, tol: float = 1e-3, check_every: int = 1, courant: float = 0.5, seed: int = 0,
        est_pairs: int = 16384, est_steps: int = 1500, calib_pairs: int = 4096, plain_steps: int = 2,
        gain: str = "pair_tc", check_gain: str = "pair", device: int = 0, log=None) -> dict:
    import torch
    from . import surrogate as S
    dev = torch.device("cuda", device)
    plain_name, check_name = gain, check_gain
    spec = GridSpec(grid, R=radius)
    ctx = Context(spec, device=device)
    ctx.set_gain_path(GAINS[gain])
    if check_gain == gain:
        check_ctx = ctx
    else:
        check_ctx = Context(spec, device=device)
        check_ctx.set_gain_path(GAINS[check_gain])
    g = spec.fill()
    n = ctx.n_pnt
    stream = torch.cuda.current_stream(dev)

    t0 = time.perf_counter()
    model = S.fit(ctx, g, pairs=pairs, steps=train_steps, est_pairs=est_pairs, est_steps=est_steps,
                  calib_pairs=calib_pairs, max_cells=cells, seed=seed, log=log)
    fit_s = time.perf_counter() - t0
    tol_arg = model.tol_arg(tol)

    f_host = inputs.cavity_field(g, cells, seed=seed)
    f = torch.from_numpy(f_host).to(dev)
    nu = torch.empty_like(f)
    gain = torch.empty_like(f)
    q = torch.empty(f.shape, dtype=torch.float64, device=dev)
    nu_p = torch.empty_like(f)
    gain_p = torch.empty_like(f)
    q_p = torch.empty_like(q)
    err = torch.empty(cells, dtype=torch.float64, device=dev)
    t_sim = torch.zeros(1, dtype=torch.float32, device=dev)
    phi = S._basis(ctx, dev)
    m_first = (phi @ f.to(torch.float64)).clone()

    per_step = []
    ms_total = 0.0
    fallbacks = 0
    for k in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        nfb = model.surrogate.gain(f, cells, cells, tol_arg, nu, gain, stream=stream)
        ctx.project(f, nu, gain, cells, cells, nu_corr=nu, q=q, stream=stream)
        check = check_every > 0 and (k % check_every == 0 or k == steps - 1)
        if check:
            e1.record(stream)
            # plain Q of the same f, before the relaxation changes it
            check_ctx.collision(f, cells, cells, nu_p, gain_p, stream=stream)
            check_ctx.project(f, nu_p, gain_p, cells, cells, q=q_p, stream=stream)
            cell_rel_l2(q, cells, q_p, cells, n, cells, err, stream=stream)
            rec = {"step": k, "fallback_fraction": nfb / cells,
                   "batch_rel_l2": float((q - q_p).norm() / q_p.norm()),
                   "cell_rel_l2_median": float(err.median()), "cell_rel_l2_max": float(err.max()),
                   "conservation_max": float(((phi @ q).abs() / (phi.abs() @ q.abs()).clamp_min(1e-300)).max())}
            e2 = torch.cuda.Event(enable_timing=True)
            e2.record(stream)
            ctx.relax(f, nu, gain, cells, cells, DT_COURANT, courant, time=t_sim, stream=stream)
            e3 = torch.cuda.Event(enable_timing=True)
            e3.record(stream)
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1) + e2.elapsed_time(e3)
            rec["ms"] = ms
            per_step.append(rec)
            if log:
                log(json.dumps(rec))
        else:
            ctx.relax(f, nu, gain, cells, cells, DT_COURANT, courant, time=t_sim, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1)
        ms_total += ms
        fallbacks += nfb
    ctx.check(stream=stream)
    m_last = phi @ f.to(torch.float64)
    d = (m_last - m_first).abs().max(dim=1).values
    scale = m_first.abs().max(dim=1).values
    drift = {"n": float(d[0] / scale[0]), "nu": float(d[1:4].max() / scale[0]), "E": float(d[4] / scale[4])}

    # the plain step on the same cells, for the speed comparison
    fp = torch.from_numpy(f_host).to(dev)
    ctx.step(fp, cells, cells, DT_COURANT, courant, stream=stream)        # warm-up
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(plain_steps):
        ctx.step(fp, cells, cells, DT_COURANT, courant, stream=stream)
    e1.record(stream)
    ctx.check()
    torch.cuda.synchronize(dev)
    plain_ms = e0.elapsed_time(e1) / max(1, plain_steps)

    value = cells * steps / (ms_total * 1e-3)
    plain_value = cells / (plain_ms * 1e-3)
    return {"grid": grid, "radius": radius, "n_pnt": n, "cells": cells, "steps": steps, "tol": tol,
            "plain_gain": plain_name, "check_gain": check_name, "fit": model.report, "fit_s": round(fit_s, 1),
            "surrogate_step": {"cell_steps_per_s": value, "ms_per_step": ms_total / steps,
                               "fallback_fraction": fallbacks / (cells * steps)},
            "plain_step": {"cell_steps_per_s": plain_value, "ms_per_step": plain_ms, "steps": plain_steps},
            "speedup_vs_plain": value / plain_value, "time": float(t_sim.item()), "moment_drift": drift,
            "checked_steps": per_step}


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--grid", type=int, default=32)
    p.add_argument("--radius", type=float, default=5.5)
    p.add_argument("--cells", type=int, default=16384)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--pairs", type=int, default=65536)
    p.add_argument("--train-steps", type=int, default=4000)
    p.add_argument("--est-pairs", type=int, default=16384)
    p.add_argument("--est-steps", type=int, default=1500)
    p.add_argument("--calib-pairs", type=int, default=4096)
    p.add_argument("--tol", type=float, default=1e-3)
    p.add_argument("--check-every", type=int, default=1)
    p.add_argument("--plain-steps", type=int, default=2)
    p.add_argument("--gain", choices=sorted(GAINS), default="pair_tc",
                   help="plain method: labels, fallback and the timed plain step")
    p.add_argument("--check-gain", choices=sorted(GAINS), default="pair", help="plain method of the per-step checks")
    p.add_argument("--seed", type=int, default=0)
    a = p.parse_args(argv)
    log = lambda s: print(s, file=sys.stderr, flush=True)
    res = run(a.grid, a.radius, a.cells, a.steps, a.pairs, a.train_steps, a.tol, a.check_every, seed=a.seed,
              est_pairs=a.est_pairs, est_steps=a.est_steps, calib_pairs=a.calib_pairs,
              plain_steps=a.plain_steps, gain=a.gain, check_gain=a.check_gain, log=log)
    print(json.dumps(res))
    return 0 if math.isfinite(res["surrogate_step"]["cell_steps_per_s"]) else 1


if __name__ == "__main__":
    sys.exit(main())
