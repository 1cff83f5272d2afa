"""Batched cells on uneven velocity grids, stepped as one CUDA graph.

    python -m gpu_determ_gb300.batched [--cells 4096] [--grids 12 16 20 24] [--steps 50]
                                       [--radius 4.8] [--mach 3] [--no-graph] [--no-autotune]
                                       [--fused {cmatrix,pair_tc}]

The cells sample a Mach-3 normal shock (inputs.shock_profile: tanh blend of
the Rankine-Hugoniot upstream and downstream Maxwellians, gamma = 5/3,
upstream n = 1, T = 1) and are dealt round-robin to the grids, so every grid
holds a full sampling of the profile.  Each grid is a context whose gain
launch the autotuner picks on its own cells; one gd_batch holds all groups,
and each step (collision, FP64 projection, Courant relaxation per grid) is
one CUDA graph launch after the first two.  With --fused, every grid's gain
runs in ONE launch per step: the collision-matrix kernel over all grids'
(cell tile, node) pairs (cmatrix), or the persistent pair-product kernel over
all grids' (cell tile, s-chunk) units (pair_tc).  Reported: cells*steps/s over the
timed steps (CUDA events on the launching stream), per-grid moment drift
between the first and last step, the autotuner's choices.
"""
from __future__ import annotations

import argparse
import json
import sys

import numpy as np

from . import (BATCH_FUSED_CMATRIX, BATCH_FUSED_PAIR_TC, DT_COURANT, GAIN_CMATRIX_BF16X3, GAIN_PAIR, GAIN_PAIR_TC, Batch, Context, GridSpec,
               inputs)


def build(cells: int = 4096, grids=(12, 16, 20, 24), radius: float = 4.8, mach: float = 3.0,
          courant: float = 0.5, autotune: bool = True, mem_budget: float = 120e9, device: int = 0,
          fused: str | None = None):
    """Contexts, device arrays and the batch; returns a dict of them.  With
    fused = "cmatrix", every grid uses BF16x3 collision matrices and the batch
    computes all gains in one launch of the collision-matrix kernel
    (BATCH_FUSED_CMATRIX); with fused = "pair_tc", every grid runs the pair
    products with the contraction on the tensor cores in one persistent launch
    (BATCH_FUSED_PAIR_TC); otherwise each grid's gain path is autotuned."""
    import torch
    dev = torch.device("cuda", device)
    groups = []
    b = Batch()
    for k, n in enumerate(grids):
        mine = np.arange(k, cells, len(grids))
        spec = GridSpec(n, R=radius)
        ctx = Context(spec, device=device)
        g = spec.fill()
        f_all = inputs.shock_profile(g, cells, mach=mach)
        f = torch.from_numpy(np.ascontiguousarray(f_all[:, mine])).to(dev)
        nc = len(mine)
        tune = None
        if fused == "cmatrix":
            ctx.set_gain_path(GAIN_CMATRIX_BF16X3)
        elif fused == "pair_tc":
            ctx.set_gain_path(GAIN_PAIR_TC)
        elif autotune:
            tune = ctx.autotune(f, nc, nc,
                                path_mask=(1 << GAIN_PAIR) | (1 << GAIN_PAIR_TC) | (1 << GAIN_CMATRIX_BF16X3),
                                mem_budget=mem_budget)
        m5 = torch.zeros((nc, 5), dtype=torch.float64, device=dev)
        t = torch.zeros(1, dtype=torch.float32, device=dev)
        b.add(ctx, f, nc, nc, DT_COURANT, courant, m5=m5, time=t)
        groups.append({"grid": n, "n_pnt": ctx.n_pnt, "cells": nc, "ctx": ctx, "f": f, "m5": m5, "time": t,
                       "autotune": tune})
    if fused:
        b.set_mode(BATCH_FUSED_CMATRIX if fused == "cmatrix" else BATCH_FUSED_PAIR_TC)
    return {"batch": b, "groups": groups, "device": dev, "fused": fused}


def run(state: dict, steps: int = 50, use_graph: bool = True, warmup: int = 2) -> dict:
    """warmup steps (eager, then capture), then `steps` timed steps."""
    import torch
    b = state["batch"]
    st = torch.cuda.current_stream(state["device"])
    for _ in range(warmup):
        b.step(use_graph, stream=st)
    torch.cuda.synchronize(state["device"])
    m_first = [g["m5"].clone() for g in state["groups"]]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(steps):
        b.step(use_graph, stream=st)
    e1.record(st)
    b.check()
    torch.cuda.synchronize(state["device"])
    ms = e0.elapsed_time(e1)
    cells = sum(g["cells"] for g in state["groups"])
    out = {"cells": cells, "steps": steps, "graph": bool(use_graph), "fused_gain_launch": state.get("fused", False),
           "ms_total": ms,
           "cell_steps_per_s": cells * steps / (ms * 1e-3), "batch": b.info(), "grids": []}
    for g, m0 in zip(state["groups"], m_first):
        m1 = g["m5"]
        # largest change over the cells, relative to the largest mass (n, n u) or
        # energy (E) of any cell
        d = (m1 - m0).abs().max(dim=0).values
        scale = m0.abs().max(dim=0).values
        drift = {"n": float(d[0] / scale[0]), "nu": float(d[1:4].max() / scale[0]), "E": float(d[4] / scale[4])}
        out["grids"].append({"grid": g["grid"], "n_pnt": g["n_pnt"], "cells": g["cells"],
                             "time": float(g["time"].item()), "moment_drift": drift,
                             "autotune": g["autotune"]})
    return out


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--cells", type=int, default=4096)
    p.add_argument("--grids", type=int, nargs="+", default=[12, 16, 20, 24])
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--radius", type=float, default=4.8)
    p.add_argument("--mach", type=float, default=3.0)
    p.add_argument("--no-graph", action="store_true")
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--compare-eager", action="store_true", help="also time the same steps without the graph")
    p.add_argument("--fused", nargs="?", const="cmatrix", choices=["cmatrix", "pair_tc"],
                   help="every grid's gain in one launch: collision matrices (default) or the persistent "
                        "pair-product kernel")
    a = p.parse_args(argv)
    state = build(a.cells, a.grids, a.radius, a.mach, autotune=not a.no_autotune, fused=a.fused)
    res = run(state, a.steps, use_graph=not a.no_graph)
    if a.compare_eager:
        res["eager"] = {k: v for k, v in run(state, a.steps, use_graph=False, warmup=0).items()
                        if k in ("ms_total", "cell_steps_per_s")}
    res["shock"] = {k: float(v) for k, v in inputs.rankine_hugoniot(a.mach).items()}
    print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
