"""Space-homogeneous relaxation: repeated collision steps with moments per step.

    python -m gpu_determ_gb300.relaxation [--grid 20] [--radius 4.8] [--steps 100]
                                          [--courant 0.5 | --dt DT] [--cells 1]
                                          [--init two_beam|mixture] [--seed 0]
                                          [--gain pair|bf16|bf16x3]

Each step is gd_step (loss, gain, FP64 conservation projection, f <- f + dt Q) on
every cell; before each step the FP64 moments of f are read back and reported as
one JSON line per step with density n, bulk velocity u, energy E = sum f xi^2 d3v
and temperature T in the convention f ~ exp(-|xi - u|^2 / T), i.e.
E / n = |u|^2 + 3 T / 2.  The two-beam start is M(0.5, +1.5 e_x, 1) + M(0.5, -1.5 e_x, 1).

The step is explicit, so dt must stay below 1 / max nu for f to remain
positive.  With the reference's normalisation (b = 4 pi |g| d3v) the collision
frequency reaches ~100 at the edge of the velocity sphere, so the default is the
reference's Courant rule dt = courant / max nu (relax_f with courant 0.5).
"""
from __future__ import annotations

import argparse
import json
import sys

import numpy as np

from . import DT_COURANT, DT_FIXED, GAIN_CMATRIX_BF16, GAIN_CMATRIX_BF16X3, GAIN_PAIR, Context, GridSpec, inputs

GAIN_PATHS = {"pair": GAIN_PAIR, "bf16": GAIN_CMATRIX_BF16, "bf16x3": GAIN_CMATRIX_BF16X3}


def moments_to_state(m5: np.ndarray) -> dict:
    """(n, n u, E) per cell -> n, u, E, T arrays."""
    n = m5[:, 0]
    u = m5[:, 1:4] / n[:, None]
    E = m5[:, 4]
    T = (2.0 / 3.0) * (E / n - np.sum(u * u, axis=1))
    return {"n": n, "u": u, "E": E, "T": T}


def run(grid: int = 20, radius: float = 4.8, steps: int = 100, dt: float | None = None,
        courant: float = 0.5, cells: int = 1, init: str = "two_beam", seed: int = 0, device: int = 0,
        callback=None, gain: str = "pair"):
    """Relax `cells` homogeneous distributions for `steps` steps with the
    Courant step (or a fixed dt when given); returns the final f (numpy
    [n_pnt][cells]) and the per-step records."""
    import torch

    spec = GridSpec(grid, R=radius)
    ctx = Context(spec, device=device)
    ctx.set_gain_path(GAIN_PATHS[gain])
    g = spec.fill()
    f0 = inputs.two_beam(g, cells) if init == "two_beam" else inputs.mixtures(g, cells, seed=seed)
    f = torch.from_numpy(np.ascontiguousarray(f0)).cuda(device)
    m5 = torch.zeros((cells, 5), dtype=torch.float64, device=f.device)
    t = torch.zeros(1, dtype=torch.float32, device=f.device)
    mode, param = (DT_FIXED, dt) if dt is not None else (DT_COURANT, courant)
    records = []
    for k in range(steps + 1):
        time_now = float(t.item())
        if k < steps:
            ctx.step(f, cells, cells, mode, param, m5=m5, time=t)
        else:
            ctx.moments(f, cells, cells, m5)
        st = moments_to_state(m5.cpu().numpy())
        rec = {"step": k, "time": time_now, "n": st["n"].tolist(), "u": st["u"].tolist(),
               "E": st["E"].tolist(), "T": st["T"].tolist()}
        records.append(rec)
        if callback is not None:
            callback(rec, f)
    torch.cuda.synchronize()
    out = f.cpu().numpy()
    ctx.close()
    return out, records


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--grid", type=int, default=20)
    p.add_argument("--radius", type=float, default=4.8)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--dt", type=float, default=None, help="fixed step (default: Courant rule)")
    p.add_argument("--courant", type=float, default=0.5)
    p.add_argument("--cells", type=int, default=1)
    p.add_argument("--init", choices=["two_beam", "mixture"], default="two_beam")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--gain", choices=sorted(GAIN_PATHS), default="pair")
    a = p.parse_args(argv)
    _, recs = run(a.grid, a.radius, a.steps, a.dt, a.courant, a.cells, a.init, a.seed, gain=a.gain)
    for r in recs:
        print(json.dumps(r))
    return 0


if __name__ == "__main__":
    sys.exit(main())
