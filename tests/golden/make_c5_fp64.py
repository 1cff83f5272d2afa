"""Generate c5_fp64_cells.npz: FP64 collision integrals of four cells of the
32^3 cavity-field batch, for the GPU test that states the 32^3 paths' error
against FP64.

    python tests/golden/make_c5_fp64.py      # ~5 min on 8 cores

Lattice 32^3 on [-5,5]^3 cut to R = 5.5 (21 992 nodes).  Cells: the
Maxwellians M(1, u_c, T_c) of inputs.cavity_field for the 16 384-cell batch
(seed 0), cells 0, 5461, 10922 and 16383 (a corner, two interior cells and the
opposite corner of the 128 x 128 cell grid).  For each: the oracle's FP64 loss
nu and gain I (collision_integral.cu:32-72, 75-188 restated in oracle.c), then
the conservation projection in FP64 (Oracle.project_f64).

Outputs (npz): f [n][4] float32 (the inputs, so the test does not regenerate
them), q [n][4] float64, gain [n][4] float64, cells [4] int64.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gpu_determ_gb300 import inputs  # noqa: E402
from oracle.pyoracle import Oracle  # noqa: E402

CELLS = (0, 5461, 10922, 16383)
BATCH = 16384


def main():
    o = Oracle(32, R=5.5)
    g = {"u": o.u, "v": o.v, "w": o.w, "ui": o.ui, "vi": o.vi, "wi": o.wi}
    vel, T = inputs.cavity_field_params(BATCH, seed=0)
    xu, xv, xw = inputs.node_velocities(g)
    f = np.empty((o.n_pnt, len(CELLS)), np.float32)
    for k, c in enumerate(CELLS):
        c2 = (xu - vel[c, 0]) ** 2 + (xv - vel[c, 1]) ** 2 + (xw - vel[c, 2]) ** 2
        f[:, k] = (np.pi * T[c]) ** -1.5 * np.exp(-c2 / T[c])
    fb = o.to_box(f)
    nu = o.loss_f64(fb)
    gain = o.gain_f64(fb)
    q = o.project_f64(f, nu, gain)
    out = os.path.join(HERE, "c5_fp64_cells.npz")
    np.savez_compressed(out, f=f, q=q, gain=gain, cells=np.asarray(CELLS, np.int64))
    print("wrote", out, "n_pnt", o.n_pnt)


if __name__ == "__main__":
    main()
