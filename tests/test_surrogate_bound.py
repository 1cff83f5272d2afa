"""How close a surrogate built on the operator's bilinear structure can get.

A latent bilinear form I_hat_i = z^T H_i z over a linear encoding z = E f of
rank r equals, at best, the exact gain of f's projection onto E's row space
(H_i = P^T G_i P for an orthonormal basis P of that space, G_i the collision
matrix of node i).  Over a fixed training distribution the best rank-r space
for f is its principal subspace.  This test computes that bound on the CPU
with the oracle: the principal basis of the training mixtures (weights
Dirichlet(1), u ~ N(0, I), T ~ U[0.5, 2]), the exact gain of each held-out f
projected onto it, the exact loss of f and the FP64 conservation projection,
against the exact Q of 64 held-out mixtures of the same distribution.

At 12^3, R = 4.8 (840 nodes) no held-out cell is within the 1e-3 per-cell
tolerance at a quarter of the lattice's dimension, and few are at half, where
the form's r (r + 1) / 2 multiply-adds per node and cell already outnumber the
exact operator's terms (the reference's (i, i1, n) enumeration, per node):
the cancellation in Q = I - f nu asks the gain to be right to ~1e-5 relative
for typical cells, which a rank-r encoding of these narrow, shifted
Maxwellians does not give.  At full rank the same pipeline reproduces Q,
which checks the construction.

GD_BOUND_GRID=20 runs the same computation at 20^3 (16 000 training
mixtures) and prints its figures without the 12^3 thresholds."""
import os

import numpy as np

from gpu_determ_gb300 import inputs
from oracle.pyoracle import Oracle


def _q(o, f, nu, gain):
    _, q, _, _ = o.project(f, nu.astype(np.float32), gain.astype(np.float32))
    return q


def test_principal_subspace_bilinear_bound():
    grid = int(os.environ.get("GD_BOUND_GRID", "12"))
    o = Oracle(grid, R=4.8)
    g = {"u": o.u, "v": o.v, "w": o.w, "ui": o.ui, "vi": o.vi, "wi": o.wi}
    n = o.n_pnt
    train = inputs.dirichlet_mixtures(g, 4000 if grid <= 12 else 16000, seed=101).astype(np.float64)
    test = inputs.dirichlet_mixtures(g, 64, seed=202)
    _, V = np.linalg.eigh(train @ train.T)
    V = V[:, ::-1]

    nu = o.loss_f64(o.to_box(test))
    q = _q(o, test, nu, o.gain_f64(o.to_box(test)))
    qn = np.linalg.norm(q, axis=0)

    within, median = {}, {}
    for r in (n // 8, n // 4, n // 2, n):
        P = V[:, :r]
        fh = (P @ (P.T @ test.astype(np.float64))).astype(np.float32)
        qh = _q(o, test, nu, o.gain_f64(o.to_box(fh)))
        err = np.linalg.norm(qh - q, axis=0) / qn
        within[r] = float((err <= 1e-3).mean())
        median[r] = float(np.median(err))
    print("%d^3, %d nodes: rank -> (fraction of cells within 1e-3, median per-cell error) %s"
          % (grid, n, {r: (within[r], round(median[r], 6)) for r in within}))
    assert within[n] == 1.0, within
    half = n // 2
    assert half * (half + 1) // 2 > o.count_work()["terms"] / n
    assert median[n // 8] > median[n // 4] > median[n // 2]
    if grid == 12:
        assert within[n // 8] == 0.0 and within[n // 4] == 0.0, within
        assert within[n // 2] <= 0.2 and median[n // 2] > 1e-3, (within, median)
