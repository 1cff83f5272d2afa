"""FP64 numpy restatement of the surrogate network, its loss and its gradients.

Test infrastructure only: the tests use it as the oracle for the tensor-core
training and inference kernels (gd_mlp_* in libgpu_determ.so); nothing in the
library calls it.  The surrogate has no counterpart in the reference, so this
restatement is pinned by finite differences (tests/test_mlp_oracle.py), not by
reference vectors.

Network on one cell x (features in the compact node order), padded feature
counts n_in_p = 64 * ceil(n_in / 64), n_out_p likewise:
    h0 = W0 x + b0,            h1 = GELU(W1 h0 + b1),  h2 = GELU(W2 h1 + b2),
    z  = W3 h2 + b3 + h0,      y  = W4 z + b4
with GELU(a) = a/2 (1 + erf(a / sqrt 2)).  With scale_input each cell's x is
divided by its mean over the n_in features (s); with scale_output y is
multiplied by s^2 and the targets divided by s^2.  Global gains: the scaled
input is multiplied by in_gain, the network output by out_gain (targets divided
by it).  Loss: mean over the batch of sum_i (y_i - t_i)^2 / den, den =
sum_i tden_i^2 (relative), its batch mean (batch-relative) or n_out (mse).

``bf16=True`` rounds to BF16 (nearest even) exactly where the GPU kernels hold
BF16 copies: the network input, the weights, the GEMM inputs h0, h1, h2, z and
the back-propagated dy, dz, da2, da1, dh0.
"""
from __future__ import annotations

import math

import numpy as np

try:
    from scipy.special import erf as _erf
except ImportError:  # pragma: no cover - scipy is present wherever the tests run
    _erf = np.vectorize(math.erf)

SCALE_INPUT, SCALE_OUTPUT, LOSS_MSE, LOSS_BATCH = 1, 2, 4, 8


def pad64(n: int) -> int:
    return (n + 63) // 64 * 64


def layer_shapes(n_in: int, n_out: int):
    return [(256, pad64(n_in)), (512, 256), (512, 512), (256, 512), (pad64(n_out), 256)]


def unpack(params: np.ndarray, n_in: int, n_out: int):
    """Flat FP32 block (W_k [out][in] then b_k per layer) -> [(W, b)] in FP64."""
    out, off = [], 0
    for o, i in layer_shapes(n_in, n_out):
        W = params[off:off + o * i].reshape(o, i).astype(np.float64)
        off += o * i
        b = params[off:off + o].astype(np.float64)
        off += o
        out.append((W, b))
    assert off == params.size
    return out


def pack(layers) -> np.ndarray:
    return np.concatenate([np.concatenate([W.ravel(), b]) for W, b in layers])


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as FP64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(a):
    return 0.5 * a * (1.0 + _erf(a / math.sqrt(2.0)))


def gelu_grad(a):
    return 0.5 * (1.0 + _erf(a / math.sqrt(2.0))) + a * np.exp(-0.5 * a * a) / math.sqrt(2.0 * math.pi)


def cell_scales(x: np.ndarray, flags: int) -> np.ndarray:
    """x is [n_in][B] (library layout); per-cell mean, or ones."""
    if flags & SCALE_INPUT:
        return x.astype(np.float64).mean(axis=0)
    return np.ones(x.shape[1])


def _inv(s):
    return np.where(s != 0, 1.0 / np.where(s != 0, s, 1.0), 0.0)


def forward(layers, x: np.ndarray, flags: int, bf16: bool = False, n_out: int | None = None,
            in_gain: float = 1.0, out_gain: float = 1.0):
    """x [n_in][B] -> (y [n_out][B] in the caller's units, cache); without
    n_out the padded outputs are returned too."""
    r = bf16_round if bf16 else (lambda a: a)
    n_in, B = x.shape
    (W0, b0), (W1, b1), (W2, b2), (W3, b3), (W4, b4) = [(r(W), b) for W, b in layers]
    s = cell_scales(x, flags)
    X = np.zeros((B, W0.shape[1]))
    X[:, :n_in] = x.T.astype(np.float64) * (_inv(s) * np.float32(in_gain))[:, None]
    X = r(X)
    h0 = X @ W0.T + b0
    h0b = r(h0)
    a1 = h0b @ W1.T + b1
    h1b = r(gelu(a1))
    a2 = h1b @ W2.T + b2
    h2b = r(gelu(a2))
    z = h2b @ W3.T + b3 + h0
    zb = r(z)
    y = zb @ W4.T + b4
    cache = dict(X=X, h0b=h0b, a1=a1, h1b=h1b, a2=a2, h2b=h2b, zb=zb, y=y, s=s,
                 W=(W0, W1, W2, W3, W4))
    out = (y.T if n_out is None else y[:, :n_out].T) * float(np.float32(out_gain))
    if flags & SCALE_OUTPUT:
        out *= (s * s)[None, :]
    return out, cache


def loss_and_grads(layers, x, t, flags: int, n_out: int, tden=None, bf16: bool = False, in_gain: float = 1.0,
                   out_gain: float = 1.0):
    """Mean loss and the gradients [(dW, db)] of the training step.

    x [n_in][B], t [n_out][B] (and tden) in the library layout."""
    r = bf16_round if bf16 else (lambda a: a)
    _, c = forward(layers, x, flags, bf16, in_gain=in_gain)
    B = x.shape[1]
    y = c["y"]
    n_out_p = y.shape[1]
    s = c["s"]
    tt = np.zeros((B, n_out_p))
    tt[:, :n_out] = t.T.astype(np.float64)
    dd = (t if tden is None else tden).T.astype(np.float64)
    f2 = (_inv(s * s) if flags & SCALE_OUTPUT else np.ones(B))[:, None] / float(np.float32(out_gain))
    tt[:, :n_out] *= f2
    dd = dd * f2
    den = np.full(B, float(n_out)) if flags & LOSS_MSE else np.sum(dd * dd, axis=1)
    if flags & LOSS_BATCH and not flags & LOSS_MSE:
        den = np.full(B, den.mean())
    den = np.maximum(den, 1e-30)
    diff = y - tt
    diff[:, n_out:] = 0.0
    row = np.sum(diff * diff, axis=1) / den
    loss = float(row.mean())
    dy = 2.0 * diff / den[:, None] / B
    W0, W1, W2, W3, W4 = c["W"]
    dyb = r(dy)
    g4 = (dyb.T @ c["zb"], dy.sum(axis=0))
    dz = dyb @ W4
    dzb = r(dz)
    g3 = (dzb.T @ c["h2b"], dz.sum(axis=0))
    da2 = (dzb @ W3) * gelu_grad(c["a2"])
    da2b = r(da2)
    g2 = (da2b.T @ c["h1b"], da2.sum(axis=0))
    da1 = (da2b @ W2) * gelu_grad(c["a1"])
    da1b = r(da1)
    g1 = (da1b.T @ c["h0b"], da1.sum(axis=0))
    dh0 = da1b @ W1 + dz
    dh0b = r(dh0)
    g0 = (dh0b.T @ c["X"], dh0.sum(axis=0))
    return loss, row, [g0, g1, g2, g3, g4]


def adam_update(p, g, m, v, step, lr, wd=0.0, b1=0.9, b2=0.999, eps=1e-8):
    """One decoupled-weight-decay Adam step on flat arrays (returns p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    p = p - lr * ((m / c1) / (np.sqrt(v / c2) + eps) + wd * p)
    return p, m, v


def init_like_library(n_in: int, n_out: int, seed: int) -> np.ndarray:
    """Parameter block with random weights drawn by numpy (tests only; the
    library draws its own from an LCG)."""
    rng = np.random.default_rng(seed)
    layers = []
    for k, (o, i) in enumerate(layer_shapes(n_in, n_out)):
        fan = n_in if k == 0 else i
        W = rng.uniform(-1, 1, (o, i)) / math.sqrt(fan)
        if k == 0:
            W[:, n_in:] = 0
        if k == 4:
            W[n_out:, :] = 0
        b = rng.normal(0, 0.05, o)
        if k == 4:
            b[n_out:] = 0
        layers.append((W, b))
    return pack(layers).astype(np.float32)
