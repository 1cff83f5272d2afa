"""The FP64 surrogate oracle (oracle/mlp_ref.py) against finite differences,
and its BF16 emulation against the exact form (CPU only)."""
import numpy as np
import pytest

from oracle import mlp_ref as M


def _case(n_in=70, n_out=40, B=6, flags=M.SCALE_INPUT | M.SCALE_OUTPUT, seed=0):
    rng = np.random.default_rng(seed)
    p = M.init_like_library(n_in, n_out, seed).astype(np.float64)
    x = rng.uniform(0.1, 1.0, (n_in, B))
    t = rng.normal(0, 1, (n_out, B))
    return p, x, t, flags


def _loss(p, x, t, flags, n_in, n_out, tden=None, gains=(1.0, 1.0)):
    return M.loss_and_grads(M.unpack(p, n_in, n_out), x, t, flags, n_out, tden=tden, in_gain=gains[0],
                            out_gain=gains[1])[0]


@pytest.mark.parametrize("flags,gains", [(0, (1.0, 1.0)), (M.SCALE_INPUT, (1.0, 1.0)),
                                         (M.SCALE_INPUT | M.SCALE_OUTPUT, (1.0, 1.0)),
                                         (M.SCALE_INPUT | M.LOSS_MSE, (1.0, 1.0)),
                                         (M.SCALE_INPUT | M.SCALE_OUTPUT | M.LOSS_BATCH, (0.25, 3.0))])
def test_directional_derivatives(flags, gains):
    n_in, n_out = 70, 40
    p, x, t, _ = _case(n_in, n_out, flags=flags)
    layers = M.unpack(p, n_in, n_out)
    _, _, grads = M.loss_and_grads(layers, x, t, flags, n_out, in_gain=gains[0], out_gain=gains[1])
    g = M.pack(grads)
    rng = np.random.default_rng(1)
    # keep padded entries fixed, as the library does
    mask = np.concatenate([np.concatenate([(W != 0).ravel() | (k not in (0, 4)), np.ones(b.size, bool)])
                           for k, (W, b) in enumerate(layers)])
    for _ in range(4):
        d = rng.normal(0, 1, p.size) * mask
        eps = 1e-5
        num = (_loss(p + eps * d, x, t, flags, n_in, n_out, gains=gains)
               - _loss(p - eps * d, x, t, flags, n_in, n_out, gains=gains)) / (2 * eps)
        ana = float(g @ d)
        assert abs(num - ana) <= 1e-6 * max(1.0, abs(ana)), (num, ana)


def test_tden_denominator():
    n_in, n_out = 70, 40
    p, x, t, flags = _case(n_in, n_out)
    tden = 3.0 * t
    l1 = _loss(p, x, t, flags, n_in, n_out)
    l2 = _loss(p, x, t, flags, n_in, n_out, tden=tden)
    assert l2 == pytest.approx(l1 / 9.0, rel=1e-12)


def test_output_scaling_is_quadratic():
    n_in, n_out = 70, 40
    p, x, _, flags = _case(n_in, n_out)
    layers = M.unpack(p, n_in, n_out)
    y1, _ = M.forward(layers, x, flags)
    y2, _ = M.forward(layers, 2.5 * x, flags)
    np.testing.assert_allclose(y2, 6.25 * y1, rtol=1e-12)


def test_bf16_rounding():
    a = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7 + 2 ** -8, -3.14159, 0.0, 1e-20])
    r = M.bf16_round(a)
    assert r[0] == 1.0 and r[1] == 1.0                 # tie to even (down)
    assert r[2] == 1.0 + 2 ** -6                       # tie to even (up)
    assert r[3] == -3.140625 and r[4] == 0.0
    assert abs(r[5] - 1e-20) <= 1e-20 * 2 ** -8
    # the emulated network stays close to the exact one
    n_in, n_out = 70, 40
    p, x, _, flags = _case(n_in, n_out)
    layers = M.unpack(p, n_in, n_out)
    y, _ = M.forward(layers, x, flags)
    yb, _ = M.forward(layers, x, flags, bf16=True)
    assert np.linalg.norm(yb - y) / np.linalg.norm(y) < 2e-2


def test_adam_first_step_is_sign_descent():
    g = np.array([1e-3, -2.0, 5e-2])
    p, m, v = M.adam_update(np.zeros(3), g, np.zeros(3), np.zeros(3), 1, lr=0.01)
    np.testing.assert_allclose(p, -0.01 * np.sign(g), rtol=1e-4)
