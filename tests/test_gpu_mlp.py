"""Surrogate network kernels (tcgen05 GEMMs, GELU epilogues, Adam) against the
FP64 oracle in oracle/mlp_ref.py with the same BF16 rounding points.

Tolerances: the GPU accumulates in FP32 in another order than numpy, and a
BF16 rounding of an intermediate may fall the other way, so outputs agree to
rel-L2 5e-4 and gradients to 2e-3; the un-emulated FP64 network differs by
3e-3 to 6e-3 in both, so these bounds do test the BF16 rounding points."""
import numpy as np
import pytest

from oracle import mlp_ref as M

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def _inputs(n_in, n_out, B, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.05, 1.0, (n_in, B)).astype(np.float32)
    t = rng.normal(0, 1.0, (n_out, B)).astype(np.float32)
    return x, t


@pytest.mark.parametrize("n_in,n_out,B,flags", [
    (200, 100, 192, M.SCALE_INPUT | M.SCALE_OUTPUT),   # M tail, N tail (128-wide output tile)
    (3648, 3648, 256, M.SCALE_INPUT | M.SCALE_OUTPUT),  # 20^3 lattice cut to R = 4.8
    (300, 1, 100, M.SCALE_INPUT | M.LOSS_MSE),           # error head shape
])
def test_forward_matches_oracle(gdlib, cuda, n_in, n_out, B, flags):
    torch = cuda
    net = gdlib.Mlp(n_in, n_out, batch_cap=256, flags=flags, seed=3)
    p = M.init_like_library(n_in, n_out, seed=5)
    net.set_params(p)
    x, _ = _inputs(n_in, n_out, B, 7)
    ld = B + 3
    xd = torch.zeros((n_in, ld), dtype=torch.float32, device="cuda")
    xd[:, :B] = torch.from_numpy(x).cuda()
    yd = torch.full((n_out, ld), float("nan"), dtype=torch.float32, device="cuda")
    net.forward(xd, ld, B, yd, ld)
    net.check()
    y = yd[:, :B].cpu().numpy()
    assert np.isnan(yd[:, B:].cpu().numpy()).all()      # nothing written past the batch
    layers = M.unpack(p, n_in, n_out)
    ref, _ = M.forward(layers, x, flags, bf16=True, n_out=n_out)
    assert _rel(y, ref) < 5e-4
    exact, _ = M.forward(layers, x, flags, bf16=False, n_out=n_out)
    assert _rel(y, exact) < 3e-2


@pytest.mark.parametrize("flags,gains", [(M.SCALE_INPUT | M.SCALE_OUTPUT, (1.0, 1.0)),
                                         (M.SCALE_INPUT | M.SCALE_OUTPUT | M.LOSS_BATCH, (0.3, 2.5))])
def test_gradients_match_oracle(gdlib, cuda, flags, gains):
    torch = cuda
    n_in, n_out, B = 200, 100, 128
    net = gdlib.Mlp(n_in, n_out, batch_cap=256, flags=flags, seed=3)
    net.set_io_scale(*gains)
    p = M.init_like_library(n_in, n_out, seed=11)
    net.set_params(p)
    x, t = _inputs(n_in, n_out, B, 12)
    tden = (2.0 * t + 0.5).astype(np.float32)
    xd, td, dd = (torch.from_numpy(a).cuda() for a in (x, t, tden))
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    net.train_step(xd, B, td, B, B, lr=0.0, loss=loss, tden=dd, ldd=B)
    net.check()
    g = net.get_grads()
    layers = M.unpack(p, n_in, n_out)
    ref_loss, _, ref = M.loss_and_grads(layers, x, t, flags, n_out, tden=tden, bf16=True, in_gain=gains[0],
                                        out_gain=gains[1])
    assert float(loss.item()) == pytest.approx(ref_loss, rel=2e-3)
    got = M.unpack(g, n_in, n_out)
    for k, ((gw, gb), (rw, rb)) in enumerate(zip(got, ref)):
        assert _rel(gw, rw) < 2e-3, f"layer {k} weights"
        assert _rel(gb, rb) < 2e-3, f"layer {k} bias"
    # lr = 0 leaves the parameters as they were
    np.testing.assert_array_equal(net.get_params(), p)


def test_adam_step(gdlib, cuda):
    torch = cuda
    n_in, n_out, B = 128, 64, 64
    flags = M.SCALE_INPUT | M.SCALE_OUTPUT
    net = gdlib.Mlp(n_in, n_out, batch_cap=64, flags=flags, seed=1)
    p0 = net.get_params()
    x, t = _inputs(n_in, n_out, B, 2)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    lr, wd = 1e-3, 1e-2
    net.train_step(xd, B, td, B, B, lr=lr, weight_decay=wd)
    net.check()
    g = net.get_grads().astype(np.float64)
    p1 = net.get_params().astype(np.float64)
    ref, _, _ = M.adam_update(p0.astype(np.float64), g, np.zeros_like(g), np.zeros_like(g), 1, lr, wd)
    live = np.abs(g) > 1e-5
    np.testing.assert_allclose(p1[live], ref[live], rtol=0, atol=1e-6)


def test_training_fits_a_linear_map(gdlib, cuda):
    """A few hundred Adam steps on the tensor-core kernels fit y = A x."""
    torch = cuda
    n_in, n_out, B = 256, 128, 512
    rng = np.random.default_rng(0)
    A = rng.normal(0, 1 / np.sqrt(n_in), (n_out, n_in)).astype(np.float32)
    x = rng.uniform(0.0, 1.0, (n_in, 4096)).astype(np.float32)
    t = A @ x
    net = gdlib.Mlp(n_in, n_out, batch_cap=B, flags=0, seed=4)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    row = torch.zeros(B, dtype=torch.float32, device="cuda")
    net.loss(xd, 4096, td, 4096, B, row)
    first = float(row.mean().item())
    for it in range(300):
        c0 = (it * B) % 4096
        net.train_step(xd[:, c0:], 4096, td[:, c0:], 4096, B, lr=1e-3)
    net.loss(xd, 4096, td, 4096, B, row)
    net.check()
    last = float(row.mean().item())
    assert last < 0.05 * first, (first, last)
