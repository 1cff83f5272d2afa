"""Surrogate gain with plain fallback (gd_surrogate_gain) on a 12^3 lattice.

The error network is given hand-set parameters so that its estimate is a
known function of f (est = f at one node), which fixes which cells fall back;
fallback cells must then carry exactly the plain gain of the same gathered
block, the others the network's Q plus nu f."""
import numpy as np
import pytest

from oracle import mlp_ref as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(gdlib, cuda):
    torch = cuda
    spec = gdlib.GridSpec(12, R=4.8)
    ctx = gdlib.Context(spec)
    grid = spec.fill()
    from gpu_determ_gb300 import inputs
    f = torch.from_numpy(inputs.dirichlet_mixtures(grid, 256, seed=5)).cuda()
    return gdlib, ctx, grid, f


def _selector_est(gdlib, n, node, cap):
    """est(f) = f[node] (flags 0): W0 row 0 picks the node, W4[0][0] = 1."""
    est = gdlib.Mlp(n, 1, batch_cap=cap, flags=0, seed=0)
    layers = [(np.zeros((o, i)), np.zeros(o)) for o, i in M.layer_shapes(n, 1)]
    layers[0][0][0, node] = 1.0
    layers[4][0][0, 0] = 1.0
    est.set_params(M.pack(layers).astype(np.float32))
    return est


def test_tol_zero_is_the_plain_method(setup, cuda):
    gd, ctx, grid, f = setup
    torch = cuda
    n, N = f.shape
    net = gd.Mlp(n, n, batch_cap=256, seed=1)
    s = gd.Surrogate(ctx, net, None, 256)
    nu, gain = torch.empty_like(f), torch.empty_like(f)
    assert s.gain(f, N, N, 0.0, nu, gain) == N
    nu_p, gain_p = torch.empty_like(f), torch.empty_like(f)
    ctx.collision(f, N, N, nu_p, gain_p)
    torch.cuda.synchronize()
    assert torch.equal(gain, gain_p) and torch.equal(nu, nu_p)


def test_fallback_split(setup, cuda):
    gd, ctx, grid, f = setup
    torch = cuda
    n, N = f.shape
    node = int(np.argmax(np.asarray(f[:, 0].cpu())))
    net = gd.Mlp(n, n, batch_cap=256, seed=2)
    est = _selector_est(gd, n, node, 256)
    s = gd.Surrogate(ctx, net, est, 256)
    vals = f[node, :].cpu().numpy()
    thr = float(np.median(vals))
    nu, gain = torch.empty_like(f), torch.empty_like(f)
    est_out = torch.empty(N, dtype=torch.float32, device="cuda")
    nfb = s.gain(f, N, N, 10.0 ** thr, nu, gain, est_out)
    torch.cuda.synchronize()
    e = est_out.cpu().numpy()
    np.testing.assert_allclose(e, M.bf16_round(vals), rtol=1e-6)
    fb = np.nonzero(~(e <= np.float32(np.log10(np.float32(10.0 ** thr)))))[0]
    assert nfb == len(fb) and 0 < nfb < N
    # fallback cells: the plain gain of the gathered block
    idx = torch.from_numpy(fb).cuda()
    fs = f[:, idx].contiguous()
    gs = torch.empty_like(fs)
    ctx.collision(fs, nfb, nfb, None, gs)
    # other cells: network Q + nu f
    q_net = torch.empty_like(f)
    net.forward(f, N, N, q_net, N)
    nu_p = torch.empty_like(f)
    ctx.collision(f, N, N, nu_p, None)
    torch.cuda.synchronize()
    assert torch.equal(nu, nu_p)
    assert torch.equal(gain[:, idx], gs)
    keep = torch.from_numpy(np.setdiff1d(np.arange(N), fb)).cuda()
    ref = q_net[:, keep] + nu_p[:, keep] * f[:, keep]
    assert torch.allclose(gain[:, keep], ref, rtol=1e-6, atol=1e-7)


def test_cell_rel_l2(gdlib, cuda):
    torch = cuda
    rng = np.random.default_rng(0)
    a = rng.normal(size=(50, 7))
    b = rng.normal(size=(50, 7))
    out = torch.empty(7, dtype=torch.float64, device="cuda")
    A, B = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    gdlib.cell_rel_l2(A, 7, B, 7, 50, 7, out)
    ref = np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-12)


def test_all_cells_fall_back(setup, cuda):
    """An estimate above tolerance everywhere sends every cell to the plain
    path, which then runs in place: the gain is bitwise the plain gain."""
    gd, ctx, grid, f = setup
    torch = cuda
    n, N = f.shape
    net = gd.Mlp(n, n, batch_cap=256, seed=4)
    est = gd.Mlp(n, 1, batch_cap=256, flags=0, seed=0)
    layers = [(np.zeros((o, i)), np.zeros(o)) for o, i in M.layer_shapes(n, 1)]
    layers[4][1][0] = 5.0          # estimate log10(error) = 5 for every cell
    est.set_params(M.pack(layers).astype(np.float32))
    s = gd.Surrogate(ctx, net, est, 256)
    nu, gain = torch.empty_like(f), torch.empty_like(f)
    assert s.gain(f, N, N, 1e-3, nu, gain) == N
    gain_p = torch.empty_like(f)
    ctx.collision(f, N, N, None, gain_p)
    torch.cuda.synchronize()
    assert torch.equal(gain, gain_p)
