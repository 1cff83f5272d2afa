"""Pair-product gain with the weight contraction on the tensor cores
(GD_GAIN_PAIR_TC): pair products and weights split into BF16 hi + lo,
P_hi W_hi + P_hi W_lo + P_lo W_hi accumulated in FP32.  Checked against the
FP64 oracle (small grids) and the FP32 pair kernel (the 24^3 grid, whose
largest class boxes hold more than 256 row groups and run in two passes);
stated tolerance: relative L2 of I over all nodes and cells <= 2e-5."""
import numpy as np
import pytest

from gpu_determ_gb300 import inputs
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def _gain(gd, ctx, path, ft, nc, ld, torch):
    ctx.set_gain_path(path)
    out = torch.full_like(ft, -1.0)
    ctx.collision(ft, nc, ld, None, out)
    torch.cuda.synchronize()
    return out


@pytest.mark.parametrize("n,R,nc,ld", [(8, 16.5, 40, 40), (12, 4.8, 200, 203), (16, 4.8, 300, 300)])
def test_pair_tc_matches_oracle(cuda, gdlib, n, R, nc, ld):
    torch = cuda
    spec = gdlib.GridSpec(n, R=R)
    ctx = gdlib.Context(spec)
    f = inputs.dirichlet_mixtures(spec.fill(), nc, seed=n + 3)
    ft = torch.zeros((ctx.n_pnt, ld), dtype=torch.float32, device="cuda")
    ft[:, :nc] = torch.from_numpy(f).cuda()
    out = _gain(gdlib, ctx, gdlib.GAIN_PAIR_TC, ft, nc, ld, torch)
    again = _gain(gdlib, ctx, gdlib.GAIN_PAIR_TC, ft, nc, ld, torch)
    assert torch.equal(out, again)                      # bitwise reproducible
    assert bool((out[:, nc:] == -1.0).all())            # padding columns untouched
    got = out[:, :nc].cpu().numpy().astype(np.float64)
    if n <= 12:
        o = Oracle(n, R=R)
        ref = o.gain_f64(o.to_box(f))
    else:
        ref = _gain(gdlib, ctx, gdlib.GAIN_PAIR, ft, nc, ld, torch)[:, :nc].cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel <= 2e-5, rel
    ctx.check()


def test_pair_tc_two_passes_at_24cube(cuda, gdlib):
    """24^3 (6272 nodes): boxes with up to 412 row groups take two passes of
    at most 256; the result matches the FP32 pair kernel."""
    torch = cuda
    spec = gdlib.GridSpec(24, R=4.8)
    ctx = gdlib.Context(spec)
    nc = 130
    ft = torch.from_numpy(inputs.dirichlet_mixtures(spec.fill(), nc, seed=24)).cuda()
    ref = _gain(gdlib, ctx, gdlib.GAIN_PAIR, ft, nc, nc, torch)
    out = _gain(gdlib, ctx, gdlib.GAIN_PAIR_TC, ft, nc, nc, torch)
    rel = float((out - ref).norm() / ref.norm())
    assert rel <= 2e-5, rel
    ctx.check()


def test_pair_tc_step_conserves(cuda, gdlib):
    """gd_step on the tensor-core pair path: FP64 projection, Courant step;
    moments of f change only at its FP32 rounding."""
    torch = cuda
    spec = gdlib.GridSpec(12, R=4.8)
    ctx = gdlib.Context(spec)
    ctx.set_gain_path(gdlib.GAIN_PAIR_TC)
    nc = 96
    f = torch.from_numpy(inputs.mixtures(spec.fill(), nc, seed=9)).cuda()
    m0 = torch.zeros((nc, 5), dtype=torch.float64, device="cuda")
    m1 = torch.zeros_like(m0)
    ctx.moments(f, nc, nc, m0)
    t = torch.zeros(1, dtype=torch.float32, device="cuda")
    for _ in range(3):
        ctx.step(f, nc, nc, gdlib.DT_COURANT, 0.5, time=t)
    ctx.moments(f, nc, nc, m1)
    ctx.check()
    torch.cuda.synchronize()
    d = (m1 - m0).abs().max(dim=0).values
    scale = m0.abs().max(dim=0).values
    assert float(d[0] / scale[0]) < 1e-5 and float(d[4] / scale[4]) < 1e-5
    assert float(t.item()) > 0


def test_autotune_includes_pair_tc(cuda, gdlib):
    torch = cuda
    spec = gdlib.GridSpec(12, R=4.8)
    ctx = gdlib.Context(spec)
    nc = 128
    f = torch.from_numpy(inputs.mixtures(spec.fill(), nc, seed=4)).cuda()
    mask = (1 << gdlib.GAIN_PAIR) | (1 << gdlib.GAIN_PAIR_TC)
    r = ctx.autotune(f, nc, nc, path_mask=mask, mem_budget=8e9)
    paths = [c["path"] for c in r["candidates"]]
    assert paths.count("pair") == 3 and paths.count("pair_tc") == 1
    assert all(c["ms"] > 0 for c in r["candidates"])
    assert r["best_ms"] == pytest.approx(min(c["ms"] for c in r["candidates"]))


@pytest.mark.parametrize("nc,ld", [(1, 1), (129, 136)])
def test_pair_tc_edge_cell_counts(cuda, gdlib, nc, ld):
    """One cell, and one cell past a 128-cell tile (a nearly empty second
    tile), with a leading dimension past the cells: the FP32 kernel's gain to
    2e-5 and untouched padding columns."""
    torch = cuda
    spec = gdlib.GridSpec(8, R=16.5)
    ctx = gdlib.Context(spec)
    ft = torch.zeros((ctx.n_pnt, ld), dtype=torch.float32, device="cuda")
    ft[:, :nc] = torch.from_numpy(inputs.mixtures(spec.fill(), nc, seed=nc)).cuda()
    ref = _gain(gdlib, ctx, gdlib.GAIN_PAIR, ft, nc, ld, torch)
    out = _gain(gdlib, ctx, gdlib.GAIN_PAIR_TC, ft, nc, ld, torch)
    assert bool((out[:, nc:] == -1.0).all())
    rel = float((out[:, :nc] - ref[:, :nc]).norm() / ref[:, :nc].norm())
    assert rel <= 2e-5, rel
    ctx.check()


def test_pair_tc_fixed_point_scale_is_exact(cuda, gdlib):
    """Each cell's outputs accumulate in 64-bit fixed point scaled by a power
    of two set from its own max|f|: scaling a cell's f by 2^e shifts its scale
    exponent by -2e, so its gain is the unscaled gain times 2^(2e), bit for
    bit (while every value stays a normal float), and the other cells do not
    change.  A cell with a non-finite f gets NaN outputs and leaves the others
    untouched."""
    torch = cuda
    spec = gdlib.GridSpec(12, R=4.8)
    ctx = gdlib.Context(spec)
    nc = 160
    f = torch.from_numpy(inputs.dirichlet_mixtures(spec.fill(), nc, seed=5)).cuda()
    base = _gain(gdlib, ctx, gdlib.GAIN_PAIR_TC, f, nc, nc, torch)
    g = f.clone()
    g[:, 3] *= 2.0 ** 20
    g[:, 7] *= 2.0 ** -8
    g[5, 11] = float("nan")
    g[9, 140] = float("inf")
    out = _gain(gdlib, ctx, gdlib.GAIN_PAIR_TC, g, nc, nc, torch)
    assert torch.equal(out[:, 3], base[:, 3] * 2.0 ** 40)
    assert torch.equal(out[:, 7], base[:, 7] * 2.0 ** -16)
    assert bool(torch.isnan(out[:, 11]).all()) and bool(torch.isnan(out[:, 140]).all())
    keep = [c for c in range(nc) if c not in (3, 7, 11, 140)]
    assert torch.equal(out[:, keep], base[:, keep])
    ctx.check()
