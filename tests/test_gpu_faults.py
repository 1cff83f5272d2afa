"""Failure handling injected on the host (no GPU fault): non-finite inputs and
singular systems reach the caller as a status from gd_ctx_check, a memory cap
makes object creation fail cleanly with GD_ERR_OUT_OF_MEMORY."""
import numpy as np
import pytest

from gpu_determ_gb300 import inputs

pytestmark = pytest.mark.gpu


def _setup(gd, torch, cells=64):
    spec = gd.GridSpec(12, R=4.8)
    ctx = gd.Context(spec)
    f = torch.from_numpy(inputs.mixtures(spec.fill(), cells, seed=4)).cuda()
    return ctx, f


def _q(ctx, f, cells, torch):
    nu, gain = torch.empty_like(f), torch.empty_like(f)
    q = torch.zeros(f.shape, dtype=torch.float64, device="cuda")
    ctx.collision(f, cells, cells, nu, gain)
    ctx.project(f, nu, gain, cells, cells, q=q)
    return q


def test_nonfinite_cell_is_reported(gdlib, cuda):
    torch = cuda
    ctx, f = _setup(gdlib, torch)
    q_ok = _q(ctx, f, 64, torch)
    ctx.check()                                  # clean so far
    bad = f.clone()
    bad[100, 5] = float("nan")
    bad[7, 9] = float("inf")
    q_bad = _q(ctx, bad, 64, torch)
    with pytest.raises(gdlib.GDError) as e:
        ctx.check()
    assert e.value.code == 5 and "first affected cell 5" in str(e.value)
    ctx.check()                                  # the record was cleared
    keep = [c for c in range(64) if c not in (5, 9)]
    assert torch.equal(q_bad[:, keep], q_ok[:, keep])   # the other cells are untouched


def test_empty_cell_is_not_an_error(gdlib, cuda):
    torch = cuda
    ctx, f = _setup(gdlib, torch)
    f[:, 3] = 0.0
    q = _q(ctx, f, 64, torch)
    ctx.check()
    assert torch.count_nonzero(q[:, 3]) == 0


def test_memory_limit(gdlib, cuda):
    torch = cuda
    ctx, f = _setup(gdlib, torch)
    try:
        gdlib.set_memory_limit(1 << 20)
        with pytest.raises(gdlib.GDError) as e:
            ctx.set_gain_path(gdlib.GAIN_CMATRIX_BF16)
        assert e.value.code == 3
        with pytest.raises(gdlib.GDError) as e:
            gdlib.Mlp(ctx.n_pnt, ctx.n_pnt, batch_cap=256)
        assert e.value.code == 3
        with pytest.raises(gdlib.GDError) as e:
            ctx.set_gain_path(gdlib.GAIN_PAIR_TC)      # its per-box weight table
        assert e.value.code == 3
        # the context keeps working on the pair kernel
        q = _q(ctx, f, 64, torch)
        ctx.check()
        assert torch.isfinite(q).all()
    finally:
        gdlib.set_memory_limit(0)
    ctx.set_gain_path(gdlib.GAIN_CMATRIX_BF16)
    ctx.check()
    ctx.set_gain_path(gdlib.GAIN_PAIR_TC)
    ctx.check()
