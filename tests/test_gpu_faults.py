"""Failure handling injected on the host (no GPU fault): non-finite inputs and
singular systems reach the caller as a status from gd_ctx_check, a memory cap
makes object creation fail cleanly with GD_ERR_OUT_OF_MEMORY, and a bounded
device wait that is made to run out (an mbarrier that nothing arrives at,
waited on before any copy or MMA is issued) is reported once by the check,
leaves the tensor memory free, and the next call is bitwise the clean one."""
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


def test_timed_out_wait_on_context_is_reported_once(gdlib, cuda):
    """The collision calls only enqueue work on the tensor-core path; a timed
    out pipeline wait of the tensor-core loss GEMM reaches the caller through
    gd_ctx_check, which clears it."""
    torch = cuda
    ctx, f = _setup(gdlib, torch)      # 64 cells: one CTA per tensor-core MMA
    ctx.set_gain_path(gdlib.GAIN_CMATRIX_BF16)
    nu0, g0 = torch.empty_like(f), torch.empty_like(f)
    ctx.collision(f, 64, 64, nu0, g0)
    ctx.check()
    ctx.inject_timeout(256)
    nu1, g1 = torch.empty_like(f), torch.empty_like(f)
    ctx.collision(f, 64, 64, nu1, g1)  # enqueues; reports nothing itself
    with pytest.raises(gdlib.GDError) as e:
        ctx.check()
    assert e.value.code == 2 and "timed out" in str(e.value)
    ctx.check()                        # the record was cleared
    nu2, g2 = torch.empty_like(f), torch.empty_like(f)
    ctx.collision(f, 64, 64, nu2, g2)  # a new tcgen05 allocation succeeds: the stalled CTAs freed theirs
    ctx.check()
    assert torch.equal(nu2, nu0) and torch.equal(g2, g0)
    with pytest.raises(gdlib.GDError):
        ctx.inject_timeout(0)
    ctx.set_gain_path(gdlib.GAIN_PAIR)
    with pytest.raises(gdlib.GDError) as e:
        ctx.inject_timeout(256)        # the FP32 path has no tensor-core wait to stall
    assert e.value.code == 4


def test_timed_out_wait_on_network_is_reported_once(gdlib, cuda):
    torch = cuda
    ctx, f = _setup(gdlib, torch)
    net = gdlib.Mlp(ctx.n_pnt, ctx.n_pnt, batch_cap=64)
    y0 = torch.empty_like(f)
    net.forward(f, 64, 64, y0, 64)
    net.check()
    net.inject_timeout(256)
    y1 = torch.empty_like(f)
    net.forward(f, 64, 64, y1, 64)
    with pytest.raises(gdlib.GDError) as e:
        net.check()
    assert e.value.code == 2 and "timed out" in str(e.value)
    net.check()
    y2 = torch.empty_like(f)
    net.forward(f, 64, 64, y2, 64)
    net.check()
    assert torch.equal(y2, y0)
