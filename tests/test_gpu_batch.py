"""Batches of uneven grids (gd_batch_*) and the autotuner (gd_ctx_autotune).

Steps of a batch, eager or replayed from the captured CUDA graph, must give
bitwise the same distributions and times as stepping each group alone with
gd_step: the graph holds the same launches in the same order per context."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 4


def _groups(gd, torch):
    from gpu_determ_gb300 import inputs
    out = []
    for n, cells, seed in ((8, 64, 1), (12, 96, 2)):
        spec = gd.GridSpec(n, R=4.8)
        ctx = gd.Context(spec)
        g = spec.fill()
        out.append((ctx, inputs.shock_profile(g, cells), cells))
        out.append((ctx, inputs.mixtures(g, 40, seed=seed), 40))   # second group on the same context
    return out


def _run_single(gd, torch, groups):
    fs, ts = [], []
    for ctx, f0, cells in groups:
        f = torch.from_numpy(f0).cuda()
        t = torch.zeros(1, dtype=torch.float32, device="cuda")
        for _ in range(STEPS):
            ctx.step(f, cells, cells, gd.DT_COURANT, 0.5, time=t)
        fs.append(f)
        ts.append(t)
    torch.cuda.synchronize()
    return [f.cpu().numpy() for f in fs], [float(t.item()) for t in ts]


def _run_batch(gd, torch, groups, use_graph):
    b = gd.Batch()
    fs, ts, ms = [], [], []
    for ctx, f0, cells in groups:
        f = torch.from_numpy(f0).cuda()
        t = torch.zeros(1, dtype=torch.float32, device="cuda")
        m5 = torch.zeros((cells, 5), dtype=torch.float64, device="cuda")
        b.add(ctx, f, cells, cells, gd.DT_COURANT, 0.5, m5=m5, time=t)
        fs.append(f)
        ts.append(t)
        ms.append(m5)
    for _ in range(STEPS):
        b.step(use_graph)
    b.check()
    info = b.info()
    b.close()
    return [f.cpu().numpy() for f in fs], [float(t.item()) for t in ts], info


def test_batch_matches_single_steps(gdlib, cuda):
    torch = cuda
    groups = _groups(gdlib, torch)
    f_ref, t_ref = _run_single(gdlib, torch, groups)
    for use_graph in (False, True):
        f_b, t_b, info = _run_batch(gdlib, torch, groups, use_graph)
        assert info["groups"] == 4 and info["streams"] == 2 and info["steps"] == STEPS
        if use_graph:
            assert info["graph_nodes"] > 0
        for a, b in zip(f_ref, f_b):
            assert np.array_equal(a, b)
        assert t_ref == t_b
    assert all(t > 0 for t in t_ref)


def test_autotune_picks_a_measured_candidate(gdlib, cuda):
    torch = cuda
    from gpu_determ_gb300 import inputs
    spec = gdlib.GridSpec(12, R=4.8)
    ctx = gdlib.Context(spec)
    g = spec.fill()
    cells = 128
    f = torch.from_numpy(inputs.mixtures(g, cells, seed=3)).cuda()
    ref = torch.empty_like(f)
    ctx.collision(f, cells, cells, None, ref)
    mask = (1 << gdlib.GAIN_PAIR) | (1 << gdlib.GAIN_CMATRIX_BF16X3)
    r = ctx.autotune(f, cells, cells, path_mask=mask, mem_budget=8e9)
    ms = [c["ms"] for c in r["candidates"]]
    assert len(ms) == 5 and all(m > 0 for m in ms)   # pair x 3 fills, BF16x3 matrices x 2 cluster sizes
    assert r["best_ms"] == pytest.approx(min(ms))
    gain = torch.empty_like(f)
    ctx.collision(f, cells, cells, None, gain)
    torch.cuda.synchronize()
    rel = float((gain - ref).norm() / ref.norm())
    assert rel < (1e-5 if r["path"] == "cmatrix_bf16x3" else 1e-6)
    # a budget too small for the matrices leaves only the pair kernel
    r2 = ctx.autotune(f, cells, cells, path_mask=mask, mem_budget=1e3)
    assert r2["path"] == "pair" and len(r2["candidates"]) == 3


@pytest.mark.parametrize("mode", ["pair_tc", "cmatrix"])
def test_fused_batch_one_launch_matches_single_steps(gdlib, cuda, mode):
    """The gains of uneven grids (8^3, 12^3, 16^3 with 130-300 cells, so some
    grids have more than one 128-cell tile) come from one launch per step:
    GD_BATCH_FUSED_PAIR_TC, the persistent pair-product kernel over a device
    list of (grid, cell tile, s-chunk) units; GD_BATCH_FUSED_CMATRIX, the
    BF16x3 collision-matrix kernel over every grid's (cell tile, node) pairs.
    Each grid's distribution and time after a few steps, eager and replayed
    from the graph, equal gd_step on its own context bit for bit."""
    torch = cuda
    from gpu_determ_gb300 import inputs
    specs = [(8, 200, 11), (12, 300, 12), (16, 130, 13)]
    groups = []
    for n, cells, seed in specs:
        spec = gdlib.GridSpec(n, R=4.8)
        ctx = gdlib.Context(spec)
        ctx.set_gain_path(gdlib.GAIN_PAIR_TC if mode == "pair_tc" else gdlib.GAIN_CMATRIX_BF16X3)
        groups.append((ctx, inputs.shock_profile(spec.fill(), cells) if n != 12 else
                       inputs.mixtures(spec.fill(), cells, seed=seed), cells))
    f_ref, t_ref = _run_single(gdlib, torch, groups)
    for use_graph in (False, True):
        b = gdlib.Batch()
        fs, ts = [], []
        for ctx, f0, cells in groups:
            f = torch.from_numpy(f0).cuda()
            t = torch.zeros(1, dtype=torch.float32, device="cuda")
            b.add(ctx, f, cells, cells, gdlib.DT_COURANT, 0.5, time=t)
            fs.append(f)
            ts.append(t)
        b.set_mode(gdlib.BATCH_FUSED_PAIR_TC if mode == "pair_tc" else gdlib.BATCH_FUSED_CMATRIX)
        for _ in range(STEPS):
            b.step(use_graph)
        b.check()
        info = b.info()
        b.close()
        torch.cuda.synchronize()
        for a, f in zip(f_ref, fs):
            assert np.array_equal(a, f.cpu().numpy())
        assert t_ref == [float(t.item()) for t in ts]
        if use_graph:
            assert info["graph_nodes"] > 0


def test_fused_batch_rejects_other_gain_paths(gdlib, cuda):
    torch = cuda
    from gpu_determ_gb300 import inputs
    spec = gdlib.GridSpec(8, R=4.8)
    ctx = gdlib.Context(spec)
    f = torch.from_numpy(inputs.mixtures(spec.fill(), 32, seed=1)).cuda()
    b = gdlib.Batch()
    b.add(ctx, f, 32, 32, gdlib.DT_COURANT, 0.5)
    for mode in (gdlib.BATCH_FUSED_PAIR_TC, gdlib.BATCH_FUSED_CMATRIX):
        with pytest.raises(gdlib.GDError) as e:
            b.set_mode(mode)                      # the context is on the FP32 pair kernel
        assert e.value.code == 4
    b.close()


def test_fused_cmatrix_batch_needs_one_matrix_mode(gdlib, cuda):
    """One launch of the collision-matrix kernel serves one mode: groups on
    BF16x3 and on one BF16 pass cannot be fused (GD_ERR_UNSUPPORTED, before
    anything is enqueued)."""
    torch = cuda
    from gpu_determ_gb300 import inputs
    b = gdlib.Batch()
    ctxs = []
    for n, path in ((8, gdlib.GAIN_CMATRIX_BF16X3), (12, gdlib.GAIN_CMATRIX_BF16)):
        spec = gdlib.GridSpec(n, R=4.8)
        ctx = gdlib.Context(spec)
        ctx.set_gain_path(path)
        f = torch.from_numpy(inputs.mixtures(spec.fill(), 64, seed=n)).cuda()
        b.add(ctx, f, 64, 64, gdlib.DT_COURANT, 0.5)
        ctxs.append(ctx)
    with pytest.raises(gdlib.GDError) as e:
        b.set_mode(gdlib.BATCH_FUSED_CMATRIX)
    assert e.value.code == 4
    b.close()
