"""Tensor-core collision-matrix gain (tcgen05, BF16 operands, FP32 accumulation)
against the FP64 oracle on the same seeded inputs.  Tolerances (relative L2 of
I over all nodes and cells): BF16 <= 5e-3, BF16 x3 (hi/lo split) <= 2e-5.
Results are bitwise reproducible."""
import numpy as np
import pytest

from gpu_determ_gb300 import inputs
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,R,ncells,ld", [(8, 16.5, 40, 40), (12, 4.8, 200, 203)])
def test_cmatrix_gain_matches_oracle(cuda, gdlib, n, R, ncells, ld):
    torch = cuda
    spec = gdlib.GridSpec(n, R=R)
    ctx = gdlib.Context(spec)
    f = inputs.mixtures(spec.fill(), ncells, seed=n + 7)
    ft = torch.zeros((ctx.n_pnt, ld), dtype=torch.float32, device="cuda")
    ft[:, :ncells] = torch.from_numpy(f).cuda()
    o = Oracle(n, R=R)
    ref = o.gain_f64(o.to_box(f))
    for mode, tol in ((gdlib.CMATRIX_BF16X3, 2e-5), (gdlib.CMATRIX_BF16, 5e-3)):
        cm = gdlib.CollisionMatrix(ctx, mode)
        out = torch.full_like(ft, -1.0)
        cm.gain(ft, ncells, ld, out)
        out2 = torch.full_like(ft, -1.0)
        cm.gain(ft, ncells, ld, out2)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.array_equal(got, out2.cpu().numpy())
        assert np.all(got[:, ncells:] == -1.0)
        rel = np.linalg.norm(got[:, :ncells] - ref) / np.linalg.norm(ref)
        assert rel <= tol, (mode, rel)
        cm.close()


@pytest.mark.parametrize("dims,R", [((12, 10, 8), 4.2), ((8, 12, 10), 16.5)])
def test_cmatrix_orbits_on_non_cubic_lattices(cuda, gdlib, dims, R):
    """Matrices are stored for one node per orbit of the lattice's three
    reflections, and node R(i) contracts the matrices of i with f reflected by
    R; on lattices with different extents per axis (the sphere cutting some
    of them) the result still matches the FP64 oracle."""
    torch = cuda
    nx, ny, nz = dims
    spec = gdlib.GridSpec(nx, ny, nz, R=R)
    ctx = gdlib.Context(spec)
    nc = 96
    f = inputs.mixtures(spec.fill(), nc, seed=31)
    ft = torch.from_numpy(f).cuda()
    o = Oracle(nx, ny, nz, R=R)
    ref = o.gain_f64(o.to_box(f))
    cm = gdlib.CollisionMatrix(ctx, gdlib.CMATRIX_BF16X3)
    out = torch.empty_like(ft)
    cm.gain(ft, nc, nc, out)
    torch.cuda.synchronize()
    rel = np.linalg.norm(out.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert rel <= 2e-5, rel
    cm.close()


@pytest.mark.parametrize("path,tol", [(2, 1e-4), (1, 2e-2)])
def test_step_with_cmatrix_gain_path(cuda, gdlib, path, tol):
    """gd_step with the tensor-core gain: the FP64 projection still conserves
    mass, momentum and energy to 1e-12, and Q stays within tol (relative L2)
    of the FP64 oracle's projected Q (BF16 x3: 1e-4, BF16: 2e-2)."""
    torch = cuda
    n, R, nc = 12, 4.8, 64
    spec = gdlib.GridSpec(n, R=R)
    ctx = gdlib.Context(spec)
    ctx.set_gain_path(path)
    f = inputs.mixtures(spec.fill(), nc, seed=31)
    ft = torch.from_numpy(f).cuda()
    q = torch.zeros(ft.shape, dtype=torch.float64, device="cuda")
    gain = torch.zeros_like(ft)
    ctx.step(ft, nc, nc, gdlib.DT_COURANT, 0.5, gain=gain, q=q)
    torch.cuda.synchronize()
    o = Oracle(n, R=R)
    qh = q.cpu().numpy()
    mom = o.phi().T @ qh
    scale = np.abs(o.phi()).T @ np.abs(gain.cpu().numpy().astype(np.float64))
    assert np.all(np.abs(mom) <= 1e-12 * scale)
    fb = o.to_box(f)
    _, q64, _, _ = o.project(f, o.loss_f64(fb).astype(np.float32), o.gain_f64(fb).astype(np.float32))
    rel = np.linalg.norm(qh - q64) / np.linalg.norm(q64)
    print(f"gain path {path}: Q relative L2 vs FP64 oracle = {rel:.3e}")
    assert rel <= tol


@pytest.mark.parametrize("n,R,ncells,ld", [(12, 4.8, 300, 300), (12, 4.8, 100, 103), (16, 4.8, 64, 64)])
def test_tensor_core_loss(cuda, gdlib, n, R, ncells, ld):
    """With collision matrices selected, nu = B f runs on the tensor cores
    (hi/lo split, B_hi f_hi + B_hi f_lo + B_lo f_hi in one launch, the K range
    in chunks of 256 added in FP32).  The tensor cores' FP32 accumulation
    leaves nu slightly low (mean relative bias ~1e-6 at 20^3), so the bound is
    4e-5 per node and cell (the FP32 kernel meets 1e-5) and 2e-5 on the
    mean; the FP64 projection restores exact conservation either way.  A
    leading dimension that is not a multiple of 4 falls back to the FP32 kernel
    (bitwise equal to the pair path's nu)."""
    torch = cuda
    spec = gdlib.GridSpec(n, R=R)
    ctx = gdlib.Context(spec)
    f = inputs.mixtures(spec.fill(), ncells, seed=n + 11)
    ft = torch.zeros((ctx.n_pnt, ld), dtype=torch.float32, device="cuda")
    ft[:, :ncells] = torch.from_numpy(f).cuda()
    o = Oracle(n, R=R)
    ref = o.loss_f64(o.to_box(f))
    nu_pair = torch.zeros_like(ft)
    ctx.collision(ft, ncells, ld, nu_pair, None)
    ctx.set_gain_path(gdlib.GAIN_CMATRIX_BF16)
    nu = torch.full_like(ft, -1.0)
    ctx.collision(ft, ncells, ld, nu, None)
    nu2 = torch.full_like(ft, -1.0)
    ctx.collision(ft, ncells, ld, nu2, None)
    torch.cuda.synchronize()
    got = nu.cpu().numpy()
    assert np.array_equal(got, nu2.cpu().numpy())
    assert np.all(got[:, ncells:] == -1.0)
    rel = (got[:, :ncells] - ref) / ref
    assert np.max(np.abs(rel)) < 4e-5
    assert abs(np.mean(rel)) < 2e-5
    if ld % 4:
        assert np.array_equal(got[:, :ncells], nu_pair.cpu().numpy()[:, :ncells])


@pytest.mark.parametrize("ncells", [129, 200, 300, 1000])
def test_cta_pair_is_bitwise_equal(cuda, gdlib, ncells):
    """CTA-pair MMAs (M = 256 cells over two CTAs, each loading half of every
    collision-matrix tile) give the same bits as one CTA per 128-cell tile
    (same operands, same MMA order, same epilogue); an odd number of cell
    tiles is padded to whole pairs."""
    torch = cuda
    spec = gdlib.GridSpec(12, R=4.8)
    ctx = gdlib.Context(spec)
    f = torch.from_numpy(inputs.mixtures(spec.fill(), ncells, seed=5)).cuda()
    for mode in (gdlib.CMATRIX_BF16, gdlib.CMATRIX_BF16X3):
        cm = gdlib.CollisionMatrix(ctx, mode)
        outs = []
        for ctas in (1, 2):
            cm.set_cluster(ctas)
            g = torch.full_like(f, -1.0)
            cm.gain(f, ncells, ncells, g)
            outs.append(g)
        torch.cuda.synchronize()
        assert torch.equal(outs[0], outs[1])
        cm.close()


def test_headline_grid_against_pair_kernel(cuda, gdlib):
    """20^3 (R = 4.8, 3648 nodes), the bench's lattice: the tensor-core gain
    against the FP32 pair-product kernel (itself within 1e-5 of the FP64
    oracle) on 300 seeded mixtures, with a leading dimension past the cells;
    CTA pairs and one CTA per MMA give the same bits."""
    torch = cuda
    spec = gdlib.GridSpec(20, R=4.8)
    ctx = gdlib.Context(spec)
    nc, ld = 300, 304
    ft = torch.zeros((ctx.n_pnt, ld), dtype=torch.float32, device="cuda")
    ft[:, :nc] = torch.from_numpy(inputs.dirichlet_mixtures(spec.fill(), nc, seed=11)).cuda()
    ref = torch.empty_like(ft)
    ctx.collision(ft, nc, ld, None, ref)
    ref = ref[:, :nc]
    for mode, tol in ((gdlib.CMATRIX_BF16X3, 2e-5), (gdlib.CMATRIX_BF16, 1e-3)):
        cm = gdlib.CollisionMatrix(ctx, mode)
        outs = []
        for ctas in (2, 1):
            cm.set_cluster(ctas)
            out = torch.full_like(ft, -1.0)
            cm.gain(ft, nc, ld, out)
            outs.append(out)
        torch.cuda.synchronize()
        assert torch.equal(outs[0], outs[1])
        assert bool((outs[0][:, nc:] == -1.0).all())
        rel = float((outs[0][:, :nc] - ref).norm() / ref.norm())
        assert rel <= tol, (mode, rel)
        cm.close()


def test_c2_batch_against_fp64_oracle(cuda, gdlib):
    """Config C2 (16^3, R = 4.8): seeded mixtures of 1-3 Maxwellians with
    n ~ lognormal(0, 0.3), u ~ N(0, 0.7^2) per axis, T ~ U[0.6, 1.8]; the gain
    and the FP64-projected Q of every gain path against the FP64 oracle, on
    the config's batch of 1024 (GD_C2_CELLS overrides it).  The paths with
    FP32-equivalent arithmetic (FP32 pair kernel, pair products on tensor
    cores, BF16x3 collision matrices with the tensor-core loss) also keep
    every cell's projected Q within the metric's relative L2 of 1e-3; one-pass
    BF16 does not (its per-cell tail is reported, not asserted)."""
    import os
    torch = cuda
    nc = int(os.environ.get("GD_C2_CELLS", "1024"))
    spec = gdlib.GridSpec(16, R=4.8)
    ctx = gdlib.Context(spec)
    f = inputs.mixtures(spec.fill(), nc, seed=2024)
    o = Oracle(16, R=4.8)
    nu_ref = o.loss_f64(o.to_box(f))
    i_ref = o.gain_f64(o.to_box(f))
    _, q_ref, _, _ = o.project(f, nu_ref, i_ref)
    ft = torch.from_numpy(f).cuda()
    tols = {gdlib.GAIN_PAIR: (1e-5, 1e-4), gdlib.GAIN_PAIR_TC: (2e-5, 2e-4),
            gdlib.GAIN_CMATRIX_BF16X3: (2e-5, 2e-4), gdlib.GAIN_CMATRIX_BF16: (5e-3, 5e-3)}
    report = {}
    for path, (tol_i, tol_q) in tols.items():
        ctx.set_gain_path(path)
        nu, gain = torch.empty_like(ft), torch.empty_like(ft)
        q = torch.zeros(ft.shape, dtype=torch.float64, device="cuda")
        ctx.collision(ft, nc, nc, nu, gain)
        ctx.project(ft, nu, gain, nc, nc, q=q)
        ctx.check()
        g = gain.cpu().numpy().astype(np.float64)
        qq = q.cpu().numpy()
        rel_i = np.linalg.norm(g - i_ref) / np.linalg.norm(i_ref)
        rel_q = np.linalg.norm(qq - q_ref) / np.linalg.norm(q_ref)
        cell_q = np.linalg.norm(qq - q_ref, axis=0) / np.linalg.norm(q_ref, axis=0)
        report[path] = (rel_i, rel_q, float(np.median(cell_q)), float(np.quantile(cell_q, 0.99)),
                        float(cell_q.max()))
        assert rel_i <= tol_i and rel_q <= tol_q, (path, report[path])
        if path != gdlib.GAIN_CMATRIX_BF16:
            assert cell_q.max() <= 1e-3, (path, report[path])
    print("C2 16^3,", nc, "cells: path -> (gain rel-L2, Q rel-L2, Q per-cell median, p99, max) vs FP64:", report)


def test_orbit_storage_reflection_identity_is_bitwise(cuda, gdlib):
    """Node R(i) contracts the matrices of its orbit's representative with f
    reflected by R, so the gain of f at R(i) and the gain of f o R at i run
    the same MMAs on the same operands: equal bit for bit, for every node and
    all eight reflections of the lattice."""
    torch = cuda
    n = 12
    spec = gdlib.GridSpec(n, R=4.8)
    g = spec.fill()
    ui, vi, wi = g["ui"], g["vi"], g["wi"]
    box = {(int(a), int(b), int(c)): m for m, (a, b, c) in enumerate(zip(ui, vi, wi))}
    ctx = gdlib.Context(spec)
    cm = gdlib.CollisionMatrix(ctx, gdlib.CMATRIX_BF16X3)
    nc = 140
    f = inputs.mixtures(g, nc, seed=77)
    base = torch.empty((len(ui), nc), dtype=torch.float32, device="cuda")
    cm.gain(torch.from_numpy(f).cuda(), nc, nc, base)
    torch.cuda.synchronize()
    base = base.cpu().numpy()
    for R in range(1, 8):
        perm = np.array([box[((n - 1 - a) if R & 1 else a, (n - 1 - b) if R & 2 else b, (n - 1 - c) if R & 4 else c)]
                         for a, b, c in zip(ui, vi, wi)])
        out = torch.empty((len(ui), nc), dtype=torch.float32, device="cuda")
        cm.gain(torch.from_numpy(np.ascontiguousarray(f[perm])).cuda(), nc, nc, out)  # (f o R)[m] = f[R m]
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), base[perm]), R
    cm.close()
