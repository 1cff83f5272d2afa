"""Bit-exact index map of the gain: the tables the GPU's pair-product kernels
read, expanded into the set of (output node i, pair sum s = i + i1,
post-collision offset n) terms, equal the reference's enumeration
(collision_integral.cu:88-94, 115-131, 154-155: for every output i and
partner i1 in the box, every offset n of the parity of i - i1 with a nonzero
weight whose post-collision pair l, l1 = (s +- n)/2 stays in the box).

Both sides reduce the term set to an order-independent digest (count, a
wrapping sum and an xor of two 64-bit mixes of each key) and the FP64 sum of
the weights; the oracle's digest comes from its own enumeration in the
reference's loop order (or_index_map_digest).  On the GPU side every
member's weight row is also checked, bitwise, against the GPU's own dense
table a in the reference layout (compute_matrix.cu:556-557), and the weight
table of the pair path on tensor cores against the BF16 hi/lo split of those
rows.  Grids 8^3, 12^3 and 16^3 on [-5,5]^3 cut to R = 4.8."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu

U64 = np.uint64


def _mix_a(z):
    z = z + U64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> U64(30))) * U64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> U64(27))) * U64(0x94D049BB133111EB)
    return z ^ (z >> U64(31))


def _mix_b(z):
    z = z ^ U64(0x5851F42D4C957F2D)
    z = (z ^ (z >> U64(33))) * U64(0xFF51AFD7ED558CCD)
    z = (z ^ (z >> U64(33))) * U64(0xC4CEB9FE1A85EC53)
    return z ^ (z >> U64(33))


class _Digest:
    def __init__(self):
        self.count, self.sa, self.xb, self.wsum = 0, U64(0), U64(0), 0.0
        self.keys, self.weights, self.pending = [], [], 0

    def add(self, keys, w):
        self.keys.append(keys)
        self.weights.append(w)
        self.pending += keys.size
        if self.pending > 1 << 24:
            self.flush()

    def flush(self):
        if not self.keys:
            return
        k = np.concatenate(self.keys)
        with np.errstate(over="ignore"):
            self.sa = U64((int(self.sa) + int(_mix_a(k).sum(dtype=U64))) & ((1 << 64) - 1))
            self.xb = U64(int(self.xb) ^ int(np.bitwise_xor.reduce(_mix_b(k))))
        self.count += k.size
        self.wsum += float(np.concatenate(self.weights).astype(np.float64).sum())
        self.keys, self.weights, self.pending = [], [], 0


def _bf16_bits(x):
    """Round float32 to BF16 (nearest even), as raw bits."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + U64(0x7FFF) + ((u >> U64(16)) & U64(1))) >> U64(16)).astype(np.uint16)


def _bf16_value(bits):
    return (bits.astype(np.uint32) << np.uint32(16)).view(np.float32)


def _expand(gd, ctx, spec, check_pair_tc):
    """Digest of the GPU tables' term set; checks each weight against the
    GPU's dense table, and the tensor-core pair table when asked."""
    nx, ny, nz = spec.nx, spec.ny, spec.nz
    hx, hy, hz = nx // 2, ny // 2, nz // 2
    nyz, nxyz = ny * nz, nx * ny * nz
    sy, sz = 2 * ny - 1, 2 * nz - 1
    t = ctx.pair_tables()
    assert t["nclass"] == hx * hy * hz
    grid = spec.fill()
    cmap = np.full(nxyz, -1, np.int64)
    cmap[(grid["ui"] * ny + grid["vi"]) * nz + grid["wi"]] = np.arange(len(grid["ui"]))
    import torch
    a_dev = torch.zeros(ctx.info["table_a_elems"], dtype=torch.float32, device="cuda")
    ctx.export_tables(None, a_dev)
    torch.cuda.synchronize()
    a_gpu = a_dev.cpu().numpy()
    pt = ctx.pair_tc_table() if check_pair_tc else None
    roff, ecls, ew = t["grp_row_off"], t["entry_class"], t["entry_w"]
    ioff, items, mem = t["item_off"], t["items"], t["members"]
    dig = _Digest()
    signs = np.array([[(q >> b) & 1 for b in range(3)] for q in range(8)], np.int64)  # 1 = the + target
    for Dx in range(nx):
        for Dy in range(ny):
            for Dz in range(nz):
                D = (Dx * ny + Dy) * nz + Dz
                it = items[ioff[D]:ioff[D + 1]]
                if len(it) == 0:
                    continue
                par = np.array([Dx & 1, Dy & 1, Dz & 1])
                half = np.array([Dx >> 1, Dy >> 1, Dz >> 1])
                ext = half + 1  # class box B(D) extents ex, ey, ez
                # the pair sums s with D(s) = D: s_a in {D_a, 2 n_a - 2 - D_a}
                s_axes = [sorted({Dx, 2 * nx - 2 - Dx}), sorted({Dy, 2 * ny - 2 - Dy}), sorted({Dz, 2 * nz - 2 - Dz})]
                S = np.array([(a, b, c) for a in s_axes[0] for b in s_axes[1] for c in s_axes[2]], np.int64)
                s_lin = (S[:, 0] * sy + S[:, 1]) * sz + S[:, 2]
                if pt is not None:
                    mpad = (len(it) + 15) & ~15
                    K = int(np.prod(ext))
                    nch = (K + 63) // 64
                    rows = pt["wrow"][D] + np.arange(nch)[:, None] * mpad + np.arange(mpad)[None, :]
                    got_h, got_l = pt["wh"][rows].reshape(nch, mpad, 64), pt["wl"][rows].reshape(nch, mpad, 64)
                    want_h = np.zeros_like(got_h)
                    want_l = np.zeros_like(got_l)
                for m, (grp, mb, me) in enumerate(it):
                    e = np.arange(roff[grp], roff[grp + 1])
                    e = e[ew[e] != 0.0]  # row padding
                    c = ecls[e].astype(np.int64)
                    c2 = np.stack([c // (hy * hz), (c // hz) % hy, c % hz], 1)
                    keep = np.all(c2 <= half, axis=1)  # P_s is zero outside B(D)
                    c2, w = c2[keep], ew[e][keep]
                    n = 2 * c2 + par
                    n_box = (n[:, 0] * ny + n[:, 1]) * nz + n[:, 2]
                    g2 = mem[mb:me].astype(np.int64)
                    g = 2 * np.stack([g2 & 31, (g2 >> 6) & 31, (g2 >> 12) & 31], 1) + par
                    # every member's row, entry by entry, is the dense table's row of |g|
                    a_idx = (((n[None, :, 0] >> 1) * nx + g[:, None, 0]) * (hy * hz) + (n[None, :, 1] >> 1) * hz
                             + (n[None, :, 2] >> 1)) * nyz + g[:, None, 1] * nz + g[:, None, 2]
                    assert np.array_equal(a_gpu[a_idx].view(np.uint32),
                                          np.broadcast_to(w, a_idx.shape).view(np.uint32)), (D, grp)
                    if pt is not None:
                        k = (c2[:, 0] * ext[1] + c2[:, 1]) * ext[2] + c2[:, 2]
                        hb = _bf16_bits(w)
                        want_h[k // 64, m, k % 64] = hb
                        want_l[k // 64, m, k % 64] = _bf16_bits(w - _bf16_value(hb))
                    # targets (s +- g)/2 per axis; a zero component has one target
                    tgt = (S[:, None, None, :] + (2 * signs[None, None, :, :] - 1) * g[None, :, None, :]) // 2
                    dup = np.any((signs[None, :, :] == 0) & (g[:, None, :] == 0), axis=2)  # (members, 8)
                    tb = (tgt[..., 0] * ny + tgt[..., 1]) * nz + tgt[..., 2]
                    ti = cmap[tb]
                    live = (ti >= 0) & ~dup[None, :, :]
                    s_of = np.broadcast_to(s_lin[:, None, None], ti.shape)
                    ti, s_of = ti[live], s_of[live]
                    keys = ((ti.astype(U64)[:, None] << U64(32)) | (s_of.astype(U64)[:, None] << U64(15))
                            | n_box.astype(U64)[None, :])
                    dig.add(keys.ravel(), np.broadcast_to(w[None, :], keys.shape).ravel())
                if pt is not None:
                    assert np.array_equal(got_h, want_h) and np.array_equal(got_l, want_l), D
    dig.flush()
    return dig


@pytest.mark.parametrize("n", [8, 12, 16])
def test_pair_tables_index_map_matches_reference_enumeration(gdlib, cuda, n):
    spec = gdlib.GridSpec(n, R=4.8)
    ctx = gdlib.Context(spec)
    check_pt = n <= 12
    if check_pt:
        ctx.set_gain_path(gdlib.GAIN_PAIR_TC)
    dig = _expand(gdlib, ctx, spec, check_pt)
    o = Oracle(n, R=4.8)
    count, sa, xb, wsum = o.index_map_digest()
    assert dig.count == count == o.count_work()["terms"]
    assert int(dig.sa) == sa and int(dig.xb) == xb
    # the GPU's weights are FP64-built like the oracle's and agree to a few ulp
    assert abs(dig.wsum - wsum) <= 1e-6 * abs(wsum)
    ctx.close()
