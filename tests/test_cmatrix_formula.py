"""The collision-matrix form of the gain, checked on the CPU against the
oracle: with s = a + b, d = a - b,
    G_i[a][b] = m(d) w(|2i - s|, |d|) [s - i in the box],
    m(d) = (d_x == 0 ? 1 : 1/2) (d_y == 0 ? 2 : 1) (d_z == 0 ? 2 : 1),
f^T G_i f equals the reference-order gain sum (collision_integral.cu:75-188)."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle, maxwellian


def assemble(o, k):
    N, h = o.nx, o.nx // 2
    a_tab = o.table_a().reshape(h, N, h, h, N, N)
    P = np.stack([o.ui, o.vi, o.wi], 1)
    s = P[:, None, :] + P[None, :, :]
    d = P[:, None, :] - P[None, :, :]
    ad = np.abs(d)
    i = P[k]
    i1 = s - i
    inbox = np.all((i1 >= 0) & (i1 < N), axis=-1)
    g = np.minimum(np.abs(2 * i - s), N - 1)
    W = a_tab[ad[..., 0] >> 1, g[..., 0], ad[..., 1] >> 1, ad[..., 2] >> 1, g[..., 1], g[..., 2]].astype(np.float64)
    m = np.where(d[..., 0] == 0, 1.0, 0.5) * np.where(d[..., 1] == 0, 2.0, 1.0) * np.where(d[..., 2] == 0, 2.0, 1.0)
    return m * W * inbox


@pytest.mark.parametrize("N,R", [(8, 16.5), (10, 3.9)])
def test_bilinear_form_equals_gain(N, R):
    o = Oracle(N, R=R)
    rng = np.random.default_rng(N)
    f = np.stack([maxwellian(o, 1.0, rng.normal(0, .5, 3), 0.9) + 0.3 * maxwellian(o, 1.0, rng.normal(0, .7, 3), 1.3)
                  for _ in range(3)], 1).astype(np.float32)
    ref = o.gain_f64(o.to_box(f))
    f64 = f.astype(np.float64)
    for k in range(0, o.n_pnt, max(1, o.n_pnt // 40)):
        G = assemble(o, k)
        assert np.array_equal(G, G.T)
        val = np.einsum("ac,ab,bc->c", f64, G, f64)
        assert np.all(np.abs(val - ref[k]) <= 1e-12 * np.abs(ref).max(axis=0))
