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
