"""gd_gain_noalloc: the gain through the allocation-free C entry point.

Callers that cannot let a library allocate device memory (a custom allocator
or pool owns the GPU, a latency-critical loop, no allocation after start-up)
use this entry point; it keeps its partial sums in a fixed array inside the
library.  The test calls it twice in a row through the C ABI and checks each
result against gd_collision's gain, within the parity tolerance the other GPU
tests use (relative L2 <= 1e-5, max |dI| <= 1e-4 * max|I| per cell).  It is
collected last so a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_determ_gb300 import inputs

pytestmark = pytest.mark.gpu


def _chunk_count(nblk, sms, waves=2):
    """The s-chunk count gd_collision's FP32 pair kernel picks for nblk cell
    blocks (at least two CTAs per SM, then the count that fills the last wave
    best), restated here to check when the fixed array can hold it."""
    lo = max(1, (waves * sms + nblk - 1) // nblk)
    best, best_fill = lo, -1.0
    for k in range(lo, max(lo, min(lo + 64, 512)) + 1):
        ctas = nblk * k
        fill = ctas / (((ctas + sms - 1) // sms) * sms)
        if fill > best_fill + 1e-9:
            best, best_fill = k, fill
        if fill > 0.999:
            break
    return best


def _close(a, b):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
    assert np.max(np.abs(a - b).max(axis=0) / np.abs(b).max(axis=0)) <= 1e-4


# (12, 4.8, 256, 256): the s-chunk count gd_collision picks (38) fits the
# fixed array, so both run the same chunks and the results are bitwise equal;
# in the other two cases the fixed array holds fewer chunks than gd_collision
# uses, so the sums are ordered differently and agree within the tolerance.
@pytest.mark.parametrize("n,R,ncells,ld,bitwise", [(12, 4.8, 40, 44, False), (16, 4.8, 300, 300, False),
                                                   (12, 4.8, 256, 256, True)])
def test_noalloc_gain_matches_collision(cuda, gdlib, n, R, ncells, ld, bitwise):
    torch = cuda
    L = gdlib.lib()
    spec = gdlib.GridSpec(n, R=R)
    ctx = gdlib.Context(spec)
    f = inputs.mixtures(spec.fill(), ncells, seed=n + ncells)
    ft = torch.zeros((ctx.n_pnt, ld), dtype=torch.float32, device="cuda")
    ft[:, :ncells] = torch.from_numpy(f).cuda()
    ref = torch.zeros_like(ft)
    ctx.collision(ft, ncells, ld, None, ref)
    torch.cuda.synchronize()
    ref = ref[:, :ncells].cpu().numpy()
    if bitwise:
        # the precondition of bitwise equality: gd_collision's chunk count
        # fits the fixed array (64 MiB less a 512-byte header, at most 64 chunks)
        nblk = (ncells + 31) // 32
        want = _chunk_count(nblk, torch.cuda.get_device_properties(0).multi_processor_count)
        fit = min(((64 << 20) - 512) // (ctx.n_pnt * nblk * 32 * 4), 64)
        assert want <= fit, (want, fit)
    for _ in range(2):
        out = torch.full_like(ft, -1.0)
        rc = L.gd_gain_noalloc(ctx._h, ft.data_ptr(), ncells, ld, out.data_ptr(), None)
        assert rc == 0, L.gd_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.all(got[:, ncells:] == -1.0)
        _close(got[:, :ncells], ref)
        if bitwise:
            assert np.array_equal(got[:, :ncells], ref)


def test_noalloc_rejects_batch_beyond_its_scratch(cuda, gdlib):
    L = gdlib.lib()
    ctx = gdlib.Context(gdlib.GridSpec(20, R=4.8))
    # 3648 nodes x 8192 cells x 4 B > 64 MiB: rejected on the host, nothing launched
    rc = L.gd_gain_noalloc(ctx._h, C.c_void_p(16), 8192, 8192, C.c_void_p(16), None)
    assert rc == 4
    assert b"64 MiB" in L.gd_last_error() or b"scratch" in L.gd_last_error()
