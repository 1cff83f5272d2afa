"""The config runners end to end at small sizes: the uneven-grid batch
(batched.py) and the large surrogate+fallback runner (large.py), each on a
few hundred cells so they finish in seconds."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batched_runner_small(cuda, gdlib):
    from gpu_determ_gb300 import batched
    state = batched.build(cells=192, grids=(8, 12), autotune=True, mem_budget=8e9)
    res = batched.run(state, steps=3, use_graph=True, warmup=2)
    assert res["cells"] == 192 and res["steps"] == 3 and res["batch"]["graph_nodes"] > 0
    assert res["cell_steps_per_s"] > 0
    for g in res["grids"]:
        assert g["time"] > 0
        # FP32 f, FP64 Q: moments change only at the FP32 rounding of f
        assert max(g["moment_drift"].values()) < 1e-5, g


def test_large_runner_small(cuda, gdlib):
    """The 32^3 runner's code path on a 12^3 lattice: surrogate trained on a
    few thousand pairs, cavity-field cells, the tensor-core pair path as the
    plain method and fallback, per-step checks against the FP32 pair kernel."""
    from gpu_determ_gb300 import large
    res = large.run(grid=12, radius=4.8, cells=256, steps=3, pairs=2048, train_steps=300, tol=1e-3,
                    est_pairs=1024, est_steps=200, calib_pairs=1024, plain_steps=1)
    assert res["n_pnt"] == 840 and len(res["checked_steps"]) == 3
    for rec in res["checked_steps"]:
        # cells above the tolerance took the plain gain; the rest are the
        # network's, so the step's error stays within what the served cells allow
        assert 0.0 <= rec["fallback_fraction"] <= 1.0
        assert rec["conservation_max"] < 1e-11
        if rec["fallback_fraction"] == 1.0:
            # the fallback is the tensor-core pair path: its gain is ~1e-6 from the
            # FP32 kernel's, and Q = I - nu f of these near-Maxwellian cells is
            # small next to I, which magnifies that difference ~30-fold
            assert rec["batch_rel_l2"] < 1e-4
    assert res["surrogate_step"]["cell_steps_per_s"] > 0 and res["plain_step"]["cell_steps_per_s"] > 0
    assert max(res["moment_drift"].values()) < 1e-5
    assert np.isfinite(res["time"]) and res["time"] > 0
