"""What the trained surrogate gains over the method without it (12^3, R = 4.8).

The plain method (BF16x3 collision matrices + FP64 projection) labels seeded
mixtures of 1-4 Maxwellians; surrogate.fit trains the network and its error
estimator on the GPU with the library's own kernels and calibrates the
fallback margin.  On held-out cells:

- training lowers the batch-relative loss, and the trained network's error is
  a small fraction of the untrained network's;
- without the network every cell needs a plain gain evaluation; with it, the
  tolerance decides the split: at 1e-3 every cell still takes the plain
  method (the result is the plain result), at loose tolerances part of the
  cells are served by the network and that fraction of plain evaluations is
  saved;
- the calibrated estimate holds: the cells the network serves stay within the
  tolerance (up to the calibration quantile);
- every projected Q conserves mass, momentum and energy, whichever path made
  its gain."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOLS = (1e-3, 0.1, 0.3, 1.0, 3.0, 10.0)


@pytest.fixture(scope="module")
def trained(gdlib, cuda):
    from gpu_determ_gb300 import surrogate as S
    spec = gdlib.GridSpec(12, R=4.8)
    ctx = gdlib.Context(spec)
    ctx.set_gain_path(gdlib.GAIN_CMATRIX_BF16X3)
    grid = spec.fill()
    model = S.fit(ctx, grid, pairs=16384, steps=1500, batch=512, est_pairs=4096, est_steps=800,
                  calib_pairs=2048, max_cells=2048, seed=0)
    test = S.generate(ctx, grid, 2048, seed=4321)
    evals = {t: S.evaluate(model, test, t, 2048) for t in TOLS}
    # the same architecture, untrained (its seeded initial weights)
    raw = gdlib.Mlp(ctx.n_pnt, ctx.n_pnt, batch_cap=2048,
                    flags=gdlib.MLP_SCALE_INPUT | gdlib.MLP_SCALE_OUTPUT | gdlib.MLP_LOSS_BATCH, seed=0)
    raw.set_io_scale(model.report["in_gain"], model.report["out_gain"])
    untrained = S.Model(ctx, raw, None, gdlib.Surrogate(ctx, raw, None, 2048))
    raw_err = S.cell_errors(untrained, test, float("inf"), 2048)["err"]
    print("surrogate training at 12^3:", {k: model.report[k] for k in ("loss_first", "loss_last", "margin_log10")},
          "untrained median", float(np.median(raw_err)))
    for t in TOLS:
        print({k: evals[t][k] for k in ("tol", "fallback_fraction", "batch_rel_l2", "cell_rel_l2_median",
                                          "cells_above_tol", "surrogate_only_median", "conservation_max")})
    return model, evals, raw_err


def test_training_reduces_the_error(trained):
    model, evals, raw_err = trained
    rep = model.report
    # loss_first is logged after the first 200 steps, the untrained network
    # is compared below
    assert rep["loss_last"] < 0.6 * rep["loss_first"], rep
    trained_median = evals[TOLS[0]]["surrogate_only_median"]
    assert trained_median < 0.6, trained_median
    assert trained_median < 0.5 * float(np.median(raw_err)), (trained_median, float(np.median(raw_err)))


def test_tight_tolerance_is_the_plain_method(trained):
    _, evals, _ = trained
    e = evals[1e-3]
    assert e["fallback_fraction"] == 1.0
    # the fallback gain is the plain gain; only the FP32 rounding of the
    # stored labels remains
    assert e["cell_rel_l2_max"] < 1e-6, e
    assert e["cells_above_tol"] == 0


def test_loose_tolerances_spare_plain_evaluations(trained):
    _, evals, _ = trained
    fb = [evals[t]["fallback_fraction"] for t in TOLS]
    assert all(b <= a for a, b in zip(fb, fb[1:])), fb          # monotone in the tolerance
    assert fb[-1] < 0.5, fb                                      # the network serves most cells
    for t in TOLS:
        e = evals[t]
        served = (1.0 - e["fallback_fraction"]) * e["cells"]
        # cells served by the network that miss the tolerance: within the
        # calibration quantile (1 %) plus sampling slack
        if served > 0:
            assert e["cells_above_tol"] <= 0.05 * served + 2, (t, e)
        assert e["conservation_max"] < 1e-11, (t, e)
