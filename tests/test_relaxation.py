"""Space-homogeneous relaxation (the time integrator with per-step moments):
mass, momentum and energy are conserved step after step up to the FP32 storage
of f, and the two-beam anisotropy relaxes monotonically toward isotropy.
Courant step dt = 0.5 / max nu, as the reference's relax_f."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_two_beam_relaxation_conserves_and_isotropises(cuda, gdlib):
    from gpu_determ_gb300 import relaxation

    spec = gdlib.GridSpec(12, R=4.8)
    g = spec.fill()
    xu = g["u"][g["ui"]].astype(np.float64)
    xv = g["v"][g["vi"]].astype(np.float64)
    d3v = float(g["steps"][3])
    gaps = []

    def axis_temperatures(rec, f):
        fh = f.cpu().numpy().astype(np.float64)[:, 0]
        n = fh.sum() * d3v
        ux = (fh * xu).sum() * d3v / n
        uy = (fh * xv).sum() * d3v / n
        tx = 2.0 * (fh * (xu - ux) ** 2).sum() * d3v / n
        ty = 2.0 * (fh * (xv - uy) ** 2).sum() * d3v / n
        gaps.append(tx - ty)

    _, recs = relaxation.run(grid=12, radius=4.8, steps=40, courant=0.5, cells=2, init="two_beam",
                             callback=axis_temperatures)
    n0, E0 = recs[0]["n"][0], recs[0]["E"][0]
    for r in recs:
        assert abs(r["n"][0] - n0) <= 2e-5 * n0
        assert abs(r["E"][0] - E0) <= 2e-5 * E0
        assert np.all(np.abs(np.array(r["u"][0])) <= 2e-5 * np.sqrt(E0 / n0))
        assert r["n"][0] == r["n"][1]  # identical cells stay identical
    assert gaps[0] > 3.0  # T_x - T_y of the two beams (5.5 - 1 on the continuum)
    assert all(b <= a + 1e-9 for a, b in zip(gaps, gaps[1:]))
    assert gaps[-1] < 0.5 * gaps[0]
    # the overall temperature is fixed by the conserved energy
    assert abs(recs[-1]["T"][0] - recs[0]["T"][0]) <= 1e-4 * recs[0]["T"][0]
