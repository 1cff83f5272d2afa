"""The homogeneous relaxation of the two-beam start (the time integrator of
collision_integral.cu:835-880 with the Courant step of :776-807) on the GPU's
FP32 pair-product path, against the same integrator with every collision
integral, projection and step evaluated in FP64 by the oracle (f stored in
FP32 between steps on both sides, as the reference stores it).  The two
trajectories agree to ~1e-6 over 20 steps: the FP32 arithmetic of the
plain method does not drift from its FP64 counterpart."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def _fp64_step(o, phi, f, courant):
    """One projected Courant step with FP64 loss, gain, projection and
    relaxation; returns the new FP32 f and the FP32 dt."""
    fb = o.to_box(f)
    nu = o.loss_f64(fb)
    gain = o.gain_f64(fb)
    f64 = f.astype(np.float64)
    fnu = f64 * nu
    A = np.einsum("ic,ik,il->ckl", fnu, phi, phi)
    B = np.einsum("ic,ik->ck", gain - fnu, phi)
    X = np.linalg.solve(A, B[..., None])[..., 0]
    nu_c = nu * (1.0 + phi @ X.T)
    q = gain - f64 * nu_c
    dt = np.float32(courant) / np.float32(nu_c.astype(np.float32).max())
    return (f64 + float(dt) * q).astype(np.float32), float(dt)


def test_two_beam_trajectory_matches_fp64_integrator(cuda, gdlib):
    from gpu_determ_gb300 import relaxation

    steps, courant = 20, 0.5
    gpu_f = []
    _, recs = relaxation.run(grid=12, radius=4.8, steps=steps, courant=courant, cells=1, init="two_beam",
                             callback=lambda rec, f: gpu_f.append(f.cpu().numpy().copy()))
    o = Oracle(12, R=4.8)
    phi = o.phi()
    from gpu_determ_gb300 import inputs
    f = inputs.two_beam(gdlib.GridSpec(12, R=4.8).fill(), 1)
    t = 0.0
    worst = 0.0
    for k in range(steps):
        f, dt = _fp64_step(o, phi, f, courant)
        t += dt
        g = gpu_f[k]
        rel = float(np.linalg.norm(g.astype(np.float64) - f) / np.linalg.norm(f))
        worst = max(worst, rel)
        assert rel <= 1e-5, (k, rel)
        assert abs(recs[k + 1]["time"] - t) <= 1e-5 * t, (k, recs[k + 1]["time"], t)
    print("two-beam relaxation, 12^3, %d Courant steps: max rel-L2 of f (GPU FP32 path vs FP64 integrator) %.2e"
          % (steps, worst))
