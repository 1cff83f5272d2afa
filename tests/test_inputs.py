"""Synthetic inputs of the configs (CPU): Rankine-Hugoniot states of the Mach-3
shock, the shock profile's end states and moments, Dirichlet mixtures."""
import numpy as np
import pytest

from gpu_determ_gb300 import GridSpec, inputs


def test_rankine_hugoniot_mach3():
    s = inputs.rankine_hugoniot(3.0, 5.0 / 3.0)
    assert s["density_ratio"] == pytest.approx(3.0)
    assert s["temperature_ratio"] == pytest.approx(11.0 / 3.0)
    # upstream speed = 3 sound speeds, sqrt(gamma T / 2) in the exp(-c^2/T) convention
    assert s["lab_u1"] == pytest.approx(3.0 * np.sqrt(5.0 / 6.0))
    # the three conservation laws across the shock (per unit mass, T = 2 kT/m):
    # n u, n u^2 + n T/2, u (u^2/2 + 5 T/4)
    n1, u1, T1 = s["n1"], s["lab_u1"], s["T1"]
    n2, u2, T2 = s["n2"], s["lab_u2"], s["T2"]
    assert n1 * u1 == pytest.approx(n2 * u2)
    assert n1 * u1 * u1 + n1 * T1 / 2 == pytest.approx(n2 * u2 * u2 + n2 * T2 / 2)
    assert u1 * u1 / 2 + 5 * T1 / 4 == pytest.approx(u2 * u2 / 2 + 5 * T2 / 4)
    # frame moving with the mean of the two speeds
    assert s["u1"] == pytest.approx(-s["u2"])


def test_shock_profile_end_states():
    spec = GridSpec(16, R=16.5)
    g = spec.fill()
    f = inputs.shock_profile(g, 64, half_width=8.0, thickness=0.5)
    xu, xv, xw = inputs.node_velocities(g)
    d3v = float(g["steps"][3])
    n = f.sum(axis=0) * d3v
    ux = (f * xu[:, None]).sum(axis=0) * d3v / n
    s = inputs.rankine_hugoniot()
    assert n[0] == pytest.approx(s["n1"], rel=2e-3)
    assert n[-1] == pytest.approx(s["n2"], rel=2e-3)
    assert ux[0] == pytest.approx(s["u1"], abs=5e-3)
    # the hot downstream Maxwellian (T = 11/3) loses ~0.6 % of its bulk speed to
    # the tails the [-5, 5]^3 box cuts off
    assert ux[-1] == pytest.approx(s["u2"], abs=1e-2)
    # density rises monotonically through the shock (flat to float32 precision at the ends)
    assert np.all(np.diff(n) > -1e-5) and n[33] > n[31]


def test_dirichlet_mixtures():
    spec = GridSpec(20, R=4.8)
    g = spec.fill()
    f = inputs.dirichlet_mixtures(g, 200, seed=3)
    assert f.shape == (spec.count(), 200) and f.dtype == np.float32
    n = f.sum(axis=0) * float(g["steps"][3])
    # unit total density, minus the tails cut by the sphere
    assert np.all(n <= 1.0 + 1e-3) and np.median(n) > 0.97
    w, u, T = inputs.dirichlet_mixture_params(200, seed=3)
    assert np.allclose(w.sum(axis=1), 1.0)
    assert T.min() >= 0.5 and T.max() <= 2.0
    # seeded: the same seed gives the same cells
    assert np.array_equal(f, inputs.dirichlet_mixtures(g, 200, seed=3))


def test_cavity_field():
    vel, T = inputs.cavity_field_params(4096, amp=0.8, T_amp=0.3, seed=2)
    speed = np.sqrt((vel ** 2).sum(axis=1))
    assert speed.max() == pytest.approx(0.8) and np.all(vel[:, 2] == 0.0)
    assert T.min() >= 0.7 - 1e-12 and T.max() <= 1.3 + 1e-12
    assert T.max() == pytest.approx(1.3) or T.min() == pytest.approx(0.7)
    # divergence free: finite-difference divergence on the 64 x 64 cell grid is
    # small next to the velocity gradients
    m = 64
    u = vel[:, 0].reshape(m, m)          # [row j (y)][col i (x)]
    v = vel[:, 1].reshape(m, m)
    h = 1.0 / m
    div = (u[1:-1, 2:] - u[1:-1, :-2]) / (2 * h) + (v[2:, 1:-1] - v[:-2, 1:-1]) / (2 * h)
    grad = np.abs((u[1:-1, 2:] - u[1:-1, :-2]) / (2 * h)).max()
    assert np.abs(div).max() < 2e-2 * grad
    # no flow through the walls: u ~ 0 at x = 0, 1 and v ~ 0 at y = 0, 1 (cell centres h/2 in)
    assert np.abs(u[:, 0]).max() < 0.1 and np.abs(v[0, :]).max() < 0.1
    # seeded
    v2, T2 = inputs.cavity_field_params(4096, seed=2)
    assert np.array_equal(vel, v2) and np.array_equal(T, T2)


def test_cavity_field_moments():
    spec = GridSpec(20, R=4.8)
    g = spec.fill()
    f = inputs.cavity_field(g, 64, seed=1)
    vel, T = inputs.cavity_field_params(64, seed=1)
    xu, xv, xw = inputs.node_velocities(g)
    d3v = float(g["steps"][3])
    n = f.sum(axis=0) * d3v
    assert np.allclose(n, 1.0, rtol=2e-3)
    assert np.allclose((f * xu[:, None]).sum(axis=0) * d3v / n, vel[:, 0], atol=2e-3)
    assert np.allclose((f * xv[:, None]).sum(axis=0) * d3v / n, vel[:, 1], atol=2e-3)
