"""Case plug-ins (level set + initial state) on the CPU."""
import numpy as np

from ibtfo_gb300 import cases


def test_coords_match_reference_formula():
    g = cases.Grid(40, 20, 2, 0.0, 0.0, 1.0, 0.5)
    x, y = g.coords()
    dx = 1.0 / 40
    Li = -dx * 2 + 0.0 + dx / 2
    assert x[0, 0] == Li and x[0, 5] == Li + 5 * dx
    assert y[3, 0] == Li + 3 * dx  # the reference uses dx for y as well


def test_channel_geometry():
    g = cases.Grid(256, 128, 2, 0.0, 0.0, 2.0, 1.0)
    phi = cases.channel_phi(g).reshape(g.N, g.M)
    x, y = g.coords()
    # centre line is the furthest point from both walls
    assert abs(phi.max() - 0.125) < 1e-2
    inside = phi >= 0
    frac = inside[2:-2, 2:-2].mean()
    assert 0.1 < frac < 0.35


def test_sod_states():
    g = cases.Grid(40, 10, 2, 0.0, 0.0, 1.0, 0.25)
    phi, u = cases.sod_x(g)
    u = u.reshape(g.N, g.M, 4)
    assert np.all(phi == 1.0)
    assert u[5, 2, 0] == 1.0 and u[5, -3, 0] == 0.125
    assert np.isclose(u[5, 2, 3], 1.0 / 0.4) and np.isclose(u[5, -3, 3], 0.1 / 0.4)


def test_vortex_is_periodic_and_positive():
    g = cases.Grid(64, 64, 2, 0.0, 0.0, 10.0, 10.0)
    _, u = cases.isentropic_vortex(g)
    u = u.reshape(g.N, g.M, 4)
    assert u[..., 0].min() > 0.3
    _, u10 = cases.isentropic_vortex(g, t=10.0)
    assert np.allclose(u10, u.reshape(-1), atol=1e-12)
