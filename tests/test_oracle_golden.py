"""The CPU oracle reproduces the reference's own solver bit for bit.

Every fixture in tests/golden/ was produced by the reference sources compiled
unmodified (oracle/build_ref.py + tests/golden/gen_golden.py).  The oracle gets
the same level set and initial state and must return identical bytes for the
state arrays, the geometry, the dt sequence and the mass sequence (NaN where
the reference produced NaN, at the same places).
"""
import numpy as np
import pytest

import oracle
from golden_util import load, names


def same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


@pytest.fixture(scope="module", autouse=True)
def _one_thread():
    oracle.set_threads(1)  # the mass sum is order-sensitive; the reference loop is serial
    yield


@pytest.mark.parametrize("name", names())
def test_oracle_matches_reference(name):
    fx = load(name)
    cfg = fx["config"]
    c = oracle.OracleCase(cfg["N_x"], cfg["N_y"], cfg["num_ghost_cell"], (cfg["lo_x"], cfg["lo_y"]),
                          (cfg["hi_x"], cfg["hi_y"]), cfg["gamma"], cfg["CFL_number"], cfg["scheme"],
                          cfg["riemann"], cfg["limiter"], cfg["boundary"], cfg["gbc"])
    c.setup_geometry(fx["phi"])
    if "xycoord" in fx:
        assert same(c.get("XYCOORD"), fx["xycoord"]), "geometry differs"
        assert same(c.get("SCHEME_IDX"), fx["scheme_idx"]), "ghost-fluid data differs"
    c.set_initial_state(fx["u_init"])
    s0 = c.scalars()
    assert same(s0["dt"], fx["dts"][0]) and same(s0["mass_now"], fx["masses"][0])
    dts, ms = c.run(fx["iters"], cfg["Psy_time"], cfg["max_iter"])
    assert len(dts) == fx["iters"]
    assert same(dts, fx["dts"][1:]), "dt sequence differs"
    assert same(ms, fx["masses"][1:]), "mass sequence differs"
    assert same(c.scalars()["now_t"], fx["now_t"])
    assert same(c.get("U_OLD"), fx["u_old"]), "U_OLD differs"
    assert same(c.get("U_NEW"), fx["u_new"]), "U_NEW differs"


def test_fixture_set_covers_every_variant():
    cfgs = [load(n)["config"] for n in names()]
    seen = {(c["scheme"], c["riemann"], c["limiter"], c["boundary"], c["gbc"]) for c in cfgs}
    for s in ("MUSCL", "MHM", "Godunov"):
        for r in ("HLL", "HLLC", "PVRS", "StegerWarming"):
            assert any(k[0] == s and k[1] == r for k in seen), (s, r)
    assert any(k[0] == "Lax" and k[3] == "Regular" for k in seen)
    assert any(k[0] == "Lax" and k[3] != "Regular" for k in seen)
    for b in ("Regular", "IDWBaseGFM", "LinearBaseGFM", "RiemannBaseGFM", "BCGFM", "HBCGFM"):
        assert any(k[3] == b for k in seen), b
    assert any(k[2] == "VanLeer" for k in seen)
    assert any(k[4] == "periodic" for k in seen)


def test_reference_step_leaves_solid_cells_as_they_are():
    """The reference copies U_NEW into U_OLD for fluid cells only
    (IDWBaseGFM/GFM_Bound.cpp:24-35) and rewrites the ghost cells and the
    domain ring: every other cell keeps what the caller put there, step after
    step.  ibtfo_put_state and the in-place ibtfo_step_host keep this."""
    from ibtfo_gb300 import cases
    w = cases.inclined_channel(128, 64)
    g = w.grid
    o = oracle.OracleCase(g.n_x, g.n_y, g.ng, (g.lo_x, g.lo_y), (g.hi_x, g.hi_y), w.gamma, w.cfl, w.scheme,
                          w.riemann, w.limiter, w.boundary, w.gbc)
    o.setup_geometry(cases.channel_phi(g))
    types = o.get("XYCOORD").reshape(g.N, g.M, 6)[..., 5]
    u0 = cases.channel_init(g, types.reshape(-1), w.gamma).reshape(g.N, g.M, 4)
    solid = types == 1
    solid[:2 * g.ng, :] = solid[-2 * g.ng:, :] = False  # the ring and the cells its fill reads
    solid[:, :2 * g.ng] = solid[:, -2 * g.ng:] = False
    assert solid.sum() > 1000
    mark = np.array([7.0, 0.5, -0.25, 30.0])
    u0[solid] = mark
    o.set_initial_state(u0.reshape(-1))
    o.run(3)
    u = o.get("U_OLD").reshape(g.N, g.M, 4)
    assert (u[solid] == mark).all()
    assert not np.array_equal(u[types == 0], u0[types == 0])  # the fluid did move
    o.close()
