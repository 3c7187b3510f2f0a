"""Time = RK2 in the CPU oracle (no GPU).

The reference's RK2 (Src/Base/TimeAdvance/RK2/RK2.cpp) does not compile, so
there is no reference output to pin it to; the oracle restates the two-stage
method that file describes (Heun's method over the reference's own Advance,
Boundary and Global_Boundary).  These tests pin the restatement to its
definition, built here from the oracle's single-stage calls, and check the
properties the method must have: conservation in a periodic box and a
second-order error in time where the single step is first order."""
import numpy as np
import pytest

import oracle
from ibtfo_gb300 import cases


def _vortex(n=32, scheme="MUSCL", time="SingleStep", cfl=0.1, riemann="HLL"):
    g = cases.Grid(n, n, 2, 0.0, 0.0, 10.0, 10.0)
    phi, u0 = cases.isentropic_vortex(g, 1.4, beta=5.0)
    o = oracle.OracleCase(n, n, 2, (0, 0), (10, 10), 1.4, cfl, scheme, riemann, "minmod", "Regular", "periodic",
                          time=time)
    o.setup_geometry(phi)
    o.set_initial_state(u0)
    return g, o


@pytest.mark.parametrize("scheme", ["MUSCL", "MHM", "Godunov", "Lax"])
def test_rk2_step_is_heun_over_the_single_stage_calls(scheme):
    g, o = _vortex(scheme=scheme, time="RK2")
    _, s = _vortex(scheme=scheme)
    for _ in range(3):
        o.run(1)
        dt = s.scalars()["dt"]
        u0 = s.get("U_OLD").copy()
        L = s.L
        L.or_advance(s.h, dt)
        L.or_boundary(s.h)
        L.or_global_boundary(s.h)
        u1 = s.get("U_OLD").copy()
        L.or_advance(s.h, dt)
        un = s.get("U_NEW").reshape(-1, 4)
        t = s.get("XYCOORD").reshape(-1, 6)[:, 5]
        fl = t == 0
        un[fl] = 0.5 * (u0.reshape(-1, 4)[fl] + un[fl])
        un[~fl] = u1.reshape(-1, 4)[~fl]
        # interior cells only: the combine covers [ng, n + ng) in both directions
        m = np.zeros((g.N, g.M), bool)
        m[g.ng:-g.ng, g.ng:-g.ng] = True
        full = s.get("U_NEW").reshape(-1, 4)
        full[m.reshape(-1)] = un[m.reshape(-1)]
        s.put("U_NEW", full.reshape(-1))
        L.or_boundary(s.h)
        L.or_global_boundary(s.h)
        assert np.array_equal(o.get("U_OLD"), s.get("U_OLD"))
        assert o.scalars()["dt"] == L.or_compute_dt(s.h)
        # the next step of the by-hand case starts from this state and dt
        s.set_initial_state(s.get("U_OLD"))


@pytest.mark.parametrize("scheme", ["MUSCL", "Lax"])
def test_rk2_conserves_mass_in_a_periodic_box(scheme):
    _, o = _vortex(scheme=scheme, time="RK2")
    m0 = o.scalars()["mass_now"]
    _, ms = o.run(40)
    assert abs(ms[-1] - m0) <= 1e-12 * m0


def test_rk2_time_error_is_second_order():
    # one step of size dt against two of dt/2 on a fixed grid: the difference
    # is the local error, O(dt^2) for the single step (4x smaller per halving
    # of dt) and O(dt^3) for RK2 (8x).  MUSCL with Steger-Warming: its spatial
    # operator is smooth enough on the subsonic vortex for the orders to show.
    def one(time, dt, nsub):
        _, o = _vortex(n=48, scheme="MUSCL", time=time, riemann="StegerWarming")
        L = o.L
        for _ in range(nsub):
            if time == "RK2":
                u = o.get("U_OLD").copy()
                L.or_advance(o.h, dt)
                L.or_boundary(o.h)
                L.or_global_boundary(o.h)
                L.or_advance(o.h, dt)
                un = o.get("U_NEW").reshape(-1, 4)
                t = o.get("XYCOORD").reshape(-1, 6)[:, 5]
                un[t == 0] = 0.5 * (u.reshape(-1, 4)[t == 0] + un[t == 0])
                o.put("U_NEW", un.reshape(-1))
            else:
                L.or_advance(o.h, dt)
            L.or_boundary(o.h)
            L.or_global_boundary(o.h)
        return o.get("U_OLD").reshape(-1, 4)[:, 0]

    ratios = {}
    for time in ("SingleStep", "RK2"):
        d = [np.abs(one(time, dt, 1) - one(time, dt / 2, 2)).max() for dt in (0.01, 0.005)]
        ratios[time] = d[0] / d[1]
    assert 3.6 < ratios["SingleStep"] < 4.4, ratios
    assert ratios["RK2"] > 6.5, ratios
