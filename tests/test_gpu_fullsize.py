"""GPU checks at the benchmark workloads' full sizes.

The smaller parity tests compare the CUDA path with the oracle on grids the
oracle finishes in a blink; these run the three benchmark workloads at the
size the bench times them, against the oracle where it finishes in seconds
and through size-independent properties where it does not:

* inclined channel, 2048x1024, MUSCL + HLLC + minmod, IDWBaseGFM: geometry
  bit for bit, dt / mass sequences and state within 1e-12 relative of the
  oracle after 10 steps, and the run to t_end = 0.2 with the oracle's step
  count and L1 density within 1e-10 (both FP64 keys); the host-array step (row bands
  copied while the sweep runs) bit for bit with put + step + get;
* periodic isentropic vortex, 4096x4096, MHM + minmod: with the reference's
  HLLC and single steps, within 1e-12 of the oracle after 3 steps; with the
  timed workload's HLL_Toro and Time = RK2, a periodic shift of the initial state gives
  the same shift of the result bit for bit (tile seams land on other cells),
  mass and energy are conserved (FP64 to 1e-11 relative after 20 steps: the
  rounding of 16.7 M cell updates a step accumulates; the FP32 compensated
  form to 1e-9), and the FP32 compensated form stays within 1e-5 (relative L1
  density) of FP64;
* Mach 3 shock over 24 seeded bodies with cut cells, 8192x4096 (the shock
  started inside the obstacle field): the volume
  fractions, apertures and cell types from the GPU's level set bit for bit
  with the cut-cell oracle's from the same level set, the state within 1e-12
  of the oracle after 2 FP64 steps (fluid cells; alpha U in cut cells) (the mass to n 2^-53 of the oracle's,
  which sums 33.5 M cells in one sequential loop, and to 1e-12 of a pairwise
  sum of the state), and the FP32 compensated form without NaN
  and within 1e-5 (relative L1 density) of FP64.
"""
import numpy as np
import pytest

import oracle
from test_gpu_host import same_progress
from test_gpu_parity import assert_state_close, seq_close

ib = pytest.importorskip("ibtfo_gb300")
from ibtfo_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu

FOREVER = dict(t_end=1e300, max_iter=2 ** 31 - 1)


def oracle_case(w, riemann=None):
    g = w.grid
    return oracle.OracleCase(g.n_x, g.n_y, g.ng, (g.lo_x, g.lo_y), (g.hi_x, g.hi_y), w.gamma, w.cfl, w.scheme,
                             riemann or w.riemann, w.limiter, w.boundary, w.gbc)


def steps_with_progress(c, n):
    dts, ms = [], []
    for _ in range(n):
        c.advance(1)
        p = c.progress()
        dts.append(p["dt"])
        ms.append(p["mass"])
    return np.array(dts), np.array(ms)


# ------------------------------------------------------------ inclined channel

CHANNEL_STEPS = 10


@pytest.fixture(scope="module")
def channel_oracle():
    w = cases.inclined_channel()
    oracle.set_threads(16)
    phi = cases.channel_phi(w.grid)
    o = oracle_case(w)
    o.setup_geometry(phi)
    types = o.get("XYCOORD").reshape(-1, 6)[:, 5]
    u0 = cases.channel_init(w.grid, types, w.gamma)
    o.set_initial_state(u0)
    xy = o.get("XYCOORD")
    dts, ms = o.run(CHANNEL_STEPS)
    out = dict(w=w, phi=phi, u0=u0, xy=xy, dts=dts, ms=ms, u_old=o.get("U_OLD"), u_new=o.get("U_NEW"),
               now_t=o.scalars()["now_t"])
    o.close()
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp64_fast"])
def test_channel_full_size_matches_oracle(channel_oracle, precision):
    ref = channel_oracle
    w = ref["w"]
    assert (w.grid.n_x, w.grid.n_y) == (2048, 1024)
    with ib.Case.from_workload(w, precision=precision) as c:
        c.setup_geometry(ref["phi"])
        assert np.array_equal(c.get_geometry(), ref["xy"]), "geometry differs"
        c.set_state(ref["u0"])
        dts, ms = steps_with_progress(c, CHANNEL_STEPS)
        assert seq_close(dts, ref["dts"]), "dt sequence differs"
        assert seq_close(ms, ref["ms"]), "mass sequence differs"
        assert seq_close([c.progress()["now_t"]], [ref["now_t"]])
        uo, un = c.get_state(u_new=True)
    assert_state_close(uo, ref["u_old"], "U_OLD")
    assert_state_close(un, ref["u_new"], "U_NEW")


@pytest.fixture(scope="module")
def channel_oracle_t_end():
    """The oracle's run of the full channel to its t_end = 0.2 (the loop of
    Test/InclineSod/InclineSod.cpp:131-189: stop at the first now_t >= t_end)."""
    w = cases.inclined_channel()
    oracle.set_threads(16)
    phi = cases.channel_phi(w.grid)
    o = oracle_case(w)
    o.setup_geometry(phi)
    u0 = cases.channel_init(w.grid, o.get("XYCOORD").reshape(-1, 6)[:, 5], w.gamma)
    o.set_initial_state(u0)
    o.run(10 ** 6, w.t_end)
    out = dict(w=w, phi=phi, u0=u0, u_old=o.get("U_OLD"), **o.scalars())
    o.close()
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp64_fast"])
def test_channel_full_size_to_t_end(channel_oracle_t_end, precision):
    """2048x1024 inclined channel run to t_end = 0.2 (about 500 steps): the
    same step count and now_t as the oracle, and L1 density within 1e-10
    (relative) of the oracle's."""
    ref = channel_oracle_t_end
    w = ref["w"]
    with ib.Case.from_workload(w, precision=precision) as c:
        c.setup_geometry(ref["phi"])
        c.set_state(ref["u0"])
        p = c.run()
        u = c.get_state()
    assert p["iter"] == ref["iter"], (p["iter"], ref["iter"])
    assert seq_close([p["now_t"]], [ref["now_t"]])
    a = u.reshape(-1, 4)[:, 0]
    b = ref["u_old"].reshape(-1, 4)[:, 0]
    l1 = float(np.abs(a - b).sum() / np.abs(b).sum())
    assert l1 <= 1e-10, l1


def test_channel_full_size_host_step_equals_put_step_get():
    """The row-band pipeline of ibtfo_step_host on the full 2048x1024 grid
    (eight bands, copies overlapped with the sweep, graph replays) leaves the
    bytes that put + step + get leave."""
    w = cases.inclined_channel()
    g = w.grid
    phi = cases.channel_phi(g)

    def make():
        c = ib.Case.from_workload(w, precision="fp64_fast", **FOREVER)
        c.setup_geometry(phi)
        c.set_state(cases.channel_init(g, c.cell_types(), w.gamma))
        return c

    n = g.M * g.N * 4
    with make() as a:
        u = a.get_state()
        for _ in range(5):
            a.put_state_ptr(u.ctypes.data)
            a.step()
            u = a.get_state()
        ref, pref = u.copy(), a.progress()
    buf = ib.PinnedBuffer(n)
    try:
        with make() as b:
            b.get_state_ptr(buf.ptr)
            for _ in range(5):
                p = b.step_host_ptr(buf.ptr, buf.ptr)
            assert np.array_equal(buf.array, ref)
            same_progress(p, pref)
    finally:
        buf.close()


# ------------------------------------------------------------ isentropic vortex

def periodic_state(g, interior):
    """(N, M, 4) state whose ghost layers are the periodic images of `interior`."""
    ng = g.ng
    return np.ascontiguousarray(np.pad(interior, ((ng, ng), (ng, ng), (0, 0)), mode="wrap")).reshape(-1)


def vortex_interior(g):
    _, u0 = cases.isentropic_vortex(g)
    return u0.reshape(g.N, g.M, 4)[g.ng:-g.ng, g.ng:-g.ng].copy()


def interior_of(g, u):
    return u.reshape(g.N, g.M, 4)[g.ng:-g.ng, g.ng:-g.ng]


def test_vortex_full_size_matches_oracle():
    """4096x4096 periodic vortex with the reference's HLLC, 3 steps (the
    reference's HLLC goes to NaN on this flow after a few dozen steps, not in 3)."""
    w = cases.vortex_periodic(4096, riemann="HLLC", time="SingleStep")
    g = w.grid
    phi, _ = cases.isentropic_vortex(g)
    u0 = periodic_state(g, vortex_interior(g))
    oracle.set_threads(16)
    o = oracle_case(w)
    o.setup_geometry(phi)
    o.set_initial_state(u0)
    odts, oms = o.run(3)
    ref = o.get("U_OLD")
    o.close()
    for precision in ("fp64", "fp64_fast"):
        with ib.Case.from_workload(w, precision=precision, **FOREVER) as c:
            c.setup_geometry(phi)
            c.set_state(u0)
            dts, ms = steps_with_progress(c, 3)
            assert seq_close(dts, odts) and seq_close(ms, oms), precision
            assert_state_close(c.get_state(), ref, f"U_OLD {precision}")


def run_vortex(w, precision, u0, phi, steps):
    with ib.Case.from_workload(w, precision=precision, **FOREVER) as c:
        c.setup_geometry(phi)
        c.set_state(u0)
        p0 = c.progress()
        dts, _ = steps_with_progress(c, steps)
        return c.get_state(), dts, p0


@pytest.mark.parametrize("precision", ["fp64_fast", "fp32c"])
def test_vortex_full_size_shift_equivariance(precision):
    """The update of a cell reads only its neighbours and the domain's global
    maximum wave speed, so on a periodic domain shifting the initial state by
    (37, 1001) cells shifts the state after 6 steps by the same amount, bit
    for bit, although the 32x8 tiles now cut the field along other cells."""
    w = cases.vortex_periodic(4096)
    g = w.grid
    phi, _ = cases.isentropic_vortex(g)
    base = vortex_interior(g)
    shift = (37, 1001)
    ua, dta, _ = run_vortex(w, precision, periodic_state(g, base), phi, 6)
    ub, dtb, _ = run_vortex(w, precision, periodic_state(g, np.roll(base, shift, axis=(0, 1))), phi, 6)
    assert np.array_equal(dta, dtb)
    assert np.array_equal(np.roll(interior_of(g, ua), shift, axis=(0, 1)), interior_of(g, ub))


@pytest.mark.parametrize("precision,bar", [("fp64_fast", 1e-11), ("fp32c", 1e-9)])
def test_vortex_full_size_conservation(precision, bar):
    w = cases.vortex_periodic(4096)
    g = w.grid
    phi, _ = cases.isentropic_vortex(g)
    u0 = periodic_state(g, vortex_interior(g))
    u, _, _ = run_vortex(w, precision, u0, phi, 20)
    a, b = interior_of(g, u0), interior_of(g, u)
    assert np.isfinite(b).all()
    for k in (0, 3):
        s0, s1 = a[..., k].sum(dtype=np.float64), b[..., k].sum(dtype=np.float64)
        assert abs(s1 - s0) / abs(s0) <= bar, (k, abs(s1 - s0) / abs(s0))


def test_vortex_full_size_fp32c_against_fp64():
    w = cases.vortex_periodic(4096)
    g = w.grid
    phi, _ = cases.isentropic_vortex(g)
    u0 = periodic_state(g, vortex_interior(g))
    u64, d64, _ = run_vortex(w, "fp64_fast", u0, phi, 20)
    u32, d32, _ = run_vortex(w, "fp32c", u0, phi, 20)
    r64, r32 = interior_of(g, u64)[..., 0], interior_of(g, u32)[..., 0]
    assert np.isfinite(r32).all()
    l1 = float(np.abs(r32 - r64).sum() / np.abs(r64).sum())
    assert l1 <= 1e-5, l1
    assert np.allclose(d32, d64, rtol=1e-5, atol=0)


# ------------------------------------------------------------ cut cells

def obstacle_bodies(obstacles):
    return [ib.circle(o.xc, o.yc, o.a) if o.kind == "circle" else ib.ellipse(o.xc, o.yc, o.a, o.b, o.theta)
            for o in obstacles]


def test_cut_cells_full_size_matches_oracle():
    """The Mach 3 shock over the 24 seeded circles and ellipses at 8192x4096:
    the level set the GPU builds from the bodies goes to the cut-cell oracle,
    which must derive the same geometry from it; then 2 FP64 steps of both.
    The shock starts at x = 2.4, inside the obstacle field (the timed
    workload starts it at x = 0.5, a few thousand steps before the first
    body), so that these steps update and mix cut cells in moving flow."""
    w = cases.shock_obstacles()
    g = w.grid
    bodies = obstacle_bodies(cases.random_obstacles())
    post = cases.post_shock(3.0)
    steps = 2
    res = {}
    for precision in ("fp64_fast", "fp32c"):
        with ib.Case.from_workload(w, precision=precision, **FOREVER) as c:
            c.setup_bodies(bodies)
            if precision == "fp64_fast":
                phi = c.get_geometry().reshape(-1, 6)[:, 2].copy()
                alpha, ax, ay = c.cut_cells()
                types = c.cell_types().reshape(g.N, g.M)
            c.init_x_split(2.4, post, (1.0, 0.0, 0.0, 1.0))
            c.release_geometry()
            u0 = c.get_state()
            p0 = c.progress()
            dts, ms = steps_with_progress(c, steps)
            res[precision] = (u0, p0, dts, ms, c.get_state())
    o = oracle.CcmOracle(g.n_x, g.n_y, g.ng, (g.lo_x, g.lo_y), (g.hi_x, g.hi_y), w.gamma, w.cfl, 1e300, w.scheme,
                         w.riemann, w.limiter, w.gbc)
    try:
        o.setup(phi)
        oa, oax, oay, ot = o.geometry()
        assert np.array_equal(types, ot), "cell types differ"
        assert np.array_equal(alpha, oa) and np.array_equal(ax, oax) and np.array_equal(ay, oay), \
            "volume fractions or apertures differ"
        u0, p0, dts, ms, u = res["fp64_fast"]
        o.set_state(u0)
        assert seq_close([p0["dt"]], [o.scalars()["dt"]])
        odts, oms = o.run(steps)
        # the cut-cell oracle lists the dt each step used, progress() the next one
        assert seq_close(odts, np.concatenate([[p0["dt"]], dts[:-1]]))
        assert seq_close(dts[-1:], [o.scalars()["dt"]])
        # the oracle sums the 33.5 M cells' masses in one sequential loop, whose
        # rounding is bounded by n 2^-53 = 3.7e-9 relative (measured 1.9e-10:
        # in uniform regions each addition rounds the same way); the GPU's
        # per-block partial sums agree with a pairwise sum of the state to 1e-12
        dm = float(np.max(np.abs(ms - oms) / np.abs(oms)))
        assert dm <= g.n_x * g.n_y * 2.0 ** -53, dm
        upd2 = (ot == 0) | (ot == 3)
        area = (g.hi_x - g.lo_x) / g.n_x * ((g.hi_y - g.lo_y) / g.n_y)
        m_pairwise = float((alpha * u.reshape(g.N, g.M, 4)[..., 0])[upd2].sum()) * area
        assert abs(ms[-1] - m_pairwise) <= 1e-12 * m_pairwise, (ms[-1], m_pairwise)
        # fluid cells (type 0): the state to 1e-12; cut cells (type 3): the
        # conserved amounts alpha U to 1e-12 of each variable's scale.  A cut
        # cell's update divides its flux balance by alpha (down to 1e-10), so
        # a last-bit difference of a flux appears in U amplified by 1/alpha
        # and in alpha U at its own size.
        uo = o.get_state().reshape(-1, 4)
        ug = u.reshape(-1, 4)
        fl = (ot == 0).reshape(-1)
        assert_state_close(ug[fl], uo[fl], "fluid cells")
        cut = (ot == 3).reshape(-1)
        al = alpha.reshape(-1)[cut][:, None]
        scale = np.abs(uo[fl]).max(axis=0)
        d = np.abs(al * ug[cut] - al * uo[cut]) / scale
        k = np.unravel_index(int(np.argmax(d)), d.shape)
        assert d.max() <= 1e-12, (float(d.max()), "alpha", float(al[k[0], 0]), "variable", int(k[1]),
                                  "U", float(np.abs(ug[cut][k] - uo[cut][k]) / scale[k[1]]))
        moved = np.abs(u.reshape(-1, 4)[cut] - u0.reshape(-1, 4)[cut]).max(axis=1) > 1e-3
        assert moved.sum() > 1000, int(moved.sum())
    finally:
        o.close()
    r64 = u.reshape(-1, 4)[:, 0]
    r32 = res["fp32c"][4].reshape(-1, 4)[:, 0]
    assert np.isfinite(res["fp32c"][4]).all()
    l1 = float(np.abs(r32 - r64).sum() / np.abs(r64).sum())
    assert l1 <= 1e-5, l1
