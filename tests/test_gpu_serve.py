"""Device-side case set-up and the serving loop (GPU).

* Bodies: the GPU level set of a circle equals the closed form; an ellipse's
  equals the distance to the outline (nearest point found by refined
  sampling) within 1e-9 near the body, with the sign of the inside test.
* The GPU initial state equals the host-built one bit for bit, and a case set
  up either way advances identically.
* Serving: every request's result (steps, loop time, mass, final density) is
  the same as the same request run alone through the one-case API, bit for
  bit; the memory budget and the active-case limit hold; each result's times
  are ordered arrival <= admitted <= finished."""
import math

import numpy as np
import pytest

ib = pytest.importorskip("ibtfo_gb300")
from ibtfo_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu


def test_circle_level_set_matches_closed_form():
    g = cases.Grid(96, 64, 2, 0.0, 0.0, 1.5, 1.0)
    with ib.Case(g.n_x, g.n_y, lo=(0, 0), hi=(1.5, 1.0), boundary="IDWBaseGFM") as c:
        c.setup_bodies([ib.circle(0.6, 0.45, 0.2)])
        phi_gpu = c.get_geometry().reshape(-1, 6)[:, 2]
        ref = cases.cylinder_phi(g, 0.6, 0.45, 0.2)
        assert np.allclose(phi_gpu, ref, rtol=0, atol=1e-14)
        with ib.Case(g.n_x, g.n_y, lo=(0, 0), hi=(1.5, 1.0), boundary="IDWBaseGFM") as h:
            h.setup_geometry(ref)
            assert np.array_equal(h.get_geometry(), c.get_geometry())
            assert h.num_ghost_cells == c.num_ghost_cells > 0


def test_ellipse_level_set_matches_sampled_outline():
    g = cases.Grid(96, 96, 2, 0.0, 0.0, 1.0, 1.0)
    xc, yc, a, b, th = 0.52, 0.47, 0.3, 0.12, 0.6
    with ib.Case(g.n_x, g.n_y, boundary="IDWBaseGFM") as c:
        c.setup_bodies([ib.ellipse(xc, yc, a, b, th)])
        xy = c.get_geometry().reshape(-1, 6)
    def outline(t):
        return (xc + a * np.cos(t) * math.cos(th) - b * np.sin(t) * math.sin(th),
                yc + a * np.cos(t) * math.sin(th) + b * np.sin(t) * math.cos(th))

    near = np.abs(xy[:, 2]) < 4 * (g.hi_x - g.lo_x) / g.n_x
    assert near.sum() > 100
    px, py = xy[near, 0, None], xy[near, 1, None]
    # nearest outline parameter: a coarse sample, then three local refinements
    # (each shrinks the spacing 32-fold) around the best sample of each point
    h = 2 * math.pi / 4096
    t = np.arange(4096) * h
    ex, ey = outline(t)
    best = t[np.argmin((px - ex[None]) ** 2 + (py - ey[None]) ** 2, axis=1)][:, None]
    for _ in range(3):
        tt = best + np.linspace(-h, h, 65)[None]
        ex, ey = outline(tt)
        k = np.argmin((px - ex) ** 2 + (py - ey) ** 2, axis=1)
        best = tt[np.arange(tt.shape[0]), k][:, None]
        h /= 32
    ex, ey = outline(best)
    d = np.sqrt((px - ex) ** 2 + (py - ey) ** 2)[:, 0]
    px, py = px[:, 0], py[:, 0]
    assert np.max(np.abs(np.abs(xy[near, 2]) - d)) < 1e-9
    # sign: negative inside
    u = (px - xc) * math.cos(th) + (py - yc) * math.sin(th)
    v = -(px - xc) * math.sin(th) + (py - yc) * math.cos(th)
    inside = (u / a) ** 2 + (v / b) ** 2 < 1
    assert np.all((xy[near, 2] < 0) == inside)


@pytest.mark.parametrize("precision", ["fp64_fast", "fp32c"])
def test_device_initial_state_equals_host_built(precision):
    g = cases.Grid(128, 64, 2, 0.0, 0.0, 2.0, 1.0)
    mach, xs = 2.5, 0.4
    post = ib.post_shock_state(mach)
    assert np.allclose(post, cases.post_shock(mach), rtol=1e-15)
    kw = dict(lo=(0, 0), hi=(2.0, 1.0), cfl=0.45, t_end=1e300, max_iter=2 ** 31 - 1, riemann="HLLC",
              boundary="IDWBaseGFM", precision=precision)
    with ib.Case(g.n_x, g.n_y, **kw) as a, ib.Case(g.n_x, g.n_y, **kw) as b:
        a.setup_bodies([ib.circle(1.0, 0.5, 0.15)])
        a.init_x_split(xs, post, (1.0, 0.0, 0.0, 1.0))
        b.setup_geometry(cases.cylinder_phi(g, 1.0, 0.5, 0.15))
        b.set_state(cases.shock_init(g, b.cell_types(), mach, xs))
        assert np.array_equal(a.get_state(), b.get_state())
        assert a.progress() == b.progress()
        a.release_geometry()
        a.advance(30)
        b.advance(30)
        assert np.array_equal(a.get_state(), b.get_state())
        assert np.array_equal(a.density(), b.get_state().reshape(g.N, g.M, 4)[2:-2, 2:-2, 0])
        with pytest.raises(ib.IbtfoError):
            a.get_geometry()


def shock_cylinder_request(rid, n_x, n_y, mach, r_frac, cx, cy, arrival=0.0, density_out=None):
    W = 1.0
    H = W * n_y / n_x
    post = cases.post_shock(mach)
    shock_speed = mach * math.sqrt(1.4)
    t_end = 0.3 * W / shock_speed  # a shorter run than the served stream's 1.5 crossings
    body = ib.circle(cx * W, cy * H, r_frac * H)
    return ib.request(rid, n_x, n_y, (0.0, 0.0), (W, H), t_end, bodies=[body], x_split=0.1 * W, left=post,
                      right=(1.0, 0.0, 0.0, 1.0), arrival=arrival, density_out=density_out)


def alone(req, precision="fp32c"):
    c = ib.Case(req.n_x, req.n_y, lo=(req.lo_x, req.lo_y), hi=(req.hi_x, req.hi_y), gamma=req.gamma,
                cfl=req.cfl_number, t_end=req.t_end, max_iter=2 ** 31 - 1, scheme="MUSCL", riemann="HLLC",
                boundary="IDWBaseGFM", precision=precision)
    with c:
        c.setup_bodies([req.bodies[k] for k in range(req.n_bodies)])
        c.init_x_split(req.x_split, list(req.left), list(req.right))
        p = c.run()
        return p, c.density()


def stream(n, seed=7):
    # arrivals in groups of three, 4 ms apart: a group's requests are active
    # together however fast each one runs
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        nx = int(rng.choice([64, 96, 128, 160]))
        ny = int(nx // rng.choice([1, 2]))
        out.append((k, nx, ny, float(rng.uniform(1.5, 4.0)), float(rng.uniform(0.05, 0.2)),
                    float(rng.uniform(0.35, 0.7)), float(rng.uniform(0.3, 0.7)), 0.004 * (k // 3)))
    return out


def test_served_results_equal_alone_runs():
    reqs = stream(10)
    bufs = {k: ib.PinnedBuffer(nx * ny) for (k, nx, ny, *_rest) in reqs}
    # the case path's tiles (32x16): the mass sums bit for bit as well
    with ib.Server(precision="fp32c", chunk_steps=16, tile_shape="32x16") as srv:
        built = {}
        for (k, nx, ny, m, rf, cx, cy, arr) in reqs:
            r = shock_cylinder_request(k, nx, ny, m, rf, cx, cy, arrival=arr, density_out=bufs[k])
            built[k] = r
            srv.submit(r)
        srv.run(max_seconds=600)
        res = {r["id"]: r for r in srv.poll()}
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["peak_active"] >= 2
    for k, r in res.items():
        assert r["status"] == 0
        assert r["arrival"] <= r["admitted"] <= r["finished"]
        p, rho = alone(built[k])
        assert r["iter"] == p["iter"] and r["now_t"] == p["now_t"], k
        assert r["mass"] == p["mass"] and r["nan_cells"] == p["nan_cells"] == 0, k
        nx, ny = built[k].n_x, built[k].n_y
        assert np.array_equal(bufs[k].array.reshape(ny, nx), rho), k
    for b in bufs.values():
        b.close()


def test_server_respects_budget_and_active_limit():
    reqs = stream(8, seed=11)
    cfg = ib.config(160, 160, boundary="IDWBaseGFM", precision="fp32c")
    resident, setup = ib.case_bytes(cfg)
    budget = 2 * setup + resident // 2  # room for about two of the largest cases
    with ib.Server(precision="fp32c", chunk_steps=16, memory_budget=budget, max_active=3) as srv:
        for (k, nx, ny, m, rf, cx, cy, arr) in reqs:
            srv.submit(shock_cylinder_request(k, nx, ny, m, rf, cx, cy))
        srv.run(max_seconds=600)
        res = srv.poll()
        st = srv.stats()
    assert len(res) == len(reqs) and all(r["status"] == 0 for r in res)
    assert st["peak_bytes"] <= budget and st["peak_active"] <= 3
    # a request that can never fit fails cleanly
    with ib.Server(precision="fp32c", memory_budget=resident // 4) as srv:
        srv.submit(shock_cylinder_request(99, 160, 160, 2.0, 0.1, 0.5, 0.5))
        srv.run(max_seconds=60)
        (r,) = srv.poll()
        assert r["status"] == 2  # IBTFO_ENOMEM


def served_stream_picks(n, min_mach=3.0, max_cells=200_000):
    """The first `n` requests of the seed-42 served stream with shock Mach >=
    min_mach and at most max_cells cells (the bench serves the stream's first
    64 requests at every size)."""
    return [r for r in cases.served_stream(200, 1.0, seed=42)
            if r.mach >= min_mach and r.n_x * r.n_y <= max_cells][:n]


def test_served_fp32_within_1e5_of_fp64_at_high_mach():
    """Served FP32 results against the FP64 path (fp64_fast, the plain path
    pinned to the oracle at 1e-12) on Mach >= 3 requests of the bench's
    stream (HLL_Toro, Time = RK2, CFL 0.45, 1.5 crossings): relative L1 density error <=
    1e-5 at the served run's step count.  The plain run is taken to exactly
    that step count, so what is compared is the arithmetic, not where each
    run's loop stopped (at the first now_t >= t_end, Test/Sod/Sod.cpp:123)."""
    picks = served_stream_picks(5)
    assert len(picks) >= 4 and all(r.mach >= 3.0 for r in picks)
    bufs = {r.id: ib.PinnedBuffer(r.n_x * r.n_y) for r in picks}
    post = {r.id: cases.post_shock(r.mach) for r in picks}
    with ib.Server(riemann=cases.SERVE_RIEMANN, precision="fp32c", chunk_steps=32, tile_shape="32x16",
                   time=cases.SERVE_TIME) as srv:
        for r in picks:
            srv.submit(ib.request(r.id, r.n_x, r.n_y, (0.0, 0.0), (r.width, r.height), r.t_end,
                                  bodies=[ib.circle(r.xc, r.yc, r.radius)], x_split=r.x_shock, left=post[r.id],
                                  right=(1.0, 0.0, 0.0, 1.0), cfl=r.cfl, density_out=bufs[r.id]))
        srv.run(max_seconds=600)
        res = {q["id"]: q for q in srv.poll()}
    errs = {}
    for r in picks:
        q = res[r.id]
        assert q["status"] == 0 and q["nan_cells"] == 0
        with ib.Case(r.n_x, r.n_y, lo=(0.0, 0.0), hi=(r.width, r.height), cfl=r.cfl, t_end=1e300,
                     max_iter=q["iter"], scheme="MUSCL", riemann=cases.SERVE_RIEMANN, boundary="IDWBaseGFM",
                     precision="fp64_fast", time=cases.SERVE_TIME) as c:
            c.setup_bodies([ib.circle(r.xc, r.yc, r.radius)])
            c.init_x_split(r.x_shock, post[r.id], (1.0, 0.0, 0.0, 1.0))
            p = c.run()
            assert p["iter"] == q["iter"]
            assert abs(p["now_t"] - q["now_t"]) <= 1e-6 * p["now_t"]
            rho = c.density().reshape(-1)
        errs[r.id] = float(np.abs(bufs[r.id].array - rho).sum() / np.abs(rho).sum())
    for b in bufs.values():
        b.close()
    assert max(errs.values()) <= 1e-5, errs
