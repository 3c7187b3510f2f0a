"""Batches (persistent batched sweep over many cases) against the same cases
run alone.

The bar is bit-for-bit: a case in a batch runs the same tile body as the
one-case kernels, so its state, dt, loop time and step count after n steps
equal those of the case advanced alone; with the 32 x 8 tile shape the mass
sum is bitwise equal as well (other shapes sum the per-tile mass partials in
another order: relative 1e-12).  Covers uneven grid sizes, ghost-fluid and
plain boundaries, walls and periodic domain edges (the two-phase boundary
pass), per-case loop ends, cases joining and leaving between steps, tile
shapes, Time = RK2, and the autotuner's trial steps."""
import numpy as np
import pytest

ib = pytest.importorskip("ibtfo_gb300")
from ibtfo_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu

BIG = 1e300


def specs():
    """(workload, phi, init(types) -> u0) of four unevenly sized cases, all
    MUSCL + HLLC + minmod (one kernel variant)."""
    out = []
    w = cases.inclined_channel(192, 96)
    w.t_end = BIG
    g = w.grid
    out.append((w, cases.channel_phi(g), lambda t, g=g: cases.channel_init(g, t)))
    g2 = cases.Grid(160, 40, 2, 0.0, 0.0, 1.0, 0.25)
    w2 = cases.Workload("sod", g2, 1.4, 0.5, BIG, "MUSCL", "HLLC", "minmod", "Regular")
    phi2, u2 = cases.sod_x(g2)
    out.append((w2, phi2, lambda t, u=u2: u))
    g3 = cases.Grid(128, 128, 2, 0.0, 0.0, 1.0, 1.0)
    w3 = cases.Workload("cylinder_periodic", g3, 1.4, 0.45, BIG, "MUSCL", "HLLC", "minmod", "LinearBaseGFM",
                        gbc="periodic")
    out.append((w3, cases.cylinder_phi(g3, 0.5, 0.5, 0.15),
                lambda t, g=g3: cases.uniform_init(g, t, (1.0, 0.5, 0.25, 1.0))))
    g4 = cases.Grid(96, 24, 2, 0.0, 0.0, 1.0, 0.25)
    w4 = cases.Workload("sod_short", g4, 1.4, 0.5, 0.01, "MUSCL", "HLLC", "minmod", "Regular")
    phi4, u4 = cases.sod_x(g4)
    out.append((w4, phi4, lambda t, u=u4: u))
    return out


def make(spec, precision, **over):
    w, phi, init = spec
    c = ib.Case.from_workload(w, precision=precision, max_iter=2 ** 31 - 1, **over)
    c.setup_geometry(phi)
    c.set_state(init(c.cell_types()))
    return c


def alone(spec, precision, n, **over):
    with make(spec, precision, **over) as c:
        c.advance(n)
        return c.get_state(), c.progress()


def same(a, b, exact_mass=True):
    (ua, pa), (ub, pb) = a, b
    assert np.array_equal(ua, ub, equal_nan=True)
    for k in ("iter", "now_t", "dt", "nan_cells", "status"):
        assert pa[k] == pb[k], (k, pa[k], pb[k])
    if exact_mass:
        assert pa["mass"] == pb["mass"] or (np.isnan(pa["mass"]) and np.isnan(pb["mass"]))
    else:
        assert abs(pa["mass"] - pb["mass"]) <= 1e-12 * abs(pb["mass"])


@pytest.mark.parametrize("precision", ["fp32c", "fp64_fast"])
@pytest.mark.parametrize("shape", ["32x8", "32x16", "64x8"])
def test_batch_equals_alone(precision, shape):
    n = 40  # two graph launches of 16 steps + 8 single steps
    sp = specs()
    ref = [alone(s, precision, n) for s in sp]
    cs = [make(s, precision) for s in sp]
    with ib.Batch("MUSCL", "HLLC", "minmod", precision, tile_shape=shape) as b:
        for c in cs:
            b.add(c)
        assert len(b) == len(cs)
        b.advance(n)
        prog = b.progress()
        b.synchronize()
        for k, c in enumerate(cs):
            # the mass sum is bit for bit where the batch's tiles are the case
            # path's (32x16 for fp64_fast and the FP32 form)
            same((c.get_state(), c.progress()), ref[k], exact_mass=(shape == "32x16"))
            assert prog[k][0]["iter"] == ref[k][1]["iter"]
            assert ref[k][1]["nan_cells"] == 0
    # the short case stopped at its own t_end; the others ran every step
    assert ref[3][1]["iter"] < n and ref[3][1]["now_t"] >= 0.01
    assert all(r[1]["iter"] == n for r in ref[:3])
    for c in cs:
        c.close()


@pytest.mark.parametrize("precision", ["fp32c", "fp64_fast"])
@pytest.mark.parametrize("riemann", ["HLLC", "HLL_Toro"])
def test_rk2_batch_equals_alone(precision, riemann):
    """Time = RK2 in a batch (two sweeps per step, each followed by the
    boundary pass) equals the same cases run alone with RK2, bit for bit on
    the case path's tiles (32x16), for the reference's HLL (HLLC key) and for
    HLL_Toro (whose FP32 form solves faces in difference form)."""
    n = 20  # one graph launch of 16 steps + 4 single steps
    sp = specs()
    over = dict(time="RK2", riemann=riemann)
    ref = [alone(s, precision, n, **over) for s in sp]
    cs = [make(s, precision, **over) for s in sp]
    with ib.Batch("MUSCL", riemann, "minmod", precision, tile_shape="32x16", time="RK2") as b:
        for c in cs:
            b.add(c)
        b.advance(n)
        b.synchronize()
        for k, c in enumerate(cs):
            same((c.get_state(), c.progress()), ref[k])
            assert ref[k][1]["nan_cells"] == 0
        # a single-step case does not join an RK2 batch
        with make(sp[1], precision, riemann=riemann) as other:
            with pytest.raises(ib.IbtfoError):
                b.add(other)
    for c in cs:
        c.close()


def test_batch_join_and_leave():
    precision = "fp32c"
    sp = specs()
    a, bb, cc = make(sp[0], precision), make(sp[1], precision), make(sp[2], precision)
    # the case path's tiles (32x16): the mass sums bit for bit as well
    with ib.Batch("MUSCL", "HLLC", "minmod", precision, tile_shape="32x16") as b:
        sa = b.add(a)
        b.add(bb)
        b.advance(20)
        b.add(cc)                     # joins after 20 steps
        b.advance(20)
        b.remove(sa)                  # leaves after 40 steps
        b.advance(20)
        b.synchronize()
        same((a.get_state(), a.progress()), alone(sp[0], precision, 40))
        same((bb.get_state(), bb.progress()), alone(sp[1], precision, 60))
        same((cc.get_state(), cc.progress()), alone(sp[2], precision, 40))
        assert len(b) == 2
    for c in (a, bb, cc):
        c.close()


def test_batch_autotune_steps_are_real_steps():
    precision = "fp32c"
    sp = specs()[:2]
    cs = [make(s, precision) for s in sp]
    with ib.Batch("MUSCL", "HLLC", "minmod", precision) as b:
        for c in cs:
            b.add(c)
        best, trials = b.autotune(steps=2)
        assert trials and best["ms_per_step"] > 0
        assert best["tile_shape"] in ib.TILE_SHAPES and 1 <= best["ctas_per_sm"] <= best["max_ctas_per_sm"]
        assert best["ms_per_step"] == min(t["ms_per_step"] for t in trials)
        steps = 3 * len(trials)        # one warm-up + two timed steps per trial
        b.synchronize()
        for k, c in enumerate(cs):
            same((c.get_state(), c.progress()), alone(sp[k], precision, steps), exact_mass=False)
    for c in cs:
        c.close()


def test_batch_rejects_mismatched_cases():
    sp = specs()
    c = make(sp[1], "fp64_fast")
    with ib.Batch("MUSCL", "HLLC", "minmod", "fp32c") as b:
        with pytest.raises(ib.IbtfoError):
            b.add(c)
    with pytest.raises(ib.IbtfoError):
        ib.Batch("MUSCL", "HLLC", "minmod", "fp64")
    c.close()
