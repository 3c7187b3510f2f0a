"""GPU tests of the host-facing layers: the reference-signature entry points
(include/ibtfo_ref.h) driven in the reference driver's call order, and the
C++ time-loop executable ibtfo_run."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import oracle
from golden_util import load

ib = pytest.importorskip("ibtfo_gb300")

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def same_progress(a, b):
    """Loop scalars equal; the mass to 1e-14 relative: fp64_fast and FP32 sum it over
    32x16 tiles in ibtfo_step and over the 32x8 tiles of the host step's row
    bands, an order that changes its last bits."""
    assert {k: v for k, v in a.items() if k != "mass"} == {k: v for k, v in b.items() if k != "mass"}
    assert abs(a["mass"] - b["mass"]) <= 1e-14 * abs(b["mass"]), (a["mass"], b["mass"])


def rel_linf(a, b):
    a, b = a.reshape(-1, 4), b.reshape(-1, 4)
    worst = 0.0
    for k in range(4):
        m = np.isfinite(b[:, k])
        if m.any():
            worst = max(worst, float(np.abs(a[m, k] - b[m, k]).max() / max(np.abs(b[m, k]).max(), 1e-300)))
    return worst


@pytest.mark.parametrize("name", ["refincline_MUSCL_HLL_minmod_IDWBaseGFM", "channel_MUSCL_HLLC_minmod_BCGFM",
                                  "channel_MUSCL_HLLC_minmod_LinearBaseGFM", "sodtube_MUSCL_HLL_minmod",
                                  "refsod_MUSCL_HLL_minmod"])
def test_reference_driver_sequence_through_shim(name, tmp_path, monkeypatch):
    """Test/InclineSod/InclineSod.cpp:97-189 call by call through ibtfo_ref_*,
    with WriteData before the loop and after it (Sod.cpp:139-141, :186)."""
    monkeypatch.chdir(tmp_path)
    fx = load(name)
    c = fx["config"]
    L = ib.lib()
    L.ibtfo_ref_configure(ib.SCHEMES[c["scheme"]], ib.RIEMANNS[c["riemann"]], ib.LIMITERS[c["limiter"]],
                          ib.BOUNDARIES[c["boundary"]], ib.GLOBAL_BCS[c["gbc"]], 0)
    nx, ny, ng, g = c["N_x"], c["N_y"], c["num_ghost_cell"], c["gamma"]
    M, N = nx + 2 * ng, ny + 2 * ng
    PL, PH = c["hi_x"] - c["lo_x"], c["hi_y"] - c["lo_y"]
    nsch = {"Regular": 1, "IDWBaseGFM": 8, "LinearBaseGFM": 4, "RiemannBaseGFM": 4}.get(c["boundary"], 16)
    XY = np.zeros(M * N * 6)
    SCH = np.zeros(M * N * nsch)
    U_OLD = np.zeros(M * N * 4)
    U_NEW = np.zeros(M * N * 4)
    U_TMP = np.zeros(1)
    dt_buf, m_buf = np.zeros(1), np.zeros(1)
    L.ibtfo_ref_Psy_coord(c["lo_x"], c["lo_y"], PL, PH, nx, ny, ng, _p(XY), 1, 0)
    XY.reshape(-1, 6)[:, 2] = fx["phi"]  # the case's Level_Set_function
    L.ibtfo_ref_Level_Set(nx, ny, ng, _p(XY), 1, 0)
    assert L.ibtfo_ref_status() == 0, L.ibtfo_last_error()
    if c["boundary"] != "Regular":
        L.ibtfo_ref_Scheme_Index(nx, ny, ng, _p(XY), _p(SCH), 1, 0)
        assert np.array_equal(SCH, fx["scheme_idx"])
    if "xycoord" in fx:
        assert np.array_equal(XY, fx["xycoord"])
    U_OLD[:] = fx["u_init"]  # the case's Initialize
    U_NEW[:] = fx["u_init"]
    L.ibtfo_ref_Boundary(nx, ny, ng, g, _p(U_OLD), _p(U_NEW), _p(XY), _p(SCH), 1, 0)
    L.ibtfo_ref_ComputeDt(PL, PH, nx, ny, ng, g, c["CFL_number"], _p(U_OLD), _p(XY), _p(dt_buf), 1, 0)
    L.ibtfo_ref_CaculateMass(PL, PH, nx, ny, ng, _p(U_OLD), _p(XY), _p(m_buf), 1, 0)
    assert L.ibtfo_ref_status() == 0, L.ibtfo_last_error()
    dt = dt_buf[0]
    assert np.isclose(dt, fx["dts"][0], rtol=RTOL, atol=0)
    L.ibtfo_ref_WriteData(c["lo_x"], c["lo_y"], PL, PH, nx, ny, ng, 0, 0.0, g, _p(U_OLD), _p(XY), 1, 0)
    assert L.ibtfo_ref_status() == 0, L.ibtfo_last_error()
    now_t, it, dts, ms = 0.0, 0, [], []
    while now_t < c["Psy_time"] and it < fx["iters"]:
        L.ibtfo_ref_TimeAdvance(PL, PH, nx, ny, ng, g, dt, _p(U_OLD), _p(U_TMP), _p(U_NEW), _p(XY), _p(SCH), 1, 0)
        L.ibtfo_ref_Boundary(nx, ny, ng, g, _p(U_OLD), _p(U_NEW), _p(XY), _p(SCH), 1, 0)
        L.ibtfo_ref_Global_Boundary(nx, ny, ng, g, _p(U_OLD), _p(U_NEW), 1, 0)
        L.ibtfo_ref_ComputeDt(PL, PH, nx, ny, ng, g, c["CFL_number"], _p(U_OLD), _p(XY), _p(dt_buf), 1, 0)
        L.ibtfo_ref_CaculateMass(PL, PH, nx, ny, ng, _p(U_OLD), _p(XY), _p(m_buf), 1, 0)
        assert L.ibtfo_ref_status() == 0, L.ibtfo_last_error()
        dt = dt_buf[0]
        now_t += dt
        it += 1
        dts.append(dt)
        ms.append(m_buf[0])
    assert it == fx["iters"]
    assert np.allclose(dts, fx["dts"][1:], rtol=RTOL, atol=0)
    assert np.allclose(ms, fx["masses"][1:], rtol=RTOL, atol=0)
    L.ibtfo_ref_update_self(_p(U_OLD))
    L.ibtfo_ref_update_self(_p(U_NEW))
    assert L.ibtfo_ref_status() == 0, L.ibtfo_last_error()
    assert np.array_equal(np.isfinite(U_OLD), np.isfinite(fx["u_old"]))
    assert rel_linf(U_OLD, fx["u_old"]) <= RTOL
    assert rel_linf(U_NEW, fx["u_new"]) <= RTOL
    L.ibtfo_ref_WriteData(c["lo_x"], c["lo_y"], PL, PH, nx, ny, ng, it, now_t, g, _p(U_OLD), _p(XY), 1, 0)
    assert L.ibtfo_ref_status() == 0, L.ibtfo_last_error()
    assert (tmp_path / "result.visit").read_text().split() == ["!NBLOCKS", "1", "dat_0_0.vtk", f"dat_0_{it}.vtk"]
    lines = (tmp_path / f"dat_0_{it}.vtk").read_text().split("\n")
    assert abs(float(lines[10].split()[0]) - now_t) < 1e-6
    k = lines.index("SCALARS density float  ") + 2
    rho = np.array([float(x) for x in lines[k:k + nx * ny]])
    u = U_OLD.reshape(N, M, 4)[ng:-ng, ng:-ng]
    t = XY.reshape(N, M, 6)[ng:-ng, ng:-ng, 5]
    want = np.where((t == 0) | (t == 3), np.maximum(u[..., 0], 1e-6), -1.0).reshape(-1)
    fin = np.isfinite(want)
    assert np.all(np.abs(rho[fin] - want[fin]) <= 5.1e-7 + 2e-7 * np.abs(want[fin]))
    L.ibtfo_ref_release(_p(XY))


def test_shim_rejects_several_devices():
    L = ib.lib()
    XY = np.zeros(12 * 12 * 6)
    L.ibtfo_ref_Psy_coord(0.0, 0.0, 1.0, 1.0, 8, 8, 2, _p(XY), 2, 0)
    assert L.ibtfo_ref_status() == 1  # IBTFO_EINVAL


def test_ibtfo_run_executable(tmp_path):
    """The C++ driver on a channel .inp against the oracle on the same plug-in inputs."""
    exe = os.path.join(os.path.dirname(ib.LIB_PATH), "ibtfo_run")
    assert os.path.exists(exe), "ibtfo_run is built with the library"
    inp = tmp_path / "channel.inp"
    inp.write_text("#channel\nN_x=128\nN_y=64\nlo_x=0\nlo_y=0\nhi_x=2\nhi_y=1\nCFL_number=0.45\n"
                   "Psy_time=0.2\nnum_ghost_cell=2\ngamma=1.4\nangle=30\nwidth=0.25\n"
                   "Scheme = MUSCL\nRiemann = HLLC\nLimiter = minmod\nBoundary = IDWBaseGFM\nCase = channel\n")
    out = tmp_path / "u.bin"
    p = subprocess.run([exe, str(inp), "--steps", "15", "--print-every", "5", "--out", str(out)],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("iter : ")]
    assert len(lines) == 3 and lines[-1].startswith("iter : 15.   dt :")
    u = np.fromfile(out, dtype=np.float64)

    cfg = ib.Inp(path=str(inp)).config()
    inpo = ib.Inp(path=str(inp))
    phi = ib.case_phi("channel", cfg, inpo)
    o = oracle.OracleCase(128, 64, 2, (0.0, 0.0), (2.0, 1.0), 1.4, 0.45, "MUSCL", "HLLC", "minmod", "IDWBaseGFM")
    o.setup_geometry(phi)
    o.set_initial_state(ib.case_init("channel", cfg, o.get("XYCOORD"), inpo))
    o.run(15)
    assert rel_linf(u, o.get("U_OLD")) <= RTOL


def test_ibtfo_run_vtk_series_and_restart(tmp_path):
    """--vtk writes dat_0_<iter>.vtk and result.visit at the reference
    drivers' points (every plot_per iterations, then once after the loop);
    --checkpoint then --restart continues as one uninterrupted run."""
    exe = os.path.join(os.path.dirname(ib.LIB_PATH), "ibtfo_run")
    inp = tmp_path / "channel.inp"
    inp.write_text("#channel\nN_x=96\nN_y=48\nlo_x=0\nlo_y=0\nhi_x=2\nhi_y=1\nCFL_number=0.45\n"
                   "Psy_time=0.2\nnum_ghost_cell=2\ngamma=1.4\nangle=30\nwidth=0.25\n"
                   "Scheme = MUSCL\nRiemann = HLLC\nLimiter = minmod\nBoundary = IDWBaseGFM\nCase = channel\n")

    def run(*args, cwd):
        cwd.mkdir(exist_ok=True)
        p = subprocess.run([exe, str(inp), *args], capture_output=True, text=True, timeout=300, cwd=cwd)
        assert p.returncode == 0, p.stderr
        return p.stdout

    one = tmp_path / "one"
    run("--steps", "20", "--print-every", "20", "--vtk-every", "8", "--out", str(one / "u.bin"), cwd=one)
    assert (one / "result.visit").read_text().split() == ["!NBLOCKS", "1", "dat_0_0.vtk", "dat_0_8.vtk",
                                                          "dat_0_16.vtk", "dat_0_20.vtk"]
    for k in (0, 8, 16, 20):
        assert (one / f"dat_0_{k}.vtk").read_text().startswith("# vtk DataFile Version 2.0")
    two = tmp_path / "two"
    run("--steps", "9", "--checkpoint", str(two / "c.ckpt"), cwd=two)
    run("--steps", "20", "--restart", str(two / "c.ckpt"), "--out", str(two / "u.bin"), cwd=two)
    assert np.array_equal(np.fromfile(one / "u.bin"), np.fromfile(two / "u.bin"))


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_pinned_buffers_move_the_same_bytes_as_pageable_ones(precision):
    """Transfers from and to page-locked host buffers (the e2e benchmark's)
    give the same bytes and the same loop state as from numpy arrays."""
    from ibtfo_gb300 import cases as _c
    w = _c.inclined_channel(128, 64)
    g = w.grid
    phi = _c.channel_phi(g)
    n = g.M * g.N * 4
    outs = []
    for pinned in (False, True):
        with ib.Case.from_workload(w, precision=precision) as c:
            c.setup_geometry(phi)
            u0 = _c.channel_init(g, c.cell_types(), w.gamma)
            if pinned:
                pin = ib.PinnedBuffer(n)
                pin.array[:] = u0
                c.set_state_ptr(pin.ptr)
            else:
                c.set_state(u0)
            c.advance(5)
            if pinned:
                c.get_state_ptr(pin.ptr)
                u = pin.array.copy()
                c.put_state_ptr(pin.ptr)       # round trip through the device
                c.advance(3)
                c.get_state_ptr(pin.ptr)
                u2 = pin.array.copy()
                pin.close()
            else:
                u = c.get_state()
                c.put_state(u)
                c.advance(3)
                u2 = c.get_state()
            outs.append((u, u2, c.progress()))
    assert np.array_equal(outs[0][0], outs[1][0], equal_nan=True)
    assert np.array_equal(outs[0][1], outs[1][1], equal_nan=True)
    assert outs[0][2] == outs[1][2]


@pytest.mark.parametrize("kind,precision", [("channel", "fp64_fast"), ("channel", "fp64"), ("channel", "fp32c"),
                                            ("channel_rk2", "fp64_fast"), ("channel_pvrs", "fp64"), ("ccm", "fp32c"),
                                            ("sod", "fp64")])
@pytest.mark.parametrize("in_place,pinned", [(True, True), (False, True), (True, False)])
def test_step_host_equals_put_step_get(kind, precision, in_place, pinned):
    """ibtfo_step_host (row-chunked copies overlapped with the banded sweep,
    replayed as a CUDA graph for page-locked arrays) leaves the same state,
    output bytes and loop scalars (the mass to its summation order) as
    ibtfo_put_state + ibtfo_step + ibtfo_get_state, step after step."""
    from ibtfo_gb300 import cases as _c
    if kind.startswith("channel"):
        w = _c.inclined_channel(512, 256)
        g = w.grid
        phi = _c.channel_phi(g)
        kw = dict(precision=precision, time="RK2" if kind.endswith("rk2") else "SingleStep")
        if kind.endswith("pvrs"):
            kw["riemann"] = "PVRS"

        def make():
            c = ib.Case.from_workload(w, **kw)
            c.setup_geometry(phi)
            c.set_state(_c.channel_init(g, c.cell_types(), w.gamma))
            return c
    elif kind == "ccm":
        g = _c.Grid(192, 128, 2, 0.0, 0.0, 1.5, 1.0)

        def make():
            c = ib.Case(g.n_x, g.n_y, lo=(0, 0), hi=(1.5, 1.0), cfl=0.3, riemann="HLL_Toro", boundary="CCM",
                        precision=precision)
            c.setup_geometry(_c.cylinder_phi(g, 0.6, 0.5, 0.2))
            c.set_state(_c.shock_init(g, c.cell_types(), 2.0, 0.2))
            return c
    else:
        g = _c.Grid(200, 40, 2, 0.0, 0.0, 1.0, 0.2)
        phi, u0 = _c.sod_x(g)

        def make():
            c = ib.Case(g.n_x, g.n_y, lo=(0, 0), hi=(1.0, 0.2), cfl=0.5, precision=precision)
            c.setup_geometry(phi)
            c.set_state(u0)
            return c
    n = (g.n_x + 2 * g.ng) * (g.n_y + 2 * g.ng) * 4
    ref, got = [], []
    with make() as a:
        u = a.get_state()
        for _ in range(4):
            a.put_state_ptr(u.ctypes.data)
            a.step()
            u = a.get_state()
            ref.append((u.copy(), a.progress()))
    with make() as b:
        if pinned:
            pin_in = ib.PinnedBuffer(n)
            pin_out = pin_in if in_place else ib.PinnedBuffer(n)
            a_in, a_out, p_in, p_out = pin_in.array, pin_out.array, pin_in.ptr, pin_out.ptr
        else:
            a_in = a_out = np.zeros(n)
            p_in = p_out = a_in.ctypes.data
        b.get_state_ptr(p_in)
        for k in range(4):
            p = b.step_host_ptr(p_in, p_out)
            got.append((a_out.copy(), p))
            if not in_place:
                a_in[:] = a_out
        assert np.array_equal(b.get_state(), got[-1][0], equal_nan=True)
    for (ur, pr), (ug, pg) in zip(ref, got):
        assert np.array_equal(ur, ug, equal_nan=True)
        same_progress(pr, pg)


def test_step_host_in_place_copies_in_only_what_the_step_reads():
    """In place, the calls after the first copy in only the cells a step
    reads (the fluid cells and two cells around them, the ghost cells, the
    domain edge).  A value the caller writes into a solid cell away from the
    fluid stays in the array and changes nothing else: the array after three
    more steps equals put + step + get of the modified array."""
    from ibtfo_gb300 import cases as _c
    w = _c.inclined_channel(512, 256)
    g = w.grid
    phi = _c.channel_phi(g)

    def make():
        c = ib.Case.from_workload(w, precision="fp64_fast")
        c.setup_geometry(phi)
        c.set_state(_c.channel_init(g, c.cell_types(), w.gamma))
        return c

    n = g.M * g.N * 4
    pin = ib.PinnedBuffer(n)
    try:
        with make() as b:
            full_in, _ = b.step_host_bytes(in_place=False)
            box_in, _ = b.step_host_bytes(in_place=True)
            assert box_in < 0.6 * full_in, (box_in, full_in)
            types = b.cell_types().reshape(g.N, g.M)
            j, i = g.N // 2, 2 * g.ng + 1  # solid, far from the channel and from the domain edge
            assert (types[j, g.ng: i + 40] == 1).all()
            b.get_state_ptr(pin.ptr)
            b.step_host_ptr(pin.ptr, pin.ptr)  # first call on the array: every row in
            b.step_host_ptr(pin.ptr, pin.ptr)
            u = pin.array.reshape(g.N, g.M, 4)
            u[j, i] = (7.0, 0.5, -0.25, 30.0)
            start = pin.array.copy()
            for _ in range(3):
                p = b.step_host_ptr(pin.ptr, pin.ptr)
            got = pin.array.copy()
        with make() as a:
            ua = a.get_state()
            for k in range(5):
                if k == 2:
                    assert np.array_equal(np.delete(ua.reshape(-1, 4), j * g.M + i, axis=0),
                                          np.delete(start.reshape(-1, 4), j * g.M + i, axis=0))
                    ua = start  # the same state with the modified solid cell
                a.put_state_ptr(ua.ctypes.data)
                a.step()
                ua = a.get_state()
            pa = a.progress()
        assert np.array_equal(got, ua, equal_nan=True)
        assert tuple(got.reshape(g.N, g.M, 4)[j, i]) == (7.0, 0.5, -0.25, 30.0)
        same_progress(p, pa)
    finally:
        pin.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_put_state_solid_cells_stay_through_steps(precision):
    """A step copies U_NEW into U_OLD for fluid cells only
    (IDWBaseGFM/GFM_Bound.cpp:24-35): a solid cell written by ibtfo_put_state
    keeps its value through the following steps."""
    from ibtfo_gb300 import cases as _c
    w = _c.inclined_channel(256, 128)
    g = w.grid
    with ib.Case.from_workload(w, precision=precision) as c:
        c.setup_geometry(_c.channel_phi(g))
        c.set_state(_c.channel_init(g, c.cell_types(), w.gamma))
        c.advance(3)
        u = c.get_state().reshape(g.N, g.M, 4)
        j, i = g.N // 2, 2 * g.ng + 1
        assert c.cell_types().reshape(g.N, g.M)[j, i] == 1
        u[j, i] = (7.0, 0.5, -0.25, 30.0)
        c.put_state(u.reshape(-1))
        for _ in range(3):
            c.advance(1)
            assert tuple(c.get_state().reshape(g.N, g.M, 4)[j, i]) == (7.0, 0.5, -0.25, 30.0)
