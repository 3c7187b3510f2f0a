"""VTK output and checkpoints (GPU).

* VTK: the header and the four fields of the reference's WriteData layout
  (Src/Utils/WriteData.cpp:30-120), ASCII values equal to the state's to the
  6 decimals of "%f", binary values equal to its float32 values; non-fluid
  cells carry the reference's markers.
* Checkpoints: a run saved after n steps and restored into a fresh case
  continues bit for bit as the uninterrupted run (state, dt, loop time, step
  count, mass) -- Regular boundaries, ghost-fluid walls and cut cells, FP64 and
  the FP32 form (whose checkpoint keeps the (hi, lo) pairs as they are); a
  checkpoint of another configuration is refused."""
import numpy as np
import pytest

ib = pytest.importorskip("ibtfo_gb300")
from ibtfo_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu


def channel_case(precision="fp64"):
    w = cases.inclined_channel(96, 48)
    c = ib.Case.from_workload(w, precision=precision, t_end=1e300, max_iter=2 ** 31 - 1)
    c.setup_geometry(cases.channel_phi(w.grid))
    c.set_state(cases.channel_init(w.grid, c.cell_types(), w.gamma))
    return w, c


def expected_fields(w, c):
    g = w.grid
    u = c.get_state().reshape(g.N, g.M, 4)[g.ng:-g.ng, g.ng:-g.ng]
    t = c.cell_types().reshape(g.N, g.M)[g.ng:-g.ng, g.ng:-g.ng]
    fl = (t == 0) | (t == 3)
    rho = u[..., 0]
    with np.errstate(all="ignore"):
        vx, vy = u[..., 1] / rho, u[..., 2] / rho
        p = (w.gamma - 1) * (u[..., 3] - 0.5 * rho * (vx * vx + vy * vy))
    return [np.where(fl, np.maximum(rho, 1e-6), -1.0), np.where(fl, vx, -100.0), np.where(fl, vy, -100.0),
            np.where(fl, p, -100.0)]


def test_vtk_ascii_and_binary(tmp_path):
    w, c = channel_case()
    with c:
        c.advance(12)
        exp = [f.reshape(-1) for f in expected_fields(w, c)]
        now_t = c.progress()["now_t"]
        pa, pb = tmp_path / "a.vtk", tmp_path / "b.vtk"
        c.write_vtk(str(pa))
        c.write_vtk(str(pb), binary=True)
    lines = pa.read_text().split("\n")
    assert lines[0].startswith("# vtk DataFile Version 2.0") and lines[2].strip() == "ASCII"
    assert lines[4].split()[1:3] == [str(w.grid.n_x), str(w.grid.n_y)]
    assert abs(float(lines[10].split()[0]) - now_t) < 1e-6
    n = w.grid.n_x * w.grid.n_y
    names, vals, k = [], [], 0
    while k < len(lines):
        if lines[k].startswith("SCALARS"):
            names.append(lines[k].split()[1])
            vals.append(np.array([float(x) for x in lines[k + 2:k + 2 + n]]))
            k += 2 + n
        else:
            k += 1
    assert names == ["density", "x-vel", "y-vel", "pressure"]
    for v, e in zip(vals, exp):
        # "%f" of the float32 value: 5e-7 absolute plus float32 rounding
        assert np.all(np.abs(v - e) <= 5.1e-7 + 2e-7 * np.abs(e))
    raw = pb.read_bytes()
    for name, e in zip(names, exp):
        start = raw.index(f"SCALARS {name} float  \nLOOKUP_TABLE default  \n".encode())
        start += len(f"SCALARS {name} float  \nLOOKUP_TABLE default  \n")
        v = np.frombuffer(raw[start:start + 4 * n], dtype=">f4")
        assert np.array_equal(v, e.astype(np.float32))


def test_vtk_written_off_the_step_path_matches_the_synchronous_file(tmp_path):
    """The asynchronous writer snapshots the state in order with the steps:
    files queued between advances equal the synchronous files of the same
    states, and the stepping itself is unchanged."""
    w, c = channel_case()
    with c:
        for k in range(3):
            c.advance(5)
            c.write_vtk(str(tmp_path / f"s{k}.vtk"), binary=True)
        ref = c.get_state()
    w, c = channel_case()
    with c:
        for k in range(3):
            c.advance(5)
            c.write_vtk(str(tmp_path / f"a{k}.vtk"), binary=True, wait=False)
        c.output_wait()
        assert np.array_equal(c.get_state(), ref)
        c.write_vtk(str(tmp_path / "missing" / "x.vtk"), wait=False)
        with pytest.raises(ib.IbtfoError, match="cannot write"):
            c.output_wait()
        c.output_wait()  # the failure is reported once
    for k in range(3):
        assert (tmp_path / f"a{k}.vtk").read_bytes() == (tmp_path / f"s{k}.vtk").read_bytes()


def _sod(precision):
    g = cases.Grid(120, 30, 2, 0.0, 0.0, 1.0, 0.25)
    w = cases.Workload("sod", g, 1.4, 0.5, 1e300, "MUSCL", "HLLC", "minmod", "Regular")
    phi, u0 = cases.sod_x(g)
    c = ib.Case.from_workload(w, precision=precision, max_iter=2 ** 31 - 1)
    c.setup_geometry(phi)
    c.set_state(u0)
    return w, c, phi


def _ccm(precision):
    g = cases.Grid(96, 64, 2, 0.0, 0.0, 1.5, 1.0)
    w = cases.Workload("ccm", g, 1.4, 0.3, 1e300, "MUSCL", "HLL_Toro", "minmod", "CCM")
    phi = cases.cylinder_phi(g, 0.6, 0.5, 0.2)
    c = ib.Case.from_workload(w, precision=precision, max_iter=2 ** 31 - 1)
    c.setup_geometry(phi)
    c.set_state(cases.shock_init(g, c.cell_types(), 2.0, 0.2))
    return w, c, phi


@pytest.mark.parametrize("kind,precision", [("sod", "fp64"), ("sod", "fp32c"), ("channel", "fp32c"),
                                            ("ccm", "fp32c"), ("ccm", "fp64_fast")])
def test_checkpoint_restart_is_bit_for_bit(tmp_path, kind, precision):
    if kind == "sod":
        w, c, phi = _sod(precision)
    elif kind == "channel":
        w, c = channel_case(precision)
        phi = cases.channel_phi(w.grid)
    else:
        w, c, phi = _ccm(precision)
    path = str(tmp_path / "run.ckpt")
    with c:
        c.advance(10)
        c.save_checkpoint(path)
        c.advance(7)
        ref_u, ref_p = c.get_state(), c.progress()
    d = ib.Case.from_workload(w, precision=precision, max_iter=2 ** 31 - 1, t_end=1e300)
    with d:
        d.setup_geometry(phi)
        d.load_checkpoint(path)
        assert d.progress()["iter"] == 10
        d.advance(7)
        assert np.array_equal(d.get_state(), ref_u, equal_nan=True)
        p = d.progress()
        for k in ("iter", "now_t", "dt", "mass", "mass_start", "nan_cells", "status"):
            assert p[k] == ref_p[k], k
    # another configuration is refused
    other = ib.Case(w.grid.n_x + 2, w.grid.n_y, precision=precision)
    with other:
        other.setup_geometry(np.ones(other.M * other.N))
        with pytest.raises(ib.IbtfoError, match="configuration"):
            other.load_checkpoint(path)
