"""The FP32 compensated precision form against the FP64 path.

Bar (the served-form bar): L1 density error <= 1e-5 relative to the FP64
result on the same inputs after the same number of steps (the isentropic
vortex against its exact solution is in test_gpu_exact.py)."""
import numpy as np
import pytest

ib = pytest.importorskip("ibtfo_gb300")
from ibtfo_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu


def l1_rel(a, b, k=0):
    a = a.reshape(-1, 4)[:, k]
    b = b.reshape(-1, 4)[:, k]
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def interior(u, g):
    return u.reshape(g.N, g.M, 4)[g.ng:-g.ng, g.ng:-g.ng].reshape(-1)


def run(w, precision, steps, phi, u0=None, init=None):
    with ib.Case.from_workload(w, precision=precision, t_end=1e300, max_iter=2 ** 31 - 1) as c:
        c.setup_geometry(phi)
        if u0 is None:
            u0 = init(c.cell_types())
        c.set_state(u0)
        c.advance(steps)
        p = c.progress()
        return c.get_state(), p


@pytest.mark.parametrize("riemann", ["HLLC", "StegerWarming", "HLLC_Toro"])
def test_fp32c_inclined_channel(riemann):
    w = cases.inclined_channel(256, 128)
    w.riemann = riemann
    g = w.grid
    phi = cases.channel_phi(g)
    init = lambda types: cases.channel_init(g, types, w.gamma)  # noqa: E731
    u64, _ = run(w, "fp64_fast", 150, phi, init=init)
    u32, p32 = run(w, "fp32c", 150, phi, init=init)
    assert p32["nan_cells"] == 0
    types = _types(w, phi)
    fluid = (types == 0)
    a = u32.reshape(-1, 4)[fluid]
    b = u64.reshape(-1, 4)[fluid]
    err = float(np.abs(a[:, 0] - b[:, 0]).sum() / np.abs(b[:, 0]).sum())
    assert err <= 1e-5, err


def _types(w, phi):
    with ib.Case.from_workload(w) as c:
        c.setup_geometry(phi)
        return c.cell_types()


def test_fp32c_rejects_pvrs():
    with pytest.raises(ib.IbtfoError) as e:
        ib.Case(32, 32, riemann="PVRS", precision="fp32c")
    assert e.value.code == 1
