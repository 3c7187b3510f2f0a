"""The allocation-free dt/mass entry point against the library's own.

ibtfo_dt_mass_noalloc is for callers that cannot call cudaMalloc (a
framework that owns all device memory through its own pool, or code that
must not let an allocation synchronise the device): it takes a state the
caller already holds on the GPU and works in a fixed scratch array inside
the library.  Here it is called through the C ABI on two states in a row --
the initial state of a ghost-fluid case and the same case five steps later
-- and each result is checked against the dt and mass that the regular
path (ibtfo_set_state / ibtfo_advance, whose reduction scratch is allocated
with the case) reports for the same state.

This file is collected last on purpose and runs alone as well as after the
other tests.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import ibtfo_gb300 as ib  # noqa: E402
from ibtfo_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # the tolerance of the other parity tests


def device_planes(case, u_aos, types, pitch):
    """state as four pitched planes and the type plane, on the GPU"""
    M, N = case.M, case.N
    planes = np.zeros((4, N, pitch))
    planes[:, :, :M] = np.moveaxis(u_aos.reshape(N, M, 4), 2, 0)
    t = np.full((N, pitch), 2, dtype=np.uint8)
    t[:, :M] = types.reshape(N, M).astype(np.uint8)
    return torch.from_numpy(planes).cuda(), torch.from_numpy(t).cuda()


def call_noalloc(w, case, du, dtype_, out, pitch):
    g = w.grid
    stream = torch.cuda.current_stream().cuda_stream
    rc = ib.lib().ibtfo_dt_mass_noalloc(du.data_ptr(), case.N * pitch, pitch, dtype_.data_ptr(), g.n_x, g.n_y,
                                        g.ng, g.lo_x, g.lo_y, g.hi_x, g.hi_y, w.gamma, w.cfl, out.data_ptr(),
                                        stream)
    assert rc == 0, ib.lib().ibtfo_last_error().decode()
    torch.cuda.synchronize()
    return out.cpu().numpy().copy()


def test_noalloc_dt_mass_matches_library_on_two_calls():
    torch.cuda.init()
    w = cases.inclined_channel(320, 160)
    g = w.grid
    with ib.Case.from_workload(w) as c:
        c.setup_geometry(cases.channel_phi(g))
        types = c.cell_types()
        c.set_state(cases.channel_init(g, types, w.gamma))
        pitch = (c.M + 7) // 8 * 8  # any pitch >= M works
        out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")

        # call 1: the initial state
        p0 = c.progress()
        du, dt_ = device_planes(c, c.get_state(), types, pitch)
        r0 = call_noalloc(w, c, du, dt_, out, pitch)
        np.testing.assert_allclose(r0, [p0["dt"], p0["mass"]], rtol=RTOL, atol=0)

        # call 2: a different state (five steps later) through the same scratch
        c.advance(5)
        p1 = c.progress()
        assert p1["iter"] == 5
        du, dt_ = device_planes(c, c.get_state(), types, pitch)
        out.fill_(float("nan"))
        r1 = call_noalloc(w, c, du, dt_, out, pitch)
        np.testing.assert_allclose(r1, [p1["dt"], p1["mass"]], rtol=RTOL, atol=0)
        assert r1[0] != r0[0]


def test_noalloc_rejects_oversized_grid():
    L = ib.lib()
    # 8192 x 4096 interior cells need 131072 tiles; the fixed scratch holds 65536
    rc = L.ibtfo_dt_mass_noalloc(1, 8196 * 4100, 8196, 1, 8192, 4096, 2, 0.0, 0.0, 4.0, 2.0, 1.4, 0.5, 1, None)
    assert rc == 1  # IBTFO_EINVAL, before any device work
    assert "too large" in L.ibtfo_last_error().decode()
