"""Host-side C++ of the library on the CPU: the .inp reader (the reference's
ParamReader rules) and the case plug-ins (restated reference Test plug-ins
checked against what the reference's own plug-ins produced)."""
import numpy as np
import pytest

import oracle
import ibtfo_gb300 as ib
from golden_util import load
from ibtfo_gb300 import cases

INP = """#do not add space in params!!!
max_iter=1000
N_x=64                 # x direction grid number
N_y = 32
Psy_time=0.25
hi_x = 2.0
CFL_number=0.45   # CFL_number
tiny=1e-5
neg=-.5
noval=abc
  # not a comment: the first character is a space
Scheme = MHM #Lax or MUSCL or MHM
Riemann = StegerWarming
Boundary = BCGFM #Regular or BaseGFM
Precision = FP64_FAST
"""


def test_inp_numbers_follow_paramreader_rules():
    p = ib.Inp(text=INP)
    assert p.get("N_x") == (64.0, True)
    assert p.get("N_y") == (32.0, True)
    assert p.get("hi_x") == (2.0, True)
    assert p.get("tiny") == (1.0, True)  # first match of [+-]?(\d*\.\d+|\d+) is "1"
    assert p.get("neg") == (-0.5, True)
    assert p.get("noval") == (0.0, True)  # no number: atof("") = 0
    assert p.get("missing", 7.0) == (7.0, False)
    assert p.get("#notacomment:thefirstcharacterisaspace")[1]  # spaces removed, kept as a key
    assert p.get("#donotaddspaceinparams!!!")[1] is False  # '#' at column 0 is skipped


def test_config_from_inp():
    cfg = ib.Inp(text=INP).config()
    assert (cfg.n_x, cfg.n_y, cfg.max_iter) == (64, 32, 1000)
    assert (cfg.hi_x, cfg.hi_y, cfg.lo_x) == (2.0, 1.0, 0.0)  # defaults of Test/Sod/Sod.cpp:34-48
    assert cfg.cfl_number == 0.45 and cfg.gamma == 1.4 and cfg.num_ghost_cell == 2
    assert cfg.scheme == ib.SCHEMES["MHM"] and cfg.riemann == ib.RIEMANNS["StegerWarming"]
    assert cfg.boundary == ib.BOUNDARIES["BCGFM"] and cfg.precision == 1


def test_unknown_slot_value_rejected():
    with pytest.raises(ib.IbtfoError):
        ib.Inp(text="Boundary = OIDWBaseGFM\n").config()
    with pytest.raises(ib.IbtfoError):
        ib.Inp(text="Time = RK4\n").config()


def test_scheme_and_time_slots_of_the_makefile():
    # Test/Sod/Makefile:1,5: Scheme = Lax | MUSCL | MHM | Godunov, Time = SingleStep | RK2
    cfg = ib.Inp(text="Scheme = Lax\nTime = RK2\n").config()
    assert cfg.scheme == ib.SCHEMES["Lax"] and cfg.time_advance == ib.TIME_ADVANCES["RK2"]
    cfg = ib.Inp(text="Scheme = MUSCL\n").config()
    assert cfg.time_advance == ib.TIME_ADVANCES["SingleStep"]


def _cfg_of(fx):
    c = fx["config"]
    return ib.config(c["N_x"], c["N_y"], c["num_ghost_cell"], (c["lo_x"], c["lo_y"]), (c["hi_x"], c["hi_y"]),
                     c["gamma"], c["CFL_number"], c["Psy_time"], c["max_iter"])


@pytest.mark.parametrize("fixture,name", [("refsod_MUSCL_HLL_minmod", "sod_ref"),
                                          ("refincline_MUSCL_HLL_minmod_IDWBaseGFM", "incline_ref"),
                                          ("refvortex_MUSCL_HLL_minmod_IDWBaseGFM", "vortex_ref")])
def test_reference_plugins_restated_bit_for_bit(fixture, name):
    fx = load(fixture)
    text = "\n".join(f"{k}={v!r}" for k, v in fx["config"].get("plugin_params", {}).items())
    inp = ib.Inp(text=text)
    cfg = _cfg_of(fx)
    phi = ib.case_phi(name, cfg, inp)
    assert np.array_equal(phi, fx["phi"])
    u0 = ib.case_init(name, cfg, fx["xycoord"], inp)
    assert np.array_equal(u0, fx["u_init"], equal_nan=True)


def test_workload_plugins_match_python_cases():
    w = cases.inclined_channel(128, 64)
    g = w.grid
    cfg = ib.config(g.n_x, g.n_y, g.ng, (g.lo_x, g.lo_y), (g.hi_x, g.hi_y), w.gamma, w.cfl)
    phi = ib.case_phi("channel", cfg)
    assert np.allclose(phi, cases.channel_phi(g), rtol=0, atol=1e-15)
    o = oracle.OracleCase(g.n_x, g.n_y, g.ng, (g.lo_x, g.lo_y), (g.hi_x, g.hi_y), w.gamma, w.cfl, w.scheme, w.riemann,
                          w.limiter, w.boundary)
    o.setup_geometry(phi)
    xy = o.get("XYCOORD")
    assert np.array_equal(ib.case_init("channel", cfg, xy), cases.channel_init(g, xy.reshape(-1, 6)[:, 5], w.gamma))
    v = cases.vortex_periodic(64)
    gv = v.grid
    cfgv = ib.config(gv.n_x, gv.n_y, gv.ng, (gv.lo_x, gv.lo_y), (gv.hi_x, gv.hi_y), v.gamma, v.cfl)
    xyv = np.zeros((gv.M * gv.N, 6))
    X, Y = gv.coords()
    xyv[:, 0], xyv[:, 1] = X.reshape(-1), Y.reshape(-1)
    _, u_py = cases.isentropic_vortex(gv)
    assert np.allclose(ib.case_init("isentropic_vortex", cfgv, xyv), u_py, rtol=1e-13, atol=1e-14)
    with pytest.raises(ib.IbtfoError):
        ib.case_phi("nosuchcase", cfg)
