"""Writes the golden fixtures in tests/golden/ by running the reference's own
solver (oracle/_ref/, built from the reference sources by oracle/build_ref.py).

Each fixture is one .npz: the case configuration (JSON), the inputs (level set
`phi` and initial state `u_init`, as the reference driver saw them) and the
reference's outputs after `iters` time steps: U_OLD, U_NEW, the dt and mass
sequences, now_t, and for ghost-fluid variants the geometry (XYCOORD) and the
per-cell boundary data (SCHEME_IDX).

Run in a container that has the reference sources:
    python oracle/build_ref.py && python tests/golden/gen_golden.py [fixture ...]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from ibtfo_gb300 import cases  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def inp_text(cfg: dict) -> str:
    keys = ["max_iter", "N_x", "N_y", "Psy_time", "lo_x", "lo_y", "hi_x", "hi_y", "CFL_number",
            "num_ghost_cell", "gamma"]
    lines = ["#do not add space in params!!!"]
    for k in keys:
        lines.append(f"{k}={cfg[k]!r}")
    for k, v in cfg.get("plugin_params", {}).items():
        lines.append(f"{k}={v!r}")
    return "\n".join(lines) + "\n"


def types_for(cfg, phi):
    """cell types from the oracle's Level_Set (used only to shape the IC)."""
    c = oracle.OracleCase(cfg["N_x"], cfg["N_y"], cfg["num_ghost_cell"], (cfg["lo_x"], cfg["lo_y"]),
                          (cfg["hi_x"], cfg["hi_y"]), cfg["gamma"], cfg["CFL_number"], cfg["scheme"],
                          cfg["riemann"], cfg["limiter"], cfg["boundary"], cfg["gbc"])
    c.setup_geometry(phi)
    return c.get("XYCOORD").reshape(-1, 6)[:, 5]


def make_inputs(cfg):
    g = cases.Grid(cfg["N_x"], cfg["N_y"], cfg["num_ghost_cell"], cfg["lo_x"], cfg["lo_y"], cfg["hi_x"], cfg["hi_y"])
    kind = cfg["case"]
    if kind == "sod_x":
        return cases.sod_x(g, cfg["gamma"])
    if kind == "quadrants":
        return cases.quadrants(g, cfg["gamma"], downward=cfg.get("downward", False))
    if kind == "channel":
        phi = cases.channel_phi(g, cfg.get("angle", 30.0), cfg.get("width", 0.25))
        return phi, cases.channel_init(g, types_for(cfg, phi), cfg["gamma"], cfg.get("angle", 30.0))
    if kind == "vortex":
        return cases.isentropic_vortex(g, cfg["gamma"], beta=cfg.get("beta", 5.0))
    raise ValueError(kind)


def variant(cfg):
    return f"ref_{cfg['scheme']}_{cfg['riemann']}_{cfg['limiter']}_{cfg['boundary']}_{cfg['plugin']}"


def run_fixture(name, cfg, nsteps):
    exe = os.path.join(REF, variant(cfg))
    if not os.path.exists(exe):
        raise FileNotFoundError(exe + " (run oracle/build_ref.py first)")
    with tempfile.TemporaryDirectory() as td:
        inp = os.path.join(td, "case.inp")
        with open(inp, "w") as f:
            f.write(inp_text(cfg))
        out = os.path.join(td, "out.bin")
        args = [exe, inp, str(nsteps), out]
        if cfg["plugin"] in ("file", "fileper"):
            phi, u0 = make_inputs(cfg)
            pp, up = os.path.join(td, "phi.bin"), os.path.join(td, "u0.bin")
            phi.astype("<f8").tofile(pp)
            u0.astype("<f8").tofile(up)
            args += [pp, up]
        subprocess.run(args, check=True, capture_output=True)
        rec = oracle.read_ref_record(out)
    keep = {"config": np.frombuffer(json.dumps(cfg).encode(), dtype=np.uint8), "iters": rec["iters"],
            "now_t": rec["now_t"], "dts": rec["dts"], "masses": rec["masses"], "phi": rec["phi"],
            "u_init": rec["u_init"], "u_old": rec["u_old"], "u_new": rec["u_new"]}
    if cfg["boundary"] != "Regular" or cfg["plugin"].startswith("ref"):
        keep["xycoord"] = rec["xycoord"]
        keep["scheme_idx"] = rec["scheme_idx"]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **keep)
    return rec


def base(case, n_x, n_y, lo, hi, cfl, t_end, scheme="MUSCL", riemann="HLL", limiter="minmod",
         boundary="Regular", plugin="file", gbc="walls", **extra):
    cfg = {"case": case, "max_iter": 100000, "N_x": n_x, "N_y": n_y, "Psy_time": t_end, "lo_x": lo[0],
           "lo_y": lo[1], "hi_x": hi[0], "hi_y": hi[1], "CFL_number": cfl, "num_ghost_cell": 2, "gamma": 1.4,
           "scheme": scheme, "riemann": riemann, "limiter": limiter, "boundary": boundary, "plugin": plugin,
           "gbc": gbc}
    cfg.update(extra)
    return cfg


def fixtures():
    fx = []
    # every scheme x solver x limiter on a four-state problem (both vertical wave directions occur)
    for s in ("MUSCL", "MHM", "Godunov"):
        for r in ("HLL", "HLLC", "PVRS", "StegerWarming"):
            for lim in (("minmod", "VanLeer") if (s, r) == ("MUSCL", "HLL") else ("minmod",)):
                fx.append((f"quad_{s}_{r}_{lim}", base("quadrants", 32, 24, (0, 0), (1, 0.75), 0.3, 1.0, s, r, lim), 10))
    for s in ("MUSCL", "MHM"):
        for r in ("HLL", "PVRS", "StegerWarming"):
            fx.append((f"quaddown_{s}_{r}_minmod",
                       base("quadrants", 32, 24, (0, 0), (1, 0.75), 0.3, 1.0, s, r, "minmod", downward=True), 10))
    # the Sod tube workload shape at a reduced size, run to t_end
    fx.append(("sodtube_MUSCL_HLL_minmod", base("sod_x", 80, 20, (0, 0), (1, 0.25), 0.5, 0.2), 1000))
    fx.append(("sodtube_MHM_HLLC_minmod", base("sod_x", 80, 20, (0, 0), (1, 0.25), 0.5, 0.2, "MHM", "HLLC"), 1000))
    # inclined channel with every ghost-fluid variant
    for b in ("IDWBaseGFM", "LinearBaseGFM", "RiemannBaseGFM", "BCGFM", "HBCGFM"):
        fx.append((f"channel_MUSCL_HLLC_minmod_{b}",
                   base("channel", 64, 32, (0, 0), (2, 1), 0.45, 0.2, "MUSCL", "HLLC", "minmod", b), 10))
    fx.append(("channel_MHM_HLL_minmod_IDWBaseGFM",
               base("channel", 64, 32, (0, 0), (2, 1), 0.45, 0.2, "MHM", "HLL", "minmod", "IDWBaseGFM"), 10))
    fx.append(("channel_MUSCL_PVRS_minmod_BCGFM",
               base("channel", 64, 32, (0, 0), (2, 1), 0.45, 0.2, "MUSCL", "PVRS", "minmod", "BCGFM"), 10))
    fx.append(("channel_MUSCL_SW_minmod_IDWBaseGFM",
               base("channel", 64, 32, (0, 0), (2, 1), 0.45, 0.2, "MUSCL", "StegerWarming", "minmod", "IDWBaseGFM"), 10))
    # periodic isentropic vortex (harness plug-in boundary)
    fx.append(("vortex_MHM_HLLC_minmod_periodic",
               base("vortex", 32, 32, (0, 0), (10, 10), 0.5, 10.0, "MHM", "HLLC", "minmod", "Regular", "fileper",
                    "periodic", beta=5.0), 10))
    # the reference's own test plug-ins
    fx.append(("refsod_MUSCL_HLL_minmod", base("refsod", 48, 24, (0, 0), (1, 0.5), 0.3, 0.1, plugin="refsod",
                                              plugin_params={"rho_L": 1, "u_L": 0, "v_L": 0, "p_L": 1, "rho_R": 0.125,
                                                             "u_R": 0, "v_R": 0, "p_R": 0.1}), 10))
    for b in ("IDWBaseGFM", "LinearBaseGFM", "BCGFM", "HBCGFM"):
        fx.append((f"refincline_MUSCL_HLL_minmod_{b}",
                   base("refincline", 48, 48, (0, 0), (1, 1), 0.3, 0.3, "MUSCL", "HLL", "minmod", b, "refincline",
                        plugin_params={"angle": 30.0, "AxisD": 0.4, "rho_L": 1, "u_L": 0, "v_L": 0, "p_L": 1,
                                       "rho_R": 0.125, "u_R": 0, "v_R": 0, "p_R": 0.1}), 10))
    # VanLeer beyond MUSCL + HLL, and more scheme x solver x ghost-fluid pairings
    # (the reference's VanLeer macro turns these to NaN within a few steps: 2 and 3 steps keep most values finite)
    fx.append(("quad_MHM_HLL_VanLeer", base("quadrants", 32, 24, (0, 0), (1, 0.75), 0.3, 1.0, "MHM", "HLL", "VanLeer"), 2))
    fx.append(("channel_MUSCL_HLL_VanLeer_IDWBaseGFM",
               base("channel", 64, 32, (0, 0), (2, 1), 0.45, 0.2, "MUSCL", "HLL", "VanLeer", "IDWBaseGFM"), 3))
    fx.append(("channel_Godunov_SW_minmod_HBCGFM",
               base("channel", 64, 32, (0, 0), (2, 1), 0.45, 0.2, "Godunov", "StegerWarming", "minmod", "HBCGFM"), 10))
    fx.append(("channel_MHM_PVRS_minmod_LinearBaseGFM",
               base("channel", 64, 32, (0, 0), (2, 1), 0.3, 0.2, "MHM", "PVRS", "minmod", "LinearBaseGFM"), 10))
    # Scheme = Lax (Lax_Scheme.cpp): four-state problem, Sod tube to t_end, ghost-fluid channel
    fx.append(("quad_Lax", base("quadrants", 32, 24, (0, 0), (1, 0.75), 0.3, 1.0, "Lax"), 10))
    fx.append(("sodtube_Lax", base("sod_x", 80, 20, (0, 0), (1, 0.25), 0.5, 0.2, "Lax"), 1000))
    for b in ("IDWBaseGFM", "BCGFM"):
        fx.append((f"channel_Lax_{b}", base("channel", 64, 32, (0, 0), (2, 1), 0.45, 0.2, "Lax", "HLL", "minmod", b), 10))
    fx.append(("refvortex_MUSCL_HLL_minmod_IDWBaseGFM",
               base("refvortex", 48, 48, (0, 0), (1, 1), 0.3, 1.0, "MUSCL", "HLL", "minmod", "IDWBaseGFM", "refvortex",
                    plugin_params={"fa": 1.0, "fw": 0, "f0": 0, "f1": 1.0}), 10))
    return fx


def main(argv=None):
    """Writes every fixture, or those whose names are given."""
    names = set((argv if argv is not None else sys.argv[1:]))
    oracle.set_threads(1)
    for name, cfg, n in fixtures():
        if names and name not in names:
            continue
        rec = run_fixture(name, cfg, n)
        u = rec["u_old"]
        print(f"{name:48s} iters={rec['iters']:4d} now_t={rec['now_t']:.6g} nan={int(np.isnan(u).sum())}")


if __name__ == "__main__":
    main()
