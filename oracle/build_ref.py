"""Build recipe for oracle/_ref/: the reference's own solver, compiled unmodified.

Test infrastructure.  Each variant is one executable that links the reference's
Src/ files for one slot choice (Scheme / Riemann / Limiter / Boundary, selected
exactly as the reference Makefiles do: by source directory plus `-I` order,
Test/Sod/Makefile:1-7,21-37) with the harness driver in oracle/harness/.
Pragmas are ignored by g++, which turns every OpenACC loop into a serial loop;
`-ffp-contract=off` keeps the arithmetic free of fused multiply-adds so the
results are the plain IEEE binary64 evaluation of the reference expressions.

Only this container has the reference sources; the products are host binaries
used to pin the C restatement in oracle/ and to write tests/golden/ fixtures.

    python oracle/build_ref.py [--ref DIR] [--jobs N] [variant ...]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

SCHEMES = ("MUSCL", "MHM", "Godunov")  # and Lax, below
RIEMANNS = ("HLL", "HLLC", "PVRS", "StegerWarming")
LIMITERS = ("minmod", "VanLeer")
BOUNDARIES = ("Regular", "IDWBaseGFM", "LinearBaseGFM", "RiemannBaseGFM", "BCGFM", "HBCGFM")
# plug-in sets: (Initialize + Level_Set_function sources, Global_Boundary source)
PLUGINS = {
    "file": (["harness/plugin_file.cpp"], "Test/Sod/Global_Boudary.cpp"),
    "fileper": (["harness/plugin_file.cpp"], "harness/gb_periodic.cpp"),
    "refsod": (["Test/Sod/Initialize.cpp", "Test/Sod/Level_Set_function.cpp"], "Test/Sod/Global_Boudary.cpp"),
    "refincline": (["Test/InclineSod/Initialize.cpp", "Test/InclineSod/Level_Set_function.cpp"],
                   "Test/InclineSod/Global_Boudary.cpp"),
    "refvortex": (["Test/Vortex/Initialize.cpp", "Test/Vortex/Level_Set_function.cpp"],
                  "Test/Vortex/Global_Boudary.cpp"),
}


def variant_name(scheme, riemann, limiter, boundary, plugin):
    return f"ref_{scheme}_{riemann}_{limiter}_{boundary}_{plugin}"


def default_variants():
    v = []
    for s in SCHEMES:
        for r in RIEMANNS:
            for lim in (LIMITERS if s != "Godunov" else ("minmod",)):
                for b in BOUNDARIES:
                    v.append((s, r, lim, b, "file"))
    v += [("MHM", "HLL", "minmod", "Regular", "fileper"), ("MUSCL", "HLL", "minmod", "Regular", "fileper"),
          ("MHM", "HLLC", "minmod", "Regular", "fileper")]
    v += [("MUSCL", "HLL", "minmod", "Regular", "refsod")]
    v += [("MUSCL", "HLL", "minmod", b, "refincline") for b in ("IDWBaseGFM", "LinearBaseGFM", "BCGFM", "HBCGFM")]
    v += [("MUSCL", "HLL", "minmod", "IDWBaseGFM", "refvortex")]
    # Scheme = Lax takes no Riemann solver or limiter; the Makefile still links one of each
    v += [("Lax", "HLL", "minmod", b, "file") for b in BOUNDARIES]
    return v


def build_one(ref, spec, force=False):
    scheme, riemann, limiter, boundary, plugin = spec
    name = variant_name(*spec)
    exe = os.path.join(OUT, name)
    if os.path.exists(exe) and not force:
        return name, True, "cached"
    src = os.path.join(ref, "Src")
    adv = os.path.join(src, "Base", "Euler", "Advection")
    rie = os.path.join(src, "Base", "Euler", "Riemann")
    bnd = os.path.join(src, "BoundaryCondition")

    def cpps(d):
        return sorted(os.path.join(d, f) for f in os.listdir(d) if f.endswith(".cpp"))

    files = cpps(os.path.join(src, "Geometry"))
    files += [os.path.join(src, "Utils", "ParamReader.cpp"), os.path.join(src, "Utils", "CaculateMass.cpp")]
    files += cpps(os.path.join(bnd, boundary)) + cpps(os.path.join(adv, scheme)) + cpps(os.path.join(src, "Base", "Common"))
    files += cpps(os.path.join(rie, riemann)) + cpps(os.path.join(src, "Base", "TimeAdvance", "SingleStep"))
    plug, gb = PLUGINS[plugin]

    def where(p):
        return os.path.join(HERE, p) if p.startswith("harness/") else os.path.join(ref, p)

    files += [where(p) for p in plug] + [where(gb), os.path.join(HERE, "harness", "harness_main.cpp")]
    incs = [os.path.join(HERE, "harness"), os.path.join(src, "Geometry"), os.path.join(src, "Utils"), bnd, adv,
            os.path.join(src, "Base", "Common"), rie, os.path.join(src, "Base", "Slope_limiter", limiter),
            os.path.join(src, "Base", "TimeAdvance"), os.path.join(bnd, boundary), os.path.join(adv, scheme)]
    defs = [] if boundary == "Regular" else ["-DHARNESS_HAS_SCHEME_INDEX"]
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w", *defs] + [f"-I{i}" for i in incs] + files + ["-o", exe]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        return name, False, p.stderr[-2000:]
    return name, True, "built"


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None,
                    help="reference source root (default: $IBTFO_REFERENCE_DIR, else ../reference beside the repo)")
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("variants", nargs="*", help="names like ref_MUSCL_HLL_minmod_Regular_file")
    a = ap.parse_args(argv)
    if a.ref is None:
        sys.path.insert(0, os.path.dirname(HERE))
        from oracle import reference_dir
        a.ref = reference_dir() or ""
    if not os.path.isdir(os.path.join(a.ref, "Src")):
        print(f"reference sources not found under {a.ref}; nothing built")
        return 0
    os.makedirs(OUT, exist_ok=True)
    specs = default_variants()
    if a.variants:
        specs = [tuple(v.split("_")[1:]) for v in a.variants]
    bad = 0
    with cf.ThreadPoolExecutor(a.jobs) as ex:
        for name, ok, msg in ex.map(lambda s: build_one(a.ref, s, a.force), specs):
            if not ok:
                bad += 1
                print(f"FAILED {name}\n{msg}")
    print(f"{len(specs) - bad}/{len(specs)} reference variants ready in {OUT}")
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main())
