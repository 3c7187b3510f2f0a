"""The reference's own driver programs link against the library.

A reference driver (Test/Sod/Sod.cpp, Test/InclineSod/InclineSod.cpp,
Test/Vortex/Vortex.cpp) is compiled unchanged with its case plug-ins
(Initialize.cpp, Level_Set_function.cpp), the reference's .inp reader
(Src/Utils/ParamReader.cpp) and ibtfo_gb300/forward/ibtfo_forward.cpp in place
of the Src/ solver files, with the include paths its Makefile's slot
selection gives (Test/Sod/Makefile:21-37), and linked against
libibtfo_gb300.so.  The forwarding file includes the reference's own headers,
so every forwarded signature is checked against the declaration the driver
calls.  Link only: what the linked calls do on the GPU is covered by
test_gpu_host.py's reference-driver sequence.

Needs the reference sources (oracle.reference_dir()) and g++; skipped
elsewhere."""
import os
import shutil
import subprocess

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "ibtfo_gb300")
FORWARD = os.path.join(LIB_DIR, "forward", "ibtfo_forward.cpp")

# (driver directory, driver source, Boundary slot, macro of that slot)
DRIVERS = [
    ("InclineSod", "InclineSod.cpp", "IDWBaseGFM", "IBTFO_BOUNDARY_IDW_GFM"),
    ("Sod", "Sod.cpp", "Regular", "IBTFO_BOUNDARY_REGULAR"),
    ("Vortex", "Vortex.cpp", "IDWBaseGFM", "IBTFO_BOUNDARY_IDW_GFM"),
]


def slot_includes(ref, scheme="MUSCL", riemann="HLL", limiter="minmod", boundary="IDWBaseGFM"):
    """-I flags of the reference Makefile for one slot choice
    (Test/InclineSod/Makefile:13-38, Equation = Euler)."""
    s = os.path.join(ref, "Src")
    dirs = ["Geometry", "Utils", "BoundaryCondition", "Base/Euler/Advection", "Base/Common", "Base/Euler/Riemann",
            f"Base/Slope_limiter/{limiter}", "Base/TimeAdvance", f"BoundaryCondition/{boundary}",
            f"Base/Euler/Advection/{scheme}"]
    return ["-I" + os.path.join(s, d) for d in dirs]


@pytest.mark.parametrize("case,driver,boundary,macro", DRIVERS)
def test_reference_driver_links(tmp_path, case, driver, boundary, macro):
    ref = oracle.reference_dir()
    if ref is None:
        pytest.skip("reference sources not present")
    if shutil.which("g++") is None:
        pytest.skip("g++ not present")
    lib = os.path.join(LIB_DIR, "libibtfo_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("libibtfo_gb300.so not built")
    tdir = os.path.join(ref, "Test", case)
    srcs = [os.path.join(tdir, driver), os.path.join(tdir, "Initialize.cpp"),
            os.path.join(tdir, "Level_Set_function.cpp"), os.path.join(ref, "Src", "Utils", "ParamReader.cpp"),
            FORWARD]
    exe = str(tmp_path / f"{case}.ex")
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-I" + os.path.join(ROOT, "oracle", "harness"),
           "-I" + os.path.join(ROOT, "include")] + slot_includes(ref, boundary=boundary) + \
        ["-DIBTFO_SCHEME=IBTFO_SCHEME_MUSCL", "-DIBTFO_RIEMANN=IBTFO_RIEMANN_HLL",
         "-DIBTFO_LIMITER=IBTFO_LIMITER_MINMOD", f"-DIBTFO_BOUNDARY={macro}"] + srcs + \
        ["-L" + LIB_DIR, "-libtfo_gb300", "-Wl,-rpath," + LIB_DIR, "-o", exe]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    # the solver entry points the driver calls come from the forwarding file,
    # and each forwards to the library's C ABI
    nm = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    for name in ("Psy_coord", "Level_Set", "Scheme_Index", "TimeAdvance", "Boundary", "Global_Boundary",
                 "ComputeDt", "CaculateMass", "WriteData"):
        assert any(f" T {name}(" in ln for ln in nm.splitlines()), name
    for sym in ("ibtfo_ref_TimeAdvance", "ibtfo_ref_Boundary", "ibtfo_ref_ComputeDt"):
        assert any(ln.strip() == f"U {sym}" for ln in nm.splitlines()), sym
