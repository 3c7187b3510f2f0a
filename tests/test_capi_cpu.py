"""CPU-only checks of the C ABI boundary: the library loads without a GPU and
exports every function include/*.h declares; argument validation happens
before any device work."""
import ctypes as C
import glob
import os
import re

import pytest

import ibtfo_gb300 as ib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(ibtfo_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = ib.lib()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    names = set(declared_functions())
    bound = set(ib.SIGNATURES) | set(ib.REF_SIGNATURES)
    assert names == bound, (names - bound, bound - names)


def test_abi_version():
    assert ib.lib().ibtfo_abi_version() == 1


@pytest.mark.parametrize("bad", [dict(ng=1), dict(n_x=1), dict(hi=(0.0, 1.0)), dict(gamma=1.0), dict(cfl=0.0)])
def test_invalid_config_rejected_without_gpu(bad):
    kw = dict(n_x=16, n_y=8)
    kw.update(bad)
    with pytest.raises(ib.IbtfoError) as e:
        ib.Case(**kw)
    assert e.value.code == 1  # IBTFO_EINVAL


def test_unknown_key_rejected():
    with pytest.raises(KeyError):
        ib.Case(16, 8, scheme="Lax-Wendroff")
    with pytest.raises(KeyError):
        ib.Case(16, 8, time="RK3")


@pytest.mark.parametrize("bad", [dict(scheme="Lax", precision="fp32c"), dict(scheme="Lax", boundary="CCM", riemann="HLL_Toro"),
                                 dict(time="RK2", boundary="CCM", riemann="HLL_Toro")])
def test_lax_and_rk2_limits_rejected_without_gpu(bad):
    with pytest.raises(ib.IbtfoError, match="Lax|RK2") as e:
        ib.Case(16, 8, **bad)
    assert e.value.code == 1


@pytest.mark.parametrize("riemann", ["HLL", "HLLC", "PVRS"])
def test_cut_cells_reject_the_reference_solvers_without_gpu(riemann):
    """A solver key names one solver whatever the boundary: the cut-cell sweep
    runs HLL_Toro, StegerWarming and HLLC_Toro, and has no form of the
    reference's HLL (the HLL and HLLC keys) or of PVRS."""
    with pytest.raises(ib.IbtfoError, match="cut-cell") as e:
        ib.Case(16, 8, boundary="CCM", riemann=riemann)
    assert e.value.code == 1


def test_null_pointers_rejected():
    L = ib.lib()
    assert L.ibtfo_create(None, None) == 1
    assert L.ibtfo_advance(None, 1) == 1
    assert L.ibtfo_get_state(None, None, None) == 1


STRUCTS = {
    "ibtfo_config": "Config", "ibtfo_progress": "Progress", "ibtfo_batch_config": "BatchConfig",
    "ibtfo_batch_tiling": "BatchTiling", "ibtfo_body": "Body", "ibtfo_server_config": "ServerConfig",
    "ibtfo_request": "Request", "ibtfo_result": "Result", "ibtfo_server_stats": "ServerStats",
}


def test_ctypes_layouts_match_the_header(tmp_path):
    """Size and every field offset of each public struct, as gcc lays out
    include/ibtfo.h, equal the ctypes mirrors in the Python binding."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ibtfo.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        py = getattr(ib, pyname)
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            s, f, v = ln.split()
            got[(s, f)] = int(v)
    for cname, pyname in STRUCTS.items():
        py = getattr(ib, pyname)
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)
