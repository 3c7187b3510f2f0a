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
        ib.Case(16, 8, scheme="Lax")


def test_null_pointers_rejected():
    L = ib.lib()
    assert L.ibtfo_create(None, None) == 1
    assert L.ibtfo_advance(None, 1) == 1
    assert L.ibtfo_get_state(None, None, None) == 1
