"""CPU-side checks of the C ABI library: it builds, loads and exports every
function declared in include/prodm_gb300.h (no compute calls without a GPU)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    txt = open(os.path.join(ROOT, "include", "prodm_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(prodm_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from prodm_gb300 import build
    build.build()
    from prodm_gb300 import _lib
    lib = _lib.load()
    names = declared()
    assert len(names) > 20
    for n in names:
        assert hasattr(lib, n), n
    # the ctypes table covers the whole header
    assert sorted(_lib.declared_symbols()) == names


def test_error_string_and_validation_without_gpu():
    from prodm_gb300 import _lib
    lib = _lib.load()
    import ctypes as C
    out = C.c_int()
    dims = (C.c_uint32 * 3)(513, 513, 513)
    assert lib.prodm_max_level(3, dims, C.byref(out)) == 0
    assert out.value == 8
    # invalid geometry is rejected on the host with a message
    bad = (C.c_uint32 * 3)(0, 5, 5)
    rc = lib.prodm_level_dims(3, bad, 1, None, None)
    assert rc == 1
    assert b"zero-sized" in lib.prodm_last_error_string()
