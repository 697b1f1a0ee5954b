"""The C-ABI library loads and exports every entry point the header declares
(no compute: no GPU needed)."""
import os
import re

import pytest

from doublyperiodicstokes_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "dpstokes_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dpst_[a-z_]+)\s*\(", txt)))


def test_header_and_binding_agree():
    assert declared_functions() == sorted(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol():
    path = build.build()
    L = _lib.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert L.dpst_version().startswith(b"dpstokes_gb300")
    assert os.path.samefile(path, build.lib_path())


def test_errors_without_gpu_are_reported_not_thrown():
    import ctypes
    L = _lib.lib(build_if_missing=True)
    h = ctypes.c_void_p()
    p = _lib.DpstParams()
    p.mode = 7
    rc = L.dpst_create(ctypes.byref(p), 10, 0, ctypes.byref(h))
    assert rc == 1
    assert b"mode" in L.dpst_last_error()
    assert L.dpst_destroy(None) == 0
