"""The C-ABI library builds, loads without a GPU and exports every symbol
that include/pysph_gb300.h declares."""
import ctypes
import os
import re

from pysph_gb300 import native

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^\s*int\s+(sph_\w+)\s*\(", txt, flags=re.M))
    return names


def test_library_exports_every_declared_symbol():
    L = native.load_library()
    declared = _declared()
    assert declared, "no declarations found"
    assert declared <= set(native.EXPORTS) | declared
    for name in declared:
        assert hasattr(L, name), name
        assert isinstance(getattr(L, name), ctypes._CFuncPtr)
    assert set(native.EXPORTS) == declared


def test_version_and_error_path_without_gpu():
    L = native.load_library()
    assert L.sph_version() >= 1
    # argument errors are reported without touching the device
    rc = L.sph_ctx_create(7, ctypes.byref(ctypes.c_void_p()))
    assert rc == native.SPH_ERR_ARG
    assert "dim" in native.last_error()
