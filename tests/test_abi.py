"""The C-ABI library loads and exports every entry point the public header declares."""
import ctypes
import os
import re

from conftest import ROOT


def header_symbols():
    syms = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            syms |= set(re.findall(r"\b(mks_[a-z0-9_]+)\s*\(", txt))
    return syms


def test_header_symbols_exported(lib):
    so = ctypes.CDLL(os.path.join(ROOT, "milc_qcd_gb300", "libmilc_ks_gb300.so"))
    missing = [s for s in sorted(header_symbols()) if not hasattr(so, s)]
    assert not missing, missing
    assert len(header_symbols()) >= 30


def test_python_signatures_cover_header(lib):
    from milc_qcd_gb300 import _lib
    assert header_symbols() <= set(_lib.SIGNATURES), header_symbols() - set(_lib.SIGNATURES)


def test_error_strings(lib):
    from milc_qcd_gb300 import _lib
    L = _lib.load()
    for st in (0, -1, -2, -3, -4, -5, -6, -7):
        assert L.mks_error_string(st)


def test_geometry_roundtrip(lib):
    dims = (4, 6, 2, 8)
    d = (ctypes.c_int * 4)(*dims)
    from milc_qcd_gb300 import _lib
    L = _lib.load()
    V = 4 * 6 * 2 * 8
    c = (ctypes.c_int * 4)()
    seen = set()
    for i in range(V):
        L.mks_site_coords(d, i, c)
        xyzt = tuple(c)
        assert (sum(xyzt) % 2 == 0) == (i < V // 2)
        assert L.mks_site_index(d, c) == i
        seen.add(xyzt)
    assert len(seen) == V
