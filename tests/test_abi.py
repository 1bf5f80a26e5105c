"""CPU: the C-ABI library loads and exports every function declared in include/ac3d.h, and the
ctypes signature table covers exactly those functions."""
import os
import re

from acoustic_reliefs_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(ac3d_[a-z0-9_]+)\s*\(", txt))
    return names


def test_every_declared_symbol_is_exported():
    lib = L.lib()
    names = declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_signature_table_matches_header():
    assert declared() == set(L.SIGNATURES)


def test_version_string():
    assert b"sm_103a" in L.lib().ac3d_version()


def test_create_rejects_bad_arguments():
    import ctypes
    import numpy as np
    h = ctypes.c_void_p()
    bands = np.array([1000.0])
    src = np.array([0.0, 100.0, 0.0])
    # cluster size 0 is rejected before any device work
    rc = L.lib().ac3d_create(ctypes.byref(h), 0, 1.5, L.ptr(bands), 1, 1, 1e-3, 1e-3, 1e-3, L.ptr(src), 50.0, 5.0, 0)
    assert rc == L.ERR_ARG and not h.value


def test_krylov_option_rejects_bad_arguments():
    """ac3d_set_krylov / ac3d_server_set_krylov validate before touching any context."""
    lib = L.lib()
    assert lib.ac3d_set_krylov(None, 1, 300) == L.ERR_ARG
    assert lib.ac3d_server_set_krylov(None, 1, 300) == L.ERR_ARG
