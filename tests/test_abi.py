"""CPU tests of the C ABI: the library loads and exports every symbol the
header declares; argument checking needs no GPU."""
import ctypes as C
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "andromeda_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(agb_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported(agb):
    L = agb.load()
    syms = declared_symbols()
    assert len(syms) >= 16
    for s in syms:
        assert hasattr(L, s), s
    from andromeda_gb300._lib import SIGNATURES
    assert sorted(SIGNATURES) == syms


def test_version_and_no_device_error(agb):
    L = agb.load()
    assert b"sm_103a" in L.agb_version()
    # a context on an absent / out-of-range device fails cleanly with a message
    h = C.c_void_p()
    rc = L.agb_create(C.byref(h), 1 << 20)
    assert rc != 0
    assert len(L.agb_last_error(None)) > 0


def test_lsqr_dropin_argument_checks(agb):
    L = agb.load()
    mi, nit, ierr = C.c_int(0), C.c_int(0), C.c_int(0)
    z = np.zeros(1)
    rc = L.agb_lsqr_solve(0, 0, 0, C.byref(mi), 1e-8, C.byref(nit), C.byref(ierr), z, np.zeros(1, np.int64),
                          np.zeros(1, np.int32), z, z, z)
    assert rc == 1  # AGB_ERR_ARG before any CUDA call
