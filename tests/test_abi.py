"""CPU tests of the C ABI: the library builds, loads and exports every
symbol include/mrgpu.h declares; host-only entry points behave."""
import ctypes as C
import os
import re

from conftest import ROOT


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "mrgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mrg_[a-z0-9_]+)\s*\(", txt)))


def test_header_symbols_exported(mrg):
    lib = mrg.load()
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/mrgpu.h but not exported"
    assert set(names) == set(mrg.EXPORTED) | (set(names) - set(mrg.EXPORTED))
    for n in mrg.EXPORTED:
        assert n in names, f"{n} bound in mrgpu.py but not declared"


def test_host_only_entry_points(mrg):
    lib = mrg.load()
    assert lib.mrg_version().decode().startswith("mrgpu")
    c = mrg.Controls()
    lib.mrg_controls_default(C.byref(c))
    # foam defaults: tolerance 1e-6, relTol 0, minIter 0, maxIter 1000
    assert (c.tolerance, c.rel_tol, c.min_iter, c.max_iter) == (1e-6, 0.0, 0, 1000)
    assert lib.mrg_ctx_destroy(None) == 0
    rc = lib.mrg_ctx_create(0, 0, None)
    assert rc == mrg.MRG_E_INVALID
    assert "NULL" in lib.mrg_last_error().decode()
