"""The C ABI library loads and exports every entry point include/chl.h declares."""
import ctypes
import os
import re

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "chl.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(chl_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "chl_build" in names and "chl_query_batch" in names
    assert len(names) > 30


def test_library_exports_every_declared_symbol(P):
    lib = ctypes.CDLL(P.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_header(P):
    missing = [n for n in declared_functions() if n not in P.SIGNATURES]
    assert not missing, f"no Python signature for: {missing}"


def test_status_strings(P):
    L = P.lib()
    for s in range(7):
        assert L.chl_status_str(s)
