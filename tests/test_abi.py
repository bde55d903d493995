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


def test_struct_layouts_match_header(P, tmp_path):
    """The ctypes mirrors of the option and statistics structs have the C
    header's size and field offsets (a mismatch would pass garbage options)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    pairs = [("chl_build_opts", P.BuildOpts), ("chl_build_stats", P.BuildStats),
             ("chl_server_opts", P.ServerOpts)]
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "chl.h"', "int main(void) {"]
    for cname, py in pairs:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in pairs:
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)
