"""The C ABI library builds for sm_103a, loads, and exports every function include/oakg.h
declares. No compute call is made here (no GPU in the CPU suite)."""
import ctypes
import os
import re

import pytest

from oak_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "oakg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:int|void|size_t)\s+\**\s*(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref in ("oak_init", "oak_assim", "oak_done", "oakg_analysis", "oakg_locanalysis"):
        assert ref in names


def test_library_exports_every_declared_symbol():
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_loads():
    build.build()
    import oak_gb300
    L = oak_gb300.lib()
    assert L.oakg_last_status() == 0


def declared_arities():
    src = open(os.path.join(ROOT, "include", "oakg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for name, params in re.findall(r"^\s*(?:int|void|size_t)\s+\**\s*(\w+)\s*\(([^)]*)\)",
                                   src, flags=re.M):
        p = params.strip()
        out[name] = 0 if p in ("", "void") else p.count(",") + 1
    return out


def test_python_argtypes_match_header():
    build.build()
    import oak_gb300
    L = oak_gb300.lib()
    bad = {}
    for name, k in declared_arities().items():
        at = getattr(L, name).argtypes
        if at is not None and len(at) != k:
            bad[name] = (len(at), k)
    assert not bad, f"argtypes length != header parameter count: {bad}"


def test_header_compiles_as_c_and_cpp(tmp_path):
    """include/oakg.h is a plain C header (C99) usable from C++ as well."""
    import shutil
    import subprocess
    header = os.path.join(ROOT, "include", "oakg.h")
    for comp, lang, std in (("gcc", "c", "-std=c99"), ("g++", "c++", "-std=c++11")):
        exe = shutil.which(comp)
        if exe is None:
            pytest.skip(f"no {comp}")
        subprocess.run([exe, "-fsyntax-only", std, "-Wall", "-Werror", "-x", lang, header],
                       check=True)
