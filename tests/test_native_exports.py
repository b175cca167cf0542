"""The C-ABI library builds for sm_103a, loads, and exports every declared entry point.

No compute calls: this runs without a GPU.
"""
import glob
import os
import re

from helpers import GOLDEN  # noqa: F401  (ensures tests/ is importable)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*[\s\*]+(sc_[A-Za-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    assert {"sc_element_matrices", "sc_assemble_values", "sc_newmark_run"} <= names


def test_library_exports_every_declared_symbol(native_lib):
    missing = [n for n in sorted(declared_functions()) if not hasattr(native_lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(native_lib):
    from scatter_gb300 import _native

    assert declared_functions() <= set(_native.SIGNATURES)


def test_status_strings(native_lib):
    assert native_lib.sc_version() >= 1
    assert native_lib.sc_status_string(0) == b"ok"
    assert b"converged" in native_lib.sc_status_string(2)


def test_built_for_sm103a(native_lib):
    from scatter_gb300 import build

    assert "arch=compute_103a,code=sm_103a" in build.ARCH
    assert os.path.getsize(build.LIB) > 0
