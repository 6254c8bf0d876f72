"""The C-ABI library loads and exports every entry point include/*.h declares."""
import ctypes
import glob
import os
import re

from parthenon_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(pgb_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_header_symbols():
    lib = ctypes.CDLL(_native.lib_path())
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert declared_symbols() <= set(_native.exported_symbols())


def test_version_and_error_string():
    L = _native.lib()
    assert L.pgb_version() >= 1
    rc = L.pgb_mesh_get_info(None, None)
    assert rc == -1
    assert b"null" in L.pgb_last_error()
