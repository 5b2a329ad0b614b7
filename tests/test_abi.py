"""The C-ABI library loads and exports every symbol include/*.h declares (no GPU calls)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(bm_\w+)\s*\(", src))
    return names


def test_header_declares_entry_points():
    names = _declared()
    assert "bm_dgbmv" in names and "bm_sgbmv" in names
    assert len(names) >= 4


def test_library_exports_every_declared_symbol(bm):
    lib = ctypes.CDLL(bm._lib.LIB_PATH)
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_header(bm):
    declared = _declared()
    bound = set(bm._lib.SIGNATURES)
    assert declared == bound, f"header-only: {declared - bound}, binding-only: {bound - declared}"


def test_library_reports_version_without_gpu(bm):
    L = bm._lib.load()
    assert L.bm_version() >= 100
    assert isinstance(L.bm_last_error(), bytes)
