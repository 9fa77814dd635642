"""The C-ABI library builds, loads and exports every entry point declared in
include/nsg.h (no compute calls: runs without a GPU)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "nsg.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(nsg_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    import networksolvers_gb300.build as nb
    lib = nb.build()
    L = ctypes.CDLL(str(lib))
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_ctypes_signatures_cover_header():
    from networksolvers_gb300 import _native
    assert set(declared_symbols()) <= set(_native.exported_symbols())


def test_product_fails_loudly_without_library(tmp_path, monkeypatch):
    from networksolvers_gb300 import _native
    monkeypatch.setenv("NSG_LIB", str(tmp_path / "missing.so"))
    monkeypatch.setattr(_native, "_LIB", None)
    import pytest
    with pytest.raises(RuntimeError):
        _native.lib()
