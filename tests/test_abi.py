"""The C-ABI library builds and exports every entry point of include/tegpu.h
(CPU only: no compute call is made)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(te_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = _declared("tegpu.h")
    assert "te_evolver_run" in names and "te_matrix_create_coo" in names


def test_library_exports_all_declared_symbols():
    import timeevolver_gb300 as te
    te.build()
    lib = ctypes.CDLL(te.LIB_PATH)
    declared = _declared("tegpu.h") + _declared("te_diag.h")
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared) <= set(te.SIGNATURES)


def test_model_library_exports_all_declared_symbols():
    import timeevolver_gb300 as te
    te.build()
    lib = ctypes.CDLL(os.path.join(os.path.dirname(te.LIB_PATH), "libtimeevolver.so"))
    missing = [n for n in _declared("te_model.h") if not hasattr(lib, n)]
    assert not missing, missing


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    import timeevolver_gb300 as te
    monkeypatch.setattr(te, "LIB_PATH", str(tmp_path / "nope.so"))
    monkeypatch.setattr(te, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        te.lib()
