"""The C-ABI library loads and exports every function include/*.h declares
(no GPU needed: nothing is called)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b(pihm_(?:gpu|bdf|batch|serve|ic|deck)_\w+|N_V\w+_PihmGpu)\s*\(", src):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = _declared()
    assert "pihm_gpu_create" in names and "pihm_gpu_rhs" in names
    assert {"pihm_bdf_solve", "pihm_batch_add", "pihm_batch_step", "pihm_serve_run"} <= names
    assert {"pihm_deck_read", "pihm_deck_mesh", "pihm_deck_bc", "pihm_deck_free"} <= names


def test_library_exports_declared_symbols():
    from pihm_gpu import capi
    if not os.path.exists(capi.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(capi.LIB_PATH)
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, missing


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from pihm_gpu import capi
    monkeypatch.setattr(capi, "LIB_PATH", str(tmp_path / "nope.so"))
    monkeypatch.setattr(capi, "_lib", None)
    with pytest.raises(FileNotFoundError):
        capi.load()
