"""Restart files in the reference's .ic format (pihm_ic_write / pihm_ic_read,
host only): a round trip through the library, and a file the library wrote
read by the reference's own ReadIc (src/read_ic.c) when its build is here."""
import ctypes
import os

import numpy as np
import pytest

import pihm_gpu.watershed as W

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_F64P = ctypes.POINTER(ctypes.c_double)


def _lib():
    from pihm_gpu import capi
    if not os.path.exists(capi.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    lib = capi.load()
    for name in ("pihm_ic_write", "pihm_ic_read"):
        f = getattr(lib, name)
        f.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, _F64P, _F64P, _F64P]
        f.restype = ctypes.c_int
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_F64P)


def _state():
    ws = W.Watershed.load(os.path.join(GOLD, "c0_watershed.npz"))
    rng = np.random.default_rng(3)
    y = W.jitter(W.reference_state(ws, 2), 4)
    cmc = rng.uniform(0, 1e-3, ws.nelem)
    sneqv = rng.uniform(0, 1e-2, ws.nelem)
    return ws, y, cmc, sneqv


def test_ic_round_trip(tmp_path):
    lib = _lib()
    ws, y, cmc, sneqv = _state()
    path = str(tmp_path / "c0.ic").encode()
    assert lib.pihm_ic_write(path, ws.nelem, ws.nriver, _p(y), _p(cmc), _p(sneqv)) == 0
    assert os.path.getsize(path) == 8 * (5 * ws.nelem + 2 * ws.nriver)
    y2, c2, s2 = np.zeros_like(y), np.zeros_like(cmc), np.zeros_like(sneqv)
    assert lib.pihm_ic_read(path, ws.nelem, ws.nriver, _p(y2), _p(c2), _p(s2)) == 0
    assert np.array_equal(y2, y) and np.array_equal(c2, cmc) and np.array_equal(s2, sneqv)
    # a file for another mesh size is refused, as the reference refuses it
    assert lib.pihm_ic_read(path, ws.nelem + 1, ws.nriver, _p(np.zeros(y.size + 3)), None, None) == -4


def test_reference_reads_the_library_ic(tmp_path):
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference build is not here")
    lib = _lib()
    ws, y, cmc, sneqv = _state()
    path = str(tmp_path / "c0.ic")
    assert lib.pihm_ic_write(path.encode(), ws.nelem, ws.nriver, _p(y), _p(cmc), _p(sneqv)) == 0
    ref = oracle.Reference()
    ref.build(ws)
    f = ref.lib.ref_read_ic
    f.argtypes = [ctypes.c_char_p, _F64P, _F64P, _F64P]
    y2, c2, s2 = np.zeros_like(y), np.zeros_like(cmc), np.zeros_like(sneqv)
    assert f(path.encode(), _p(y2), _p(c2), _p(s2)) == 0
    assert np.array_equal(y2, y) and np.array_equal(c2, cmc) and np.array_equal(s2, sneqv)
