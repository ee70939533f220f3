"""ctypes mirror of `pihm_gpu_mesh` (include/pihm_gpu.h).

`MeshDesc.from_arrays` keeps references to the numpy arrays it points at, so
the description stays valid as long as the returned object lives.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .watershed import MESH_FIELDS, RIVER_INT_FIELDS, ELEM_INT_FIELDS

_I32P = ctypes.POINTER(ctypes.c_int32)
_F64P = ctypes.POINTER(ctypes.c_double)

_ORDER = (
    "nabr", "bc_type", "area", "zmin", "zmax", "edge", "nabrdist", "nabr_x",
    "nabr_y", "depth", "ksath", "ksatv", "kinfv", "dinf", "alpha", "beta",
    "porosity", "dmac", "kmach", "kmacv", "areafv", "areafh", "rough", "rzd",
    "down", "leftele", "rightele", "intrpl_ord", "riverbc_type",
    "riv_area", "riv_zmin", "riv_zmax", "riv_zbed", "riv_node_zmax",
    "riv_dist_left", "riv_dist_right", "riv_depth", "riv_coeff", "riv_length",
    "riv_width", "riv_rough", "riv_cwr", "riv_ksath", "riv_ksatv",
    "riv_bedthick", "riv_porosity",
)
assert set(_ORDER) == set(MESH_FIELDS)
_INTS = set(ELEM_INT_FIELDS) | set(RIVER_INT_FIELDS)


class MeshDesc(ctypes.Structure):
    _fields_ = [("nelem", ctypes.c_int32), ("nriver", ctypes.c_int32)] + [
        (name, _I32P if name in _INTS else _F64P) for name in _ORDER]

    @staticmethod
    def from_arrays(nelem: int, nriver: int, arrays: dict) -> "MeshDesc":
        d = MeshDesc()
        d.nelem = nelem
        d.nriver = nriver
        keep = []
        for name in _ORDER:
            if name in _INTS:
                a = np.ascontiguousarray(arrays[name], np.int32)
                setattr(d, name, a.ctypes.data_as(_I32P))
            else:
                a = np.ascontiguousarray(arrays[name], np.float64)
                setattr(d, name, a.ctypes.data_as(_F64P))
            keep.append(a)
        d._keep = keep
        return d


def f64p(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_F64P)


def i32p(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_I32P)
