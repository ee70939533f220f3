"""ctypes binding of the device N_Vector (include/pihm_nvector.h)."""
from __future__ import annotations

import ctypes

from . import capi

_VP = ctypes.c_void_p
_D = ctypes.c_double
_NV = ctypes.c_void_p
_lib = None

COEF_HOST, COEF_NEG, COEF_INV, COEF_INV_INV, COEF_NEG_INV_INV = range(5)


class Coef(ctypes.Structure):
    """pihm_nv_coef: a linear-sum coefficient, a constant or formed from a slot."""
    _fields_ = [("kind", ctypes.c_int32), ("slot", ctypes.c_int32), ("value", ctypes.c_double)]


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    lib = capi.load()
    sig = {
        "N_VNew_PihmGpu": ([ctypes.c_long, _VP], _NV),
        "N_VMake_PihmGpu": ([ctypes.c_long, _VP, _VP], _NV),
        "N_VGetDeviceArrayPointer_PihmGpu": ([_NV], _VP),
        "N_VGetLength_PihmGpu": ([_NV], ctypes.c_long),
        "N_VCopyFromHost_PihmGpu": ([_NV, _VP], ctypes.c_int),
        "N_VCopyToHost_PihmGpu": ([_NV, _VP], ctypes.c_int),
        "N_VGetVectorID_PihmGpu": ([_NV], ctypes.c_int),
        "N_VClone_PihmGpu": ([_NV], _NV),
        "N_VCloneEmpty_PihmGpu": ([_NV], _NV),
        "N_VDestroy_PihmGpu": ([_NV], None),
        "N_VLinearSum_PihmGpu": ([_D, _NV, _D, _NV, _NV], None),
        "N_VConst_PihmGpu": ([_D, _NV], None),
        "N_VProd_PihmGpu": ([_NV, _NV, _NV], None),
        "N_VDiv_PihmGpu": ([_NV, _NV, _NV], None),
        "N_VScale_PihmGpu": ([_D, _NV, _NV], None),
        "N_VAbs_PihmGpu": ([_NV, _NV], None),
        "N_VInv_PihmGpu": ([_NV, _NV], None),
        "N_VAddConst_PihmGpu": ([_NV, _D, _NV], None),
        "N_VDotProd_PihmGpu": ([_NV, _NV], _D),
        "N_VMaxNorm_PihmGpu": ([_NV], _D),
        "N_VWrmsNorm_PihmGpu": ([_NV, _NV], _D),
        "N_VWrmsNormMask_PihmGpu": ([_NV, _NV, _NV], _D),
        "N_VMin_PihmGpu": ([_NV], _D),
        "N_VWL2Norm_PihmGpu": ([_NV, _NV], _D),
        "N_VL1Norm_PihmGpu": ([_NV], _D),
        "N_VCompare_PihmGpu": ([_D, _NV, _NV], None),
        "N_VInvTest_PihmGpu": ([_NV, _NV], ctypes.c_int),
        "N_VConstrMask_PihmGpu": ([_NV, _NV, _NV], ctypes.c_int),
        "N_VMinQuotient_PihmGpu": ([_NV, _NV], _D),
        "N_VDotProdSlot_PihmGpu": ([_NV, _NV, ctypes.c_int], ctypes.c_int),
        "N_VWrmsNormSlot_PihmGpu": ([_NV, _NV, ctypes.c_int], ctypes.c_int),
        "N_VLinearSumCoef_PihmGpu": ([ctypes.POINTER(Coef), _NV, ctypes.POINTER(Coef), _NV, _NV], ctypes.c_int),
        "N_VFetchSlots_PihmGpu": ([_NV, ctypes.c_int, ctypes.POINTER(_D), _VP, ctypes.POINTER(ctypes.c_uint)],
                                  ctypes.c_int),
        "N_VGetStream_PihmGpu": ([_NV], _VP),
        "pihm_gpu_nv_linear_sum": ([_D, _VP, _D, _VP, _VP, ctypes.c_int64, _VP], ctypes.c_int),
        "pihm_gpu_nv_wrms_norm": ([_VP, _VP, ctypes.c_int64, _VP, ctypes.POINTER(_D)], ctypes.c_int),
        "pihm_gpu_nv_dot_prod": ([_VP, _VP, ctypes.c_int64, _VP, ctypes.POINTER(_D)], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def wrms_norm(x_ptr: int, w_ptr: int, n: int, stream: int | None = None) -> float:
    lib = load()
    r = _D()
    rc = lib.pihm_gpu_nv_wrms_norm(_VP(x_ptr), _VP(w_ptr), n, _VP(stream), ctypes.byref(r))
    if rc:
        raise capi.PihmGpuError("pihm_gpu_nv_wrms_norm", rc)
    return r.value


def dot_prod(x_ptr: int, y_ptr: int, n: int, stream: int | None = None) -> float:
    lib = load()
    r = _D()
    rc = lib.pihm_gpu_nv_dot_prod(_VP(x_ptr), _VP(y_ptr), n, _VP(stream), ctypes.byref(r))
    if rc:
        raise capi.PihmGpuError("pihm_gpu_nv_dot_prod", rc)
    return r.value
