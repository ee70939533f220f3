"""ctypes binding of the C ABI in include/pihm_gpu.h.

The shared library is built in place (`make -C pihm-cuda_gb300`, or
`__graft_entry__.build()`); this module never falls back to anything else:
if lib/libpihm_gpu.so is missing or a call fails, it raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .meshdesc import MeshDesc, f64p, i32p

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libpihm_gpu.so")

ERRORS = {
    -1: "PIHM_GPU_ERR_ARG", -2: "PIHM_GPU_ERR_CUDA", -3: "PIHM_GPU_ERR_NAN",
    -4: "PIHM_GPU_ERR_MESH", -5: "PIHM_GPU_ERR_NOMEM", -6: "PIHM_GPU_ERR_BCTYPE",
}
ORDER_REFERENCE, ORDER_RCM = 0, 1

_lib = None
_F64P = ctypes.POINTER(ctypes.c_double)
_I32P = ctypes.POINTER(ctypes.c_int32)
_VP = ctypes.c_void_p


class PihmGpuError(RuntimeError):
    def __init__(self, fn: str, rc: int):
        super().__init__(f"{fn} failed: {ERRORS.get(rc, rc)}")
        self.rc = rc


def load() -> ctypes.CDLL:
    """Load lib/libpihm_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError(
            f"{LIB_PATH} is missing: build it with `make -C {PKG_DIR}` "
            "(or __graft_entry__.build()); there is no fallback path")
    lib = ctypes.CDLL(LIB_PATH)
    sig = {
        "pihm_gpu_create": ([ctypes.POINTER(MeshDesc), ctypes.c_int, ctypes.c_int,
                             ctypes.c_double, ctypes.c_int, ctypes.POINTER(_VP)], ctypes.c_int),
        "pihm_gpu_destroy": ([_VP], None),
        "pihm_gpu_set_stream": ([_VP, _VP], ctypes.c_int),
        "pihm_gpu_set_kernel_shape": ([_VP, ctypes.c_int], ctypes.c_int),
        "pihm_gpu_rhs_host_async": ([_VP, ctypes.c_double, _VP, _VP], ctypes.c_int),
        "pihm_gpu_wait": ([_VP], ctypes.c_int),
        "pihm_gpu_sizes": ([_VP, _I32P, _I32P, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
        "pihm_gpu_get_permutation": ([_VP, _I32P, _I32P], ctypes.c_int),
        "pihm_gpu_set_forcing": ([_VP, _F64P, _F64P, _F64P], ctypes.c_int),
        "pihm_gpu_set_bc": ([_VP, _F64P, _F64P], ctypes.c_int),
        "pihm_gpu_set_ws0_surf": ([_VP, _F64P], ctypes.c_int),
        "pihm_gpu_set_river_edge_ovlflow": ([_VP, _F64P], ctypes.c_int),
        "pihm_gpu_rhs": ([_VP, ctypes.c_double, _VP, _VP], ctypes.c_int),
        "pihm_gpu_status": ([_VP], ctypes.c_int),
        "pihm_gpu_rhs_host": ([_VP, ctypes.c_double, _F64P, _F64P], ctypes.c_int),
        "pihm_gpu_set_diagnostics": ([_VP, ctypes.c_int], ctypes.c_int),
        "pihm_gpu_set_host_path": ([_VP, ctypes.c_int], ctypes.c_int),
        "pihm_gpu_host_path_info": ([_VP, _I32P, _I32P], ctypes.c_int),
        "pihm_gpu_get_fluxes": ([_VP] + [_F64P] * 6, ctypes.c_int),
        "pihm_gpu_to_internal": ([_VP, _VP, _VP], ctypes.c_int),
        "pihm_gpu_to_reference": ([_VP, _VP, _VP], ctypes.c_int),
        "pihm_gpu_launch_count": ([_VP, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
        "pihm_gpu_set_profiling": ([_VP, ctypes.c_int], ctypes.c_int),
        "pihm_gpu_water_balance": ([_VP, _VP, ctypes.c_double, _F64P], ctypes.c_int),
        "pihm_gpu_kernel_times": ([_VP, _F64P, ctypes.POINTER(ctypes.c_int64), ctypes.c_int],
                                  ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _check(fn: str, rc: int) -> int:
    if rc < 0:
        raise PihmGpuError(fn, rc)
    return rc


def _c(a):
    return None if a is None else np.ascontiguousarray(a, np.float64)


class GpuRhs:
    """One watershed resident on the GPU (wraps pihm_gpu_ctx)."""

    def __init__(self, ws, order: int = ORDER_RCM, stream: int | None = None):
        self.lib = load()
        self.ws = ws
        self.desc = MeshDesc.from_arrays(ws.nelem, ws.nriver, ws.arrays)
        h = _VP()
        _check("pihm_gpu_create",
               self.lib.pihm_gpu_create(ctypes.byref(self.desc), ws.surf_mode, ws.riv_mode,
                                        float(ws.stepsize), order, ctypes.byref(h)))
        self.h = h
        if stream is not None:
            self.set_stream(stream)

    def close(self):
        if getattr(self, "h", None):
            self.lib.pihm_gpu_destroy(self.h)
            self.h = None

    __del__ = close

    @property
    def neq(self) -> int:
        return self.ws.neq

    def set_kernel_shape(self, shape: int):
        """Block shape of the element kernel (0: 512 x 2, 1: 256 x 4, 2: 128 x 8 per SM)."""
        _check("pihm_gpu_set_kernel_shape", self.lib.pihm_gpu_set_kernel_shape(self.h, int(shape)))

    def set_stream(self, stream: int):
        _check("pihm_gpu_set_stream", self.lib.pihm_gpu_set_stream(self.h, _VP(stream)))

    def permutation(self) -> np.ndarray:
        p = np.zeros(self.ws.nelem, np.int32)
        _check("pihm_gpu_get_permutation", self.lib.pihm_gpu_get_permutation(self.h, i32p(p), None))
        return p

    def set_forcing(self, pcpdrp=None, edir=None, ett=None):
        _check("pihm_gpu_set_forcing", self.lib.pihm_gpu_set_forcing(
            self.h, f64p(_c(pcpdrp)), f64p(_c(edir)), f64p(_c(ett))))

    def set_bc(self, elem_bc=None, river_bc=None):
        _check("pihm_gpu_set_bc", self.lib.pihm_gpu_set_bc(self.h, f64p(_c(elem_bc)),
                                                           f64p(_c(river_bc))))

    def water_balance(self, y_ptr: int, dt: float):
        """(sources, sinks, storage) of a model step from the device state
        y_ptr (internal order): the sums of PrintWaterBal."""
        out = np.zeros(3)
        _check("pihm_gpu_water_balance", self.lib.pihm_gpu_water_balance(self.h, _VP(y_ptr), float(dt), f64p(out)))
        return tuple(out)

    # ---- land-surface model (include/pihm_land.h) ----
    def land_init(self, land):
        """Attach a land.Land (forcing series and parameters) to the context."""
        from . import land as L
        lib = L._lib()
        p, s = land.structs()
        self._land = (land, p, s)  # the arrays stay referenced while the context lives
        _check("pihm_gpu_land_init", lib.pihm_gpu_land_init(self.h, ctypes.byref(p), ctypes.byref(s)))

    def land_set_state(self, cmc=None, sneqv=None):
        from . import land as L
        _check("pihm_gpu_land_set_state", L._lib().pihm_gpu_land_set_state(self.h, f64p(_c(cmc)), f64p(_c(sneqv))))

    def land_step(self, t: int, stepsize: float, y_ptr: int):
        """One land-surface step at model time t (s since 1970 UTC); y_ptr: the
        device state in internal order."""
        from . import land as L
        _check("pihm_gpu_land_step", L._lib().pihm_gpu_land_step(self.h, int(t), float(stepsize), _VP(y_ptr)))

    def land_get(self, field: str) -> np.ndarray:
        from . import land as L
        out = np.zeros(self.ws.nelem)
        _check("pihm_gpu_land_get", L._lib().pihm_gpu_land_get(self.h, L.FIELDS[field], f64p(out)))
        return out

    def set_ws0_surf(self, ws0):
        _check("pihm_gpu_set_ws0_surf", self.lib.pihm_gpu_set_ws0_surf(self.h, f64p(_c(ws0))))

    def set_river_edge_ovlflow(self, ovl):
        _check("pihm_gpu_set_river_edge_ovlflow",
               self.lib.pihm_gpu_set_river_edge_ovlflow(self.h, f64p(_c(ovl))))

    def set_noah(self, noah: dict):
        """Flux-PIHM right-hand side with Noah's per-step inputs (reference
        order): et [nelem, nlayers], nwtbl, nroot, sh2o0, smcmin, smcmax, fcr."""
        et = np.ascontiguousarray(noah["et"], np.float64)
        nl = et.shape[1] if et.ndim == 2 else 0
        nw = np.ascontiguousarray(noah["nwtbl"], np.int32)
        nr = np.ascontiguousarray(noah["nroot"], np.int32)
        f = self.lib.pihm_gpu_set_noah
        f.argtypes = [_VP, _F64P, ctypes.c_int, _I32P, _I32P, _F64P, _F64P, _F64P, _F64P]
        f.restype = ctypes.c_int
        _check("pihm_gpu_set_noah", f(self.h, f64p(et), nl, i32p(nw), i32p(nr),
                                      *(f64p(_c(noah[k])) for k in ("sh2o0", "smcmin", "smcmax", "fcr"))))

    def post_step(self, y_ptr: int):
        """pihm_gpu_post_step: ws0 <- the device state y_ptr (internal order)
        after a model step, as Summary sets it."""
        f = self.lib.pihm_gpu_post_step
        f.argtypes = [_VP, _VP]
        f.restype = ctypes.c_int
        _check("pihm_gpu_post_step", f(self.h, _VP(y_ptr)))

    # ---- the Noah land-surface model (include/pihm_noah.h) ----
    def noah_init(self, params: dict, state: dict):
        """Attach Noah (pihm_gpu.noah.synthetic_noah's dicts, reference order)."""
        from . import noah as N
        N.bind(self.lib)
        ps, kp = N.params_struct(params)
        ss, ks = N.state_struct(state)
        _check("pihm_gpu_noah_init", self.lib.pihm_gpu_noah_init(self.h, ctypes.byref(ps), ctypes.byref(ss)))

    def noah_set_state(self, state: dict):
        from . import noah as N
        ss, ks = N.state_struct(state)
        _check("pihm_gpu_noah_set_state", self.lib.pihm_gpu_noah_set_state(self.h, ctypes.byref(ss)))

    def noah_set_forcing(self, forcing: dict):
        from . import noah as N
        fs, kf = N.forcing_struct(forcing)
        _check("pihm_gpu_noah_set_forcing", self.lib.pihm_gpu_noah_set_forcing(self.h, ctypes.byref(fs)))

    def noah_step(self, dt: float):
        _check("pihm_gpu_noah_step", self.lib.pihm_gpu_noah_step(self.h, float(dt)))

    def noah_begin(self, y0_ptr: int):
        """The state the run starts from (device, internal order)."""
        _check("pihm_gpu_noah_begin", self.lib.pihm_gpu_noah_begin(self.h, _VP(y0_ptr)))

    def noah_post_step(self, y_ptr: int, stepsize: float):
        """After a model step ending at the device state y_ptr (internal order)."""
        _check("pihm_gpu_noah_post_step", self.lib.pihm_gpu_noah_post_step(self.h, _VP(y_ptr), float(stepsize)))

    def noah_get(self, name: str) -> np.ndarray:
        from . import noah as N
        out = np.zeros(N.field_shape(name, self.ws.nelem))
        _check("pihm_gpu_noah_get", self.lib.pihm_gpu_noah_get(self.h, N.field_id(name), f64p(out.reshape(-1))))
        return out

    def set_diagnostics(self, on: bool):
        _check("pihm_gpu_set_diagnostics", self.lib.pihm_gpu_set_diagnostics(self.h, int(on)))

    def set_host_path(self, mode: int):
        """0: rhs_host reads and writes host arrays directly where the device
        can address them; 1: it always copies through device staging."""
        _check("pihm_gpu_set_host_path", self.lib.pihm_gpu_set_host_path(self.h, int(mode)))

    def host_path_info(self):
        """(the last rhs_host accessed host memory directly, the device can
        access pageable host memory)."""
        d, p = ctypes.c_int32(), ctypes.c_int32()
        _check("pihm_gpu_host_path_info",
               self.lib.pihm_gpu_host_path_info(self.h, ctypes.byref(d), ctypes.byref(p)))
        return bool(d.value), bool(p.value)

    def rhs_host_ptr(self, y_ptr: int, ydot_ptr: int, t: float = 0.0) -> int:
        """pihm_gpu_rhs_host on raw host addresses (reference order)."""
        return self.lib.pihm_gpu_rhs_host(self.h, t, ctypes.cast(y_ptr, _F64P), ctypes.cast(ydot_ptr, _F64P))

    def rhs_host(self, y, t: float = 0.0):
        """Host arrays in reference order (in, evaluate, out; synchronous)."""
        y = _c(y)
        out = np.empty_like(y)
        rc = self.lib.pihm_gpu_rhs_host(self.h, t, f64p(y), f64p(out))
        return out, rc

    def rhs_device(self, y_ptr: int, ydot_ptr: int, t: float = 0.0):
        """Device pointers in internal order; asynchronous."""
        _check("pihm_gpu_rhs", self.lib.pihm_gpu_rhs(self.h, t, _VP(y_ptr), _VP(ydot_ptr)))

    def status(self) -> int:
        return self.lib.pihm_gpu_status(self.h)

    def to_internal(self, src_ptr: int, dst_ptr: int):
        _check("pihm_gpu_to_internal", self.lib.pihm_gpu_to_internal(self.h, _VP(src_ptr), _VP(dst_ptr)))

    def to_reference(self, src_ptr: int, dst_ptr: int):
        _check("pihm_gpu_to_reference", self.lib.pihm_gpu_to_reference(self.h, _VP(src_ptr), _VP(dst_ptr)))

    def launch_count(self) -> int:
        n = ctypes.c_int64()
        _check("pihm_gpu_launch_count", self.lib.pihm_gpu_launch_count(self.h, ctypes.byref(n)))
        return n.value

    def set_profiling(self, on: bool):
        _check("pihm_gpu_set_profiling", self.lib.pihm_gpu_set_profiling(self.h, int(on)))

    KERNEL_NAMES = ("k_elem_prep", "k_elem_grad", "k_elem_main", "k_river", "k_finish",
                    "k_edge", "k_permute", "unused")

    def kernel_times(self):
        ms = np.zeros(8)
        calls = np.zeros(8, np.int64)
        _check("pihm_gpu_kernel_times", self.lib.pihm_gpu_kernel_times(
            self.h, f64p(ms), calls.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), 8))
        return {self.KERNEL_NAMES[k]: (float(ms[k]), int(calls[k])) for k in range(8) if calls[k]}

    def fluxes(self):
        ne, nr = self.ws.nelem, self.ws.nriver
        out = dict(ovlflow=np.zeros(3 * ne), subsurf=np.zeros(3 * ne), infil=np.zeros(ne),
                   rechg=np.zeros(ne), et_split=np.zeros(5 * ne), rivflow=np.zeros(11 * nr))
        _check("pihm_gpu_get_fluxes", self.lib.pihm_gpu_get_fluxes(self.h, *(f64p(out[k]) for k in (
            "ovlflow", "subsurf", "infil", "rechg", "et_split", "rivflow"))))
        return out
