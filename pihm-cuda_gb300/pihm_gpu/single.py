"""The single-watershed GPU path as a model-step backend (pihm_gpu.solver.run_steps):
device N_Vectors (N_VNew_PihmGpu), the drop-in right-hand side pihm_gpu_ode,
the post-step update on the device.  This is the plain path one watershed at
a time; the batch engine (pihm_gpu.batch) reproduces it bit for bit."""
from __future__ import annotations

import ctypes

import numpy as np

_VP = ctypes.c_void_p


class GpuWatershed:
    def __init__(self, ws, y0, pcp, edir, ett, order=1):
        from . import nvector
        from .capi import GpuRhs
        self.g = GpuRhs(ws, order=order)
        lib = nvector.load()
        for name, args, res in (("pihm_gpu_ode", [ctypes.c_double, _VP, _VP, _VP], ctypes.c_int),
                                ("pihm_gpu_summary", [_VP, _VP], ctypes.c_int)):
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res
        self.lib = lib
        self.ws = ws
        self.y = lib.N_VNew_PihmGpu(ws.neq, None)
        y_ref = lib.N_VNew_PihmGpu(ws.neq, None)
        y0 = np.ascontiguousarray(y0, np.float64)
        assert lib.N_VCopyFromHost_PihmGpu(y_ref, y0.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
        self.g.to_internal(lib.N_VGetDeviceArrayPointer_PihmGpu(y_ref),
                           lib.N_VGetDeviceArrayPointer_PihmGpu(self.y))
        self.scratch = y_ref
        self.rhs = ctypes.cast(lib.pihm_gpu_ode, _VP)
        self.user_data = self.g.h
        self.pcp, self.edir, self.ett = pcp, edir, ett
        self.g.set_ws0_surf(y0[:ws.nelem])
        self.g.set_diagnostics(True)

    def set_forcing(self, k):
        ne = self.ws.nelem
        self.g.set_forcing(np.full(ne, self.pcp[k]), np.full(ne, self.edir[k]), np.full(ne, self.ett[k]))

    def post_step(self):
        assert self.lib.pihm_gpu_summary(self.g.h, self.y) == 0

    def read_state(self):
        self.g.to_reference(self.lib.N_VGetDeviceArrayPointer_PihmGpu(self.y),
                            self.lib.N_VGetDeviceArrayPointer_PihmGpu(self.scratch))
        out = np.zeros(self.ws.neq)
        assert self.lib.N_VCopyToHost_PihmGpu(self.scratch, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
        return out

    def water_balance(self, dt):
        return self.g.water_balance(self.lib.N_VGetDeviceArrayPointer_PihmGpu(self.y), dt)

    def outlet_flux(self, s):
        return float(self.g.fluxes()["rivflow"][11 * s + 1])

    def close(self):
        for v in (self.y, self.scratch):
            if v:
                self.lib.N_VDestroy_PihmGpu(v)
        self.y = self.scratch = None
        self.g.close()


def solve_alone(case: dict):
    """One watershed through the plain path: final state, outlet series, counters."""
    from .solver import run_steps
    b = GpuWatershed(case["ws"], case["y0"], case["pcp"], case["edir"], case["ett"])
    try:
        n = len(case["pcp"])
        r = run_steps(b, case["ctrl"], n, b.set_forcing, record_every=n, outlet=case["outlet"])
    finally:
        b.close()
    return dict(y=r["states"][-1], outlet=r["outlet"], stats=r["stats"])
