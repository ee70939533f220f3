"""Backends of pihm_gpu.solver.run_steps for the tests.

OracleBackend  the CPU restatement of the right-hand side (oracle/) over host
               N_Vectors restating the serial vector (oracle/nvector_host.c):
               test infrastructure, to compare the integrator with the
               reference's CVODE on the CPU.
GpuBackend     the product path: device N_Vector, pihm_gpu_ode, the
               post-step update on the device.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_VP = ctypes.c_void_p


def step_forcing(ws, nsteps, stepsize=60, seed=2):
    import pihm_gpu.watershed as W
    hours = (nsteps * stepsize + 3599) // 3600
    p, e, t = W.hourly_forcing(ws, hours, seed=seed)
    k = (np.arange(nsteps) * stepsize) // 3600
    return p[k].copy(), e[k].copy(), t[k].copy()


class OracleBackend:
    def __init__(self, ws, y0, pcp, edir, ett):
        from oracle import Oracle
        self.model = Oracle(ws)
        lib = self.model.lib
        lib.oracle_nv_make.restype = _VP
        lib.oracle_nv_make.argtypes = [ctypes.c_long, _VP]
        lib.oracle_nv_destroy.argtypes = [_VP]
        self.lib = lib
        self.ws = ws
        self.yarr = np.ascontiguousarray(y0, np.float64).copy()
        self.y = lib.oracle_nv_make(self.yarr.size, self.yarr.ctypes.data)
        self.rhs = ctypes.cast(lib.oracle_cvrhs, _VP)
        self.user_data = _VP(self.model.h)
        self.pcp, self.edir, self.ett = pcp, edir, ett
        self.model.set_ws0_surf(self.yarr[:ws.nelem])

    def set_forcing(self, k):
        ne = self.ws.nelem
        self.model.set_forcing(np.full(ne, self.pcp[k]), np.full(ne, self.edir[k]),
                               np.full(ne, self.ett[k]))

    def post_step(self):
        self.model.post_step(self.yarr)

    def read_state(self):
        return self.yarr.copy()

    def outlet_flux(self, s):
        return float(self.model.fluxes()["rivflow"][11 * s + 1])

    def close(self):
        if self.y:
            self.lib.oracle_nv_destroy(self.y)
            self.y = None


class GpuBackend:
    def __init__(self, ws, y0, pcp, edir, ett, order=1):
        from pihm_gpu import nvector
        from pihm_gpu.capi import GpuRhs
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

    def outlet_flux(self, s):
        return float(self.g.fluxes()["rivflow"][11 * s + 1])

    def close(self):
        for v in (self.y, self.scratch):
            if v:
                self.lib.N_VDestroy_PihmGpu(v)
        self.y = self.scratch = None
