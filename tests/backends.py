"""Backends of pihm_gpu.solver.run_steps for the tests.

OracleBackend  the CPU restatement of the right-hand side (oracle/) over host
               N_Vectors restating the serial vector (oracle/nvector_host.c):
               test infrastructure, to compare the integrator with the
               reference's CVODE on the CPU.
GpuBackend     the product path (pihm_gpu.single.GpuWatershed).
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


# the product's single-watershed path (device N_Vector, pihm_gpu_ode, the
# post-step update on the device)
from pihm_gpu.single import GpuWatershed as GpuBackend  # noqa: E402,F401
