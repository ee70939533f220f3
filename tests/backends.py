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
    def __init__(self, ws, y0, pcp, edir, ett, omp: bool = False):
        from oracle import Oracle
        self.model = Oracle(ws, omp=omp)
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
        self.k = k
        self.model.set_forcing(np.full(ne, self.pcp[k]), np.full(ne, self.edir[k]),
                               np.full(ne, self.ett[k]))

    def post_step(self):
        self.model.post_step(self.yarr)

    def read_state(self):
        return self.yarr.copy()

    def outlet_flux(self, s):
        return float(self.model.fluxes()["rivflow"][11 * s + 1])

    def water_balance(self, dt):
        """PrintWaterBal's sums (src/print.c:337-542) in its summation order
        (np.cumsum adds left to right), no canopy or snow stores."""
        a, ne, nr = self.ws.arrays, self.ws.nelem, self.ws.nriver
        y, k = self.yarr, self.k
        area = a["area"]
        src = np.cumsum(self.pcp[k] * area * dt)[-1]
        e_snk = (self.edir[k] + self.ett[k] + 0.0) * area * dt
        rivflow = self.model.fluxes()["rivflow"].reshape(nr, 11)[:, 1]
        r_snk = (rivflow * dt)[a["down"] < 0]
        snk = np.cumsum(np.concatenate([e_snk, r_snk]))[-1]
        e_strg = ((0.0 + 0.0 + y[:ne]) + (y[ne:2 * ne] + y[2 * ne:3 * ne]) * a["porosity"]) * area
        r_strg = (y[3 * ne:3 * ne + nr] + y[3 * ne + nr:] * a["riv_porosity"]) * a["riv_area"]
        strg = np.cumsum(np.concatenate([e_strg, r_strg]))[-1]
        return float(src), float(snk), float(strg)

    def close(self):
        if self.y:
            self.lib.oracle_nv_destroy(self.y)
            self.y = None


# the product's single-watershed path (device N_Vector, pihm_gpu_ode, the
# post-step update on the device)
from pihm_gpu.single import GpuWatershed as GpuBackend  # noqa: E402,F401


class OracleDeckBackend(OracleBackend):
    """An input deck on the CPU restatements: the right-hand side
    (oracle/pihm_oracle.c) and the land-surface step (oracle/land_oracle.c),
    driven the way the reference's main loop drives them
    (src/pihm.c:15-99)."""

    def __init__(self, deck):
        from oracle import OracleLand
        self.deck = deck
        self.ctrl = deck.control()
        ws = deck.watershed()
        super().__init__(ws, deck.initial_state(), None, None, None)
        self.land = OracleLand(deck.land(), ws)
        self.land.set_state(*deck.initial_storage())
        self.has_bc = bool(np.any(ws.arrays["bc_type"]) or np.any(ws.arrays["riverbc_type"]))
        self.start = int(self.ctrl.start)
        self.stepsize = int(self.ctrl.step["stepsize"])
        self.lsm_step = int(self.ctrl.lsm_step)

    def set_forcing(self, k):
        ne = self.ws.nelem
        t = self.start + k * self.stepsize
        self.k = k
        if self.has_bc:
            e, r = self.deck.bc(t)
            self.model.set_bc(e, r)
        if (t - self.start) % self.lsm_step == 0:
            y = self.yarr
            assert self.land.step(t, float(self.lsm_step), y[ne:2 * ne], y[2 * ne:3 * ne]) == 0
            self.model.set_forcing(self.land.get("pcpdrp"), self.land.get("edir"), self.land.get("ett"))

    def water_balance(self, dt):
        """PrintWaterBal's sums (src/print.c:337-542) in its summation order,
        with the land-surface model's precipitation, canopy evaporation,
        canopy storage and snow."""
        a, ne, nr = self.ws.arrays, self.ws.nelem, self.ws.nriver
        y = self.yarr
        area = a["area"]
        f = {k: self.land.get(k) for k in ("prcp", "edir", "ett", "ec", "cmc", "sneqv")}
        src = np.cumsum(f["prcp"] * area * dt)[-1]
        e_snk = (f["edir"] + f["ett"] + f["ec"]) * area * dt
        rivflow = self.model.fluxes()["rivflow"].reshape(nr, 11)[:, 1]
        r_snk = (rivflow * dt)[a["down"] < 0]
        snk = np.cumsum(np.concatenate([e_snk, r_snk]))[-1]
        e_strg = ((f["cmc"] + f["sneqv"] + y[:ne]) + (y[ne:2 * ne] + y[2 * ne:3 * ne]) * a["porosity"]) * area
        r_strg = (y[3 * ne:3 * ne + nr] + y[3 * ne + nr:] * a["riv_porosity"]) * a["riv_area"]
        strg = np.cumsum(np.concatenate([e_strg, r_strg]))[-1]
        return float(src), float(snk), float(strg)
