"""ctypes binding of the BDF integrator (include/pihm_bdf.h) and the PIHM
model-step loop around it.

`run_steps` restates the reference's per-step driver (src/main.c:217-254,
src/pihm.c:7-187, src/ode.c:413-661): per model step it applies the step's
forcing, sets the stop time to the end of the step and integrates to it
(SolveCVode), applies the post-step update (Summary) and adapts the maximum
step from the step's Newton statistics (AdjCVodeMaxStep).  It is written
against a small backend so that the same loop drives the GPU library (device
N_Vectors, pihm_gpu_ode) and, in the tests, the CPU restatement.
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

from . import capi

_VP = ctypes.c_void_p
_D = ctypes.c_double


class BdfStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_long) for n in ("nst", "nfe", "nni", "ncfn", "netf", "nli", "nfes",
                                             "njtimes", "ncfl", "nor")] + [
        ("qlast", ctypes.c_int), ("qcur", ctypes.c_int), ("hlast", _D), ("hcur", _D), ("tcur", _D)]


RHS_FN = ctypes.CFUNCTYPE(ctypes.c_int, _D, _VP, _VP, _VP)


def _bind(lib):
    sig = {
        "pihm_bdf_create": ([], _VP),
        "pihm_bdf_init": ([_VP, _VP, _D, _VP], ctypes.c_int),
        "pihm_bdf_reinit": ([_VP, _D, _VP], ctypes.c_int),
        "pihm_bdf_ss_tolerances": ([_VP, _D, _D], ctypes.c_int),
        "pihm_bdf_set_user_data": ([_VP, _VP], ctypes.c_int),
        "pihm_bdf_set_init_step": ([_VP, _D], ctypes.c_int),
        "pihm_bdf_set_max_step": ([_VP, _D], ctypes.c_int),
        "pihm_bdf_set_max_num_steps": ([_VP, ctypes.c_long], ctypes.c_int),
        "pihm_bdf_set_stab_lim_det": ([_VP, ctypes.c_int], ctypes.c_int),
        "pihm_bdf_set_stop_time": ([_VP, _D], ctypes.c_int),
        "pihm_bdf_set_deferred_scalars": ([_VP, ctypes.c_int], ctypes.c_int),
        "pihm_bdf_get_deferred_scalars": ([_VP], ctypes.c_int),
        "pihm_bdf_set_op_timing": ([_VP, ctypes.c_int], ctypes.c_int),
        "pihm_bdf_get_op_times": ([_VP, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)],
                                  ctypes.c_int),
        "pihm_bdf_solve": ([_VP, _D, _VP, ctypes.POINTER(_D)], ctypes.c_int),
        "pihm_bdf_get_stats": ([_VP, ctypes.POINTER(BdfStats)], ctypes.c_int),
        "pihm_bdf_free": ([_VP], None),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib


@dataclasses.dataclass
class StepControl:
    """The reference's solver controls (ctrl_struct, src/read_para.c:23-108)."""
    stepsize: int = 60
    reltol: float = 1e-4
    abstol: float = 1e-5
    initstep: float = 5e-5
    nncfn: float = 0.0     # NUM_NONCOV_FAIL
    nnimax: float = 3.0    # MAX_NONLIN_ITER
    nnimin: float = 1.0    # MIN_NONLIN_ITER
    decr: float = 1.2      # DECR_FACTOR
    incr: float = 1.2      # INCR_FACTOR
    stmin: float = 1.0     # MIN_MAXSTEP
    mxstep: int = 0        # internal steps per model step; 0 = 10 * stepsize (src/ode.c:497)


class Bdf:
    """One integrator instance (pihm_bdf)."""

    def __init__(self):
        self.lib = _bind(capi.load())
        self.h = self.lib.pihm_bdf_create()

    def close(self):
        if getattr(self, "h", None):
            self.lib.pihm_bdf_free(self.h)
            self.h = None

    __del__ = close

    def check(self, name, rc):
        if rc < 0:
            raise RuntimeError(f"{name} returned {rc}")
        return rc

    def stats(self) -> BdfStats:
        s = BdfStats()
        self.check("pihm_bdf_get_stats", self.lib.pihm_bdf_get_stats(self.h, ctypes.byref(s)))
        return s


def run_steps(backend, ctrl: StepControl, nsteps: int, forcing, record_every: int = 0,
              outlet: int | None = None, water_balance: bool = False, deferred_scalars: int | None = None,
              op_timing: bool = False):
    """The reference's model-step loop over `backend`, from t = 0.

    backend provides: y (N_Vector handle of the state), rhs (C function
    pointer), user_data, set_forcing(k), post_step(), read_state() ->
    numpy (reference order), outlet_flux(outlet) -> float.
    forcing(k) is called as backend.set_forcing(k) before step k.
    water_balance: record backend.water_balance(dt) -> (sources, sinks,
    storage) after every step (PrintWaterBal, src/print.c:337-542).
    deferred_scalars: pihm_bdf_set_deferred_scalars (None keeps the
    library's default: GMRES scalars kept on the device for device vectors
    with pihm_gpu_ode; the same solution either way).
    op_timing: record the host time inside the integrator's operations
    (pihm_bdf_set_op_timing), returned as op_ms / op_calls.
    Returns dict(states=[...], outlet=[...], stats=BdfStats, wb=[nsteps][3]).
    """
    bdf = Bdf()
    lib = bdf.lib
    bdf.check("init", lib.pihm_bdf_init(bdf.h, backend.rhs, 0.0, backend.y))
    bdf.check("tol", lib.pihm_bdf_ss_tolerances(bdf.h, ctrl.reltol, ctrl.abstol))
    bdf.check("ud", lib.pihm_bdf_set_user_data(bdf.h, backend.user_data))
    bdf.check("h0", lib.pihm_bdf_set_init_step(bdf.h, ctrl.initstep))
    bdf.check("stald", lib.pihm_bdf_set_stab_lim_det(bdf.h, 1))
    if deferred_scalars is not None:
        bdf.check("deferred", lib.pihm_bdf_set_deferred_scalars(bdf.h, int(deferred_scalars)))
    if op_timing:
        bdf.check("timing", lib.pihm_bdf_set_op_timing(bdf.h, 1))
    maxstep = float(ctrl.stepsize)
    bdf.check("hmax", lib.pihm_bdf_set_max_step(bdf.h, maxstep))
    bdf.check("mxstep", lib.pihm_bdf_set_max_num_steps(bdf.h, ctrl.mxstep or ctrl.stepsize * 10))
    states, qout, wb = [], [], []
    nst0 = ncfn0 = nni0 = 0
    tret = _D()
    for k in range(nsteps):
        forcing(k)
        tout = float((k + 1) * ctrl.stepsize)
        bdf.check("tstop", lib.pihm_bdf_set_stop_time(bdf.h, tout))
        bdf.check("solve", lib.pihm_bdf_solve(bdf.h, tout, backend.y, ctypes.byref(tret)))
        backend.post_step()
        # AdjCVodeMaxStep, src/ode.c:601-661
        st = bdf.stats()
        nsteps_d = float(st.nst - nst0)
        nfails = float(st.ncfn - ncfn0) / nsteps_d
        niters = float(st.nni - nni0) / nsteps_d
        if nfails > ctrl.nncfn or niters >= ctrl.nnimax:
            maxstep /= ctrl.decr
        if nfails == 0.0 and niters <= ctrl.nnimin:
            maxstep *= ctrl.incr
        maxstep = maxstep if maxstep < ctrl.stepsize else float(ctrl.stepsize)
        maxstep = maxstep if maxstep > ctrl.stmin else ctrl.stmin
        bdf.check("hmax", lib.pihm_bdf_set_max_step(bdf.h, maxstep))
        nst0, ncfn0, nni0 = st.nst, st.ncfn, st.nni
        if outlet is not None:
            qout.append(backend.outlet_flux(outlet))
        if water_balance:
            wb.append(backend.water_balance(ctrl.stepsize))
        if record_every and (k + 1) % record_every == 0:
            states.append(backend.read_state())
    out = dict(states=np.array(states), outlet=np.array(qout), stats=bdf.stats(), wb=np.array(wb),
               deferred_scalars=lib.pihm_bdf_get_deferred_scalars(bdf.h))
    if op_timing:
        ms, n = (ctypes.c_double * 3)(), (ctypes.c_int64 * 3)()
        bdf.check("times", lib.pihm_bdf_get_op_times(bdf.h, ms, n))
        out["op_ms"] = dict(zip(("elementwise", "reduction", "rhs"), list(ms)))
        out["op_calls"] = dict(zip(("elementwise", "reduction", "rhs"), list(n)))
    bdf.close()
    return out
