"""The single-watershed GPU path as a model-step backend (pihm_gpu.solver.run_steps):
device N_Vectors (N_VNew_PihmGpu), the drop-in right-hand side pihm_gpu_ode,
the post-step update on the device.  This is the plain path one watershed at
a time; the batch engine (pihm_gpu.batch) reproduces it bit for bit.

`DeckWatershed` / `run_deck` run an input deck the way the reference's main
loop does (src/main.c:217-254, src/pihm.c:7-187): the deck's boundary series
every model step, the land-surface step on the device (forcing interpolation,
interception, snow, evapotranspiration; include/pihm_land.h) every LSM_STEP,
then the integration to the end of the step, Summary and AdjCVodeMaxStep."""
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

    def device_state(self) -> int:
        """Device pointer of the state (internal order)."""
        return self.lib.N_VGetDeviceArrayPointer_PihmGpu(self.y)

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


class NoahWatershed(GpuWatershed):
    """Flux-PIHM on the device: the model-step loop of the reference built
    with _NOAH_ (src/pihm.c:21-123) -- every land-surface step the step's
    forcing and Noah() (include/pihm_noah.h), then the integration to the end
    of each model step, Summary and NoahHydrol -- with Noah's state and the
    right-hand side's Noah inputs kept on the device.  forcing(hour) returns
    the per-element forcing dict of pihm_gpu.noah.forcing for the land-surface
    step that starts at that hour; lsm_step is the land-surface step (s)."""

    def __init__(self, ws, y0, params: dict, state: dict, forcing, lsm_step: float = 3600.0, order=1):
        zero = np.zeros(1)
        super().__init__(ws, y0, zero, zero, zero, order=order)
        self.g.noah_init(params, state)
        self.g.noah_begin(self.device_state())
        self.forcing = forcing
        self.lsm_step = float(lsm_step)
        self.noah_steps = 0

    def set_forcing(self, k):
        t = k * self.ws.stepsize
        if t % self.lsm_step == 0:
            self.g.noah_set_forcing(self.forcing(int(t // 3600)))
            self.g.noah_step(self.lsm_step)
            self.noah_steps += 1

    def post_step(self):
        assert self.lib.pihm_gpu_summary(self.g.h, self.y) == 0
        self.g.noah_post_step(self.device_state(), float(self.ws.stepsize))


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


class DeckWatershed(GpuWatershed):
    """An input deck (pihm_gpu.deck.Deck) as a model-step backend: its mesh,
    initial state, boundary series and land-surface model on the GPU."""

    def __init__(self, deck, order=1):
        self.deck = deck
        self.ctrl = deck.control()
        ws = deck.watershed()
        super().__init__(ws, deck.initial_state(), None, None, None, order=order)
        self.g.land_init(deck.land())
        self.g.land_set_state(*deck.initial_storage())
        self.has_bc = bool(np.any(ws.arrays["bc_type"]) or np.any(ws.arrays["riverbc_type"]))
        self.start = int(self.ctrl.start)
        self.stepsize = int(self.ctrl.step["stepsize"])
        self.lsm_step = int(self.ctrl.lsm_step)

    def set_forcing(self, k):
        """The forcing of model step k (src/pihm.c:15-66): ApplyBc at t, and at
        every LSM_STEP the land-surface step over LSM_STEP seconds."""
        t = self.start + k * self.stepsize
        if self.has_bc:
            e, r = self.deck.bc(t)
            self.g.set_bc(e, r)
        if (t - self.start) % self.lsm_step == 0:
            self.g.land_step(t, float(self.lsm_step), self.device_state())

    def land(self, field: str) -> np.ndarray:
        return self.g.land_get(field)


def step_control(ctrl):
    """solver.StepControl from a deck's control block."""
    from .solver import StepControl
    sc = StepControl()
    for k in ("stepsize", "reltol", "abstol", "initstep", "nncfn", "nnimax", "nnimin", "decr", "incr", "stmin",
              "mxstep"):
        setattr(sc, k, type(getattr(sc, k))(ctrl.step[k]))
    return sc


def run_deck(deck, nsteps: int | None = None, record_every: int = 0, outlet: int | None = None,
             water_balance: bool = False, order: int = 1):
    """Run a deck on the GPU for nsteps model steps (default: START to END).
    Returns run_steps' dict (states in reference order, outlet flux series,
    integrator counters, water-balance sums)."""
    from .solver import run_steps
    b = DeckWatershed(deck, order=order)
    try:
        n = nsteps if nsteps is not None else (int(b.ctrl.end) - b.start) // b.stepsize
        return run_steps(b, step_control(b.ctrl), n, b.set_forcing, record_every=record_every, outlet=outlet,
                         water_balance=water_balance)
    finally:
        b.close()


def _main(argv=None):
    """python -m pihm_gpu.single: a generated watershed solved on the GPU
    from RelaxIc with hourly synthetic forcing through the plain path; prints
    the wall time and the integrator's counters as one JSON line."""
    import argparse
    import json
    import time

    from . import watershed as W
    from . import workloads as WL
    from .solver import StepControl, run_steps
    ap = argparse.ArgumentParser(prog="python -m pihm_gpu.single")
    ap.add_argument("--nelem", type=int, default=WL.RHS_NELEM)
    ap.add_argument("--nriver", type=int, default=0, help="default: workloads.river_count(nelem)")
    ap.add_argument("--seed", type=int, default=WL.RHS_SEED)
    ap.add_argument("--model-steps", type=int, default=2)
    ap.add_argument("--deferred-scalars", type=int, default=-1, choices=[-1, 0, 1])
    ap.add_argument("--op-timing", action="store_true", help="host time inside the integrator's operations")
    ap.add_argument("--noah", type=int, default=0, metavar="LAYERS",
                    help="Flux-PIHM with Noah on the device, this many soil layers (hourly synthetic forcing)")
    ap.add_argument("--mxstep", type=int, default=0, help="internal steps per model step (0: 10 x stepsize)")
    ap.add_argument("--progress", type=int, default=0, metavar="K",
                    help="print the wall time to stderr every K model steps")
    a = ap.parse_args(argv)
    ws = W.generate(a.nelem, a.nriver or WL.river_count(a.nelem), seed=a.seed)
    if a.noah:
        from . import noah as N
        params, state = N.synthetic_noah(ws, seed=a.seed + 1, nlayers=a.noah)
        m = NoahWatershed(ws, W.relax_state(ws), params, state, lambda h: N.forcing(ws, h, seed=a.seed + 2))
    else:
        pcp, edir, ett = WL.step_forcing(ws, a.model_steps, 60.0, seed=8)
        m = GpuWatershed(ws, W.relax_state(ws), pcp, edir, ett)
        m.g.set_diagnostics(False)
    try:
        import sys
        t = time.perf_counter()
        forcing = m.set_forcing
        if a.progress:
            def forcing(k):
                if k and k % a.progress == 0:
                    print(f"model step {k}: {time.perf_counter() - t:.1f} s", file=sys.stderr, flush=True)
                m.set_forcing(k)
        r = run_steps(m, StepControl(mxstep=a.mxstep), a.model_steps, forcing, deferred_scalars=a.deferred_scalars,
                      op_timing=a.op_timing)
        m.read_state()
        wall = time.perf_counter() - t
    finally:
        m.close()
    s = r["stats"]
    print(json.dumps({"nelem": ws.nelem, "nriver": ws.nriver, "model_steps": a.model_steps, "wall_s": wall,
                      "nst": s.nst, "nfe": s.nfe, "nfes": s.nfes, "nni": s.nni, "nli": s.nli,
                      "deferred_scalars": r["deferred_scalars"],
                      **({"op_ms": r["op_ms"], "op_calls": r["op_calls"]} if a.op_timing else {})}))


if __name__ == "__main__":
    _main()
