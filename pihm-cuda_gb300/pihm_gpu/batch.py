"""ctypes binding of the batch engine (include/pihm_batch.h): many watersheds
integrated together on one GPU, each bit-for-bit as the single-watershed
path would integrate it alone."""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

from . import capi
from .meshdesc import MeshDesc, f64p
from .solver import BdfStats, StepControl

_VP = ctypes.c_void_p
_D = ctypes.c_double
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_F64P = ctypes.POINTER(ctypes.c_double)

RUNNING, DONE, FAILED = 0, 1, 2


class BatchLimits(ctypes.Structure):
    _fields_ = [("max_elem", _I64), ("max_river", _I64), ("max_edge", _I64), ("max_record", _I64),
                ("max_systems", _I32)]


class StepControlC(ctypes.Structure):
    _fields_ = [(n, _D) for n in ("stepsize", "reltol", "abstol", "initstep", "nncfn", "nnimax",
                                  "nnimin", "decr", "incr", "stmin")] + [("mxstep", ctypes.c_long)]

    @staticmethod
    def of(ctrl: StepControl) -> "StepControlC":
        c = StepControlC()
        for f in dataclasses.fields(ctrl):
            setattr(c, f.name, getattr(ctrl, f.name))
        return c


class BatchJob(ctypes.Structure):
    _fields_ = [("mesh", ctypes.POINTER(MeshDesc)), ("elem_bc", _F64P), ("river_bc", _F64P),
                ("y0", _F64P), ("ctrl", StepControlC), ("nsteps", _I32), ("pcpdrp", _F64P),
                ("edir", _F64P), ("ett", _F64P), ("outlet", _I32),
                ("deck", _VP), ("land", _VP), ("forcing", _VP), ("cmc0", _F64P), ("sneqv0", _F64P),
                ("start", _I64), ("lsm_step", _I64),
                ("noah", _VP), ("noah_state", _VP), ("noah_forcing", _VP), ("noah_nforcing", _I32),
                ("noah_lsm_step", _D)]


class BatchInfo(ctypes.Structure):
    _fields_ = [(n, _I64) for n in ("rounds", "rhs_rounds", "launches", "elem_used", "elem_hwm",
                                    "resident")] + [
        (n, _D) for n in ("host_ms", "wait_ms", "program_ms", "rhs_ms")] + [
        ("program_variant", _I32), ("tuning", _I32), ("rhs_shape", _I32), ("rhs_tuning", _I32)]


class ServeRecord(ctypes.Structure):
    _fields_ = [("status", _I32), ("solver_rc", _I32), ("nelem", _I32), ("t_arrival", _D),
                ("t_admit", _D), ("t_done", _D)]


def _job(ws, y0, ctrl, pcp, edir, ett, outlet, elem_bc, river_bc):
    """A BatchJob and the arrays it points at (keep both alive)."""
    keep = dict(desc=MeshDesc.from_arrays(ws.nelem, ws.nriver, ws.arrays),
                y0=np.ascontiguousarray(y0, np.float64), pcp=np.ascontiguousarray(pcp, np.float64),
                edir=np.ascontiguousarray(edir, np.float64), ett=np.ascontiguousarray(ett, np.float64),
                ebc=None if elem_bc is None else np.ascontiguousarray(elem_bc, np.float64),
                rbc=None if river_bc is None else np.ascontiguousarray(river_bc, np.float64))
    job = BatchJob()
    job.mesh = ctypes.pointer(keep["desc"])
    job.elem_bc = f64p(keep["ebc"])
    job.river_bc = f64p(keep["rbc"])
    job.y0 = f64p(keep["y0"])
    job.ctrl = StepControlC.of(ctrl)
    job.nsteps = len(keep["pcp"])
    job.pcpdrp, job.edir, job.ett = f64p(keep["pcp"]), f64p(keep["edir"]), f64p(keep["ett"])
    job.outlet = outlet
    return job, keep


def _deck_job(deck, nsteps: int | None, outlet: int):
    """A BatchJob running an input deck (pihm_gpu.deck.Deck) with its own
    forcing -- boundary series every model step, the land-surface step every
    LSM_STEP -- as pihm_gpu.single.run_deck does; and what it points at
    (keep both alive, and the deck, while the watershed runs)."""
    from .single import step_control
    ctrl = deck.control()
    ws = deck.watershed()
    sc = step_control(ctrl)
    start, stepsize = int(ctrl.start), int(ctrl.step["stepsize"])
    n = nsteps if nsteps is not None else (int(ctrl.end) - start) // stepsize
    land = deck.land()
    p, fs = land.structs()
    cmc, sneqv = deck.initial_storage()
    zero = np.zeros(0)
    job, keep = _job(ws, deck.initial_state(), sc, zero, zero, zero, outlet, None, None)
    keep.update(land=land, p=p, fs=fs, cmc=np.ascontiguousarray(cmc), sneqv=np.ascontiguousarray(sneqv), ws=ws,
                deck=deck, surf_mode=ctrl.surf_mode, riv_mode=ctrl.riv_mode)
    job.nsteps = n
    job.pcpdrp = job.edir = job.ett = None
    job.deck = deck.h
    job.land = ctypes.cast(ctypes.pointer(p), _VP)
    job.forcing = ctypes.cast(ctypes.pointer(fs), _VP)
    job.cmc0, job.sneqv0 = f64p(keep["cmc"]), f64p(keep["sneqv"])
    job.start = start
    job.lsm_step = int(ctrl.lsm_step)
    return job, keep


def _noah_job(ws, y0, ctrl, params: dict, state: dict, forcings, lsm_step: float, nsteps: int, outlet: int):
    """A BatchJob running Flux-PIHM with Noah on the device: params, state
    (pihm_gpu.noah.synthetic_noah's dicts, reference order) and one forcing
    dict (pihm_gpu.noah.forcing) per land-surface step of lsm_step seconds;
    and what it points at (keep both alive while the watershed runs)."""
    from . import noah as N
    zero = np.zeros(0)
    job, keep = _job(ws, y0, ctrl, zero, zero, zero, outlet, None, None)
    ps, kp = N.params_struct(params)
    ss, ks = N.state_struct(state)
    fs = (N.NoahForcing * len(forcings))()
    kf = []
    for k, f in enumerate(forcings):
        one, keep_one = N.forcing_struct(f)
        fs[k] = one
        kf.append(keep_one)
    keep.update(noah=(ps, kp, ss, ks, fs, kf), ws=ws)
    job.nsteps = int(nsteps)
    job.pcpdrp = job.edir = job.ett = None
    job.noah = ctypes.cast(ctypes.pointer(ps), _VP)
    job.noah_state = ctypes.cast(ctypes.pointer(ss), _VP)
    job.noah_forcing = ctypes.cast(fs, _VP)
    job.noah_nforcing = len(forcings)
    job.noah_lsm_step = float(lsm_step)
    return job, keep


def _bind(lib):
    sig = {
        "pihm_batch_create": ([ctypes.POINTER(BatchLimits), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(_VP)], ctypes.c_int),
        "pihm_batch_destroy": ([_VP], None),
        "pihm_batch_set_stream": ([_VP, _VP], ctypes.c_int),
        "pihm_batch_set_rhs_gate": ([_VP, _D], ctypes.c_int),
        "pihm_batch_add": ([_VP, ctypes.POINTER(BatchJob), ctypes.POINTER(_I32)], ctypes.c_int),
        "pihm_batch_step": ([_VP, _I32, ctypes.POINTER(_I32)], ctypes.c_int),
        "pihm_batch_add_many": ([_VP, ctypes.POINTER(BatchJob), _I32, _I32, ctypes.POINTER(_I32),
                                 ctypes.POINTER(_I32)], ctypes.c_int),
        "pihm_batch_poll": ([_VP, _I32, ctypes.POINTER(_I32), ctypes.POINTER(_I32)], ctypes.c_int),
        "pihm_batch_result": ([_VP, _I32, _F64P, _F64P, ctypes.POINTER(BdfStats), ctypes.POINTER(_I32)],
                              ctypes.c_int),
        "pihm_batch_release": ([_VP, _I32], ctypes.c_int),
        "pihm_batch_get_info": ([_VP, ctypes.POINTER(BatchInfo)], ctypes.c_int),
        "pihm_batch_set_profiling": ([_VP, ctypes.c_int], ctypes.c_int),
        "pihm_batch_set_program_variant": ([_VP, _I32], ctypes.c_int),
        "pihm_batch_set_rhs_shape": ([_VP, _I32], ctypes.c_int),
        "pihm_batch_arena_bytes": ([ctypes.POINTER(BatchLimits), ctypes.POINTER(_I64)], ctypes.c_int),
        "pihm_batch_limits_for_memory": ([_I64, _D, _D, _D, _I32, ctypes.POINTER(BatchLimits)], ctypes.c_int),
        "pihm_serve_submit": ([_VP, ctypes.POINTER(BatchJob), _D, ctypes.POINTER(_I32)], ctypes.c_int),
        "pihm_serve_run": ([_VP, _I32], ctypes.c_int),
        "pihm_serve_record_get": ([_VP, _I32, ctypes.POINTER(ServeRecord)], ctypes.c_int),
        "pihm_serve_result": ([_VP, _I32, _F64P, _F64P, ctypes.POINTER(BdfStats)], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib


def arena_bytes(limits: BatchLimits) -> int:
    """Device memory an arena with these limits takes."""
    lib = _bind(capi.load())
    n = _I64()
    capi._check("pihm_batch_arena_bytes", lib.pihm_batch_arena_bytes(ctypes.byref(limits), ctypes.byref(n)))
    return n.value


def limits_for_memory(nbytes: int, rivers_per_elem: float = 0.03, edges_per_elem: float = 1.6,
                      records_per_elem: float = 0.01, max_systems: int = 256) -> BatchLimits:
    """The largest arena that fits in nbytes of device memory (admission is
    then gated by that memory)."""
    lib = _bind(capi.load())
    lim = BatchLimits()
    capi._check("pihm_batch_limits_for_memory", lib.pihm_batch_limits_for_memory(
        int(nbytes), float(rivers_per_elem), float(edges_per_elem), float(records_per_elem), int(max_systems),
        ctypes.byref(lim)))
    return lim


def limits_for(watersheds, nsteps: int, slack: float = 1.0) -> BatchLimits:
    """Arena capacity holding the given watersheds at once (times slack)."""
    ne = sum(w.nelem for w in watersheds)
    nr = sum(w.nriver for w in watersheds)
    lim = BatchLimits()
    lim.max_elem = int(ne * slack) + 1
    lim.max_river = int(nr * slack) + 1
    lim.max_edge = int(1.6 * ne * slack) + 16
    lim.max_record = int(nsteps * len(watersheds) * slack) + 1
    lim.max_systems = max(1, int(len(watersheds) * slack))
    return lim


class Batch:
    """A batch engine instance (pihm_batch)."""

    def __init__(self, limits: BatchLimits, surf_mode: int = 2, riv_mode: int = 2,
                 order: int = capi.ORDER_RCM):
        self.lib = _bind(capi.load())
        h = _VP()
        capi._check("pihm_batch_create", self.lib.pihm_batch_create(
            ctypes.byref(limits), surf_mode, riv_mode, order, ctypes.byref(h)))
        self.h = h
        self.jobs = {}
        self.requests = {}
        self.keep = {}  # what deck jobs point at, while they run

    def close(self):
        if getattr(self, "h", None):
            self.lib.pihm_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def add(self, ws, y0, ctrl: StepControl, pcp, edir, ett, outlet: int = -1,
            elem_bc=None, river_bc=None) -> int | None:
        """Admit a watershed; None when the arena has no room for it now."""
        job, keep = _job(ws, y0, ctrl, pcp, edir, ett, outlet, elem_bc, river_bc)
        i = _I32()
        rc = self.lib.pihm_batch_add(self.h, ctypes.byref(job), ctypes.byref(i))
        if rc == -5:  # PIHM_GPU_ERR_NOMEM: no room now
            return None
        capi._check("pihm_batch_add", rc)
        self.jobs[i.value] = (ws, job.nsteps, outlet)
        return i.value

    def add_deck(self, deck, nsteps: int | None = None, outlet: int = -1) -> int | None:
        """Admit an input deck with its own forcing (boundary series, land-surface
        step), nsteps model steps from START (default: to END); None when the
        arena has no room for it now.  The deck's modes must be the batch's."""
        job, keep = _deck_job(deck, nsteps, outlet)
        i = _I32()
        rc = self.lib.pihm_batch_add(self.h, ctypes.byref(job), ctypes.byref(i))
        if rc == -5:
            return None
        capi._check("pihm_batch_add", rc)
        self.jobs[i.value] = (keep["ws"], job.nsteps, outlet)
        self.keep[i.value] = keep
        return i.value

    def add_noah(self, ws, y0, ctrl: StepControl, params: dict, state: dict, forcings, lsm_step: float,
                 nsteps: int, outlet: int = -1) -> int | None:
        """Admit a Flux-PIHM watershed with Noah on the device (see _noah_job);
        None when the arena has no room for it now."""
        job, keep = _noah_job(ws, y0, ctrl, params, state, forcings, lsm_step, nsteps, outlet)
        i = _I32()
        rc = self.lib.pihm_batch_add(self.h, ctypes.byref(job), ctypes.byref(i))
        if rc == -5:
            return None
        capi._check("pihm_batch_add", rc)
        self.jobs[i.value] = (ws, job.nsteps, outlet)
        self.keep[i.value] = keep
        return i.value

    def add_many(self, cases, threads: int = 16):
        """Admit many cases (dicts with ws, y0, ctrl, pcp, edir, ett, outlet),
        prepared in parallel on host threads; returns their ids (None where a
        case did not fit)."""
        n = len(cases)
        jobs = (BatchJob * n)()
        keeps = []
        for k, c in enumerate(cases):
            job, keep = _job(c["ws"], c["y0"], c["ctrl"], c["pcp"], c["edir"], c["ett"], c.get("outlet", -1),
                             c.get("elem_bc"), c.get("river_bc"))
            jobs[k] = job
            keeps.append(keep)
        ids = (_I32 * n)()
        admitted = _I32()
        rc = self.lib.pihm_batch_add_many(self.h, jobs, n, threads, ids, ctypes.byref(admitted))
        if rc not in (0, -5):
            capi._check("pihm_batch_add_many", rc)
        out = []
        for k, c in enumerate(cases):
            if ids[k] < 0:
                out.append(None)
                continue
            self.jobs[ids[k]] = (c["ws"], jobs[k].nsteps, jobs[k].outlet)
            out.append(ids[k])
        return out

    def set_profiling(self, on: bool):
        capi._check("pihm_batch_set_profiling", self.lib.pihm_batch_set_profiling(self.h, int(on)))

    def set_program_variant(self, variant: int):
        capi._check("pihm_batch_set_program_variant", self.lib.pihm_batch_set_program_variant(self.h, variant))

    def set_rhs_shape(self, shape: int):
        """Force the element kernel's block shape (0..2), or -1 to let the
        engine time them (the default)."""
        capi._check("pihm_batch_set_rhs_shape", self.lib.pihm_batch_set_rhs_shape(self.h, shape))

    def set_rhs_gate(self, gate: float):
        capi._check("pihm_batch_set_rhs_gate", self.lib.pihm_batch_set_rhs_gate(self.h, gate))

    def step(self, max_rounds: int = 0) -> int:
        n = _I32()
        capi._check("pihm_batch_step", self.lib.pihm_batch_step(self.h, max_rounds, ctypes.byref(n)))
        return n.value

    def poll(self, i: int):
        st, rc = _I32(), _I32()
        capi._check("pihm_batch_poll", self.lib.pihm_batch_poll(self.h, i, ctypes.byref(st), ctypes.byref(rc)))
        return st.value, rc.value

    def result(self, i: int):
        ws, nsteps, outlet = self.jobs[i]
        y = np.zeros(ws.neq)
        q = np.zeros(nsteps if outlet >= 0 else 0)
        stats = BdfStats()
        done = _I32()
        capi._check("pihm_batch_result", self.lib.pihm_batch_result(
            self.h, i, f64p(y), f64p(q) if q.size else None, ctypes.byref(stats), ctypes.byref(done)))
        return dict(y=y, outlet=q, stats=stats, steps_done=done.value)

    def release(self, i: int):
        capi._check("pihm_batch_release", self.lib.pihm_batch_release(self.h, i))
        self.jobs.pop(i, None)

    def info(self) -> BatchInfo:
        inf = BatchInfo()
        capi._check("pihm_batch_get_info", self.lib.pihm_batch_get_info(self.h, ctypes.byref(inf)))
        return inf

    # ---- serving ----------------------------------------------------------
    def submit(self, ws, y0, ctrl: StepControl, pcp, edir, ett, arrival: float, outlet: int = -1,
               elem_bc=None, river_bc=None) -> int:
        """Queue a request arriving `arrival` seconds after serve() starts."""
        job, keep = _job(ws, y0, ctrl, pcp, edir, ett, outlet, elem_bc, river_bc)
        t = _I32()
        capi._check("pihm_serve_submit", self.lib.pihm_serve_submit(self.h, ctypes.byref(job), float(arrival),
                                                                     ctypes.byref(t)))
        self.requests[t.value] = (ws, job.nsteps, outlet)
        return t.value

    def submit_deck(self, deck, arrival: float, nsteps: int | None = None, outlet: int = -1) -> int:
        """Queue an input deck with its own forcing arriving `arrival` seconds
        after serve() starts."""
        job, keep = _deck_job(deck, nsteps, outlet)
        t = _I32()
        capi._check("pihm_serve_submit", self.lib.pihm_serve_submit(self.h, ctypes.byref(job), float(arrival),
                                                                     ctypes.byref(t)))
        self.requests[t.value] = (keep["ws"], job.nsteps, outlet)
        self.keep[("serve", t.value)] = keep
        return t.value

    def submit_noah(self, ws, y0, ctrl: StepControl, params: dict, state: dict, forcings, lsm_step: float,
                    nsteps: int, arrival: float, outlet: int = -1) -> int:
        """Queue a Flux-PIHM request (see _noah_job) arriving `arrival` seconds
        after serve() starts."""
        job, keep = _noah_job(ws, y0, ctrl, params, state, forcings, lsm_step, nsteps, outlet)
        t = _I32()
        capi._check("pihm_serve_submit", self.lib.pihm_serve_submit(self.h, ctypes.byref(job), float(arrival),
                                                                     ctypes.byref(t)))
        self.requests[t.value] = (ws, job.nsteps, outlet)
        self.keep[("serve", t.value)] = keep
        return t.value

    def serve(self, workers: int = 4):
        """Serve every submitted request (returns when all are finished)."""
        capi._check("pihm_serve_run", self.lib.pihm_serve_run(self.h, workers))

    def record(self, ticket: int) -> ServeRecord:
        r = ServeRecord()
        capi._check("pihm_serve_record_get", self.lib.pihm_serve_record_get(self.h, ticket, ctypes.byref(r)))
        return r

    def served(self, ticket: int):
        ws, nsteps, outlet = self.requests[ticket]
        y = np.zeros(ws.neq)
        q = np.zeros(nsteps if outlet >= 0 else 0)
        stats = BdfStats()
        capi._check("pihm_serve_result", self.lib.pihm_serve_result(
            self.h, ticket, f64p(y), f64p(q) if q.size else None, ctypes.byref(stats)))
        return dict(y=y, outlet=q, stats=stats)
