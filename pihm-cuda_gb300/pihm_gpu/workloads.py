"""Synthetic workloads for the batch and serving engines.

batched  many independent watersheds from the generator, element counts
         log-uniform in [lo, hi], each with its own seed (soil, terrain,
         forcing), river segments 100 (n / 1000)^0.826 (the generator's
         1,000-element / 100-segment and 1,000,000-element / 30,000-segment
         cases both follow it).
serving  calibration requests: a generator watershed of lo..hi elements
         (log-uniform) with Ksat (KSATH, KSATV) x U(0.3, 3) and Manning n
         x U(0.5, 2) (the reference's calibration multipliers,
         src/read_calib.c), its own model step, and Poisson arrivals.

Every case starts from the relaxed initial condition (RelaxIc) under its own
hourly rainfall and PET series, held for each model step.
"""
from __future__ import annotations

import dataclasses
import multiprocessing as mp
import os

import numpy as np

from . import watershed as W
from .solver import StepControl


def river_count(nelem: int) -> int:
    return max(4, int(round(100 * (nelem / 1000.0) ** 0.826)))


# The right-hand-side benchmark: one 1,000,000-element / 30,000-segment
# watershed (generator seed 0) evaluated on 100 perturbed states.
RHS_NELEM, RHS_NRIVER, RHS_SEED, RHS_NSTATES = 1_000_000, 30_000, 0, 100


def rhs_base_state(ws) -> np.ndarray:
    """The wet reference state the benchmark's states perturb (reference order)."""
    return W.reference_state(ws, 1)


def rhs_state(base: np.ndarray, k: int) -> np.ndarray:
    """State k of the benchmark set: every storage of `base` x U(0.9, 1.1),
    seeded by k, so every user of the set (both benchmark arms, the parity
    tests) evaluates the same numbers."""
    return W.jitter(base, 100 + int(k))


def rhs_forcing(ws):
    """The benchmark's forcing (pcpdrp, edir, ett) and ws0.surf."""
    return W.random_forcing(ws, 3)


def log_uniform_sizes(n: int, lo: int, hi: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)


def step_forcing(ws, nsteps: int, stepsize: float, seed: int):
    """Hourly forcing held for each model step: (pcpdrp, edir, ett) [nsteps]."""
    hours = int((nsteps * stepsize + 3599) // 3600) + 1
    p, e, t = W.hourly_forcing(ws, hours, seed=seed)
    k = ((np.arange(nsteps) * stepsize) // 3600).astype(np.int64)
    return p[k].copy(), e[k].copy(), t[k].copy()


@dataclasses.dataclass
class CaseSpec:
    nelem: int
    seed: int
    nsteps: int
    stepsize: float = 60.0
    ksat_mult: float = 1.0
    rough_mult: float = 1.0


def make_case(spec: CaseSpec) -> dict:
    ws = W.generate(int(spec.nelem), river_count(int(spec.nelem)), seed=int(spec.seed))
    ws.stepsize = float(spec.stepsize)
    if spec.ksat_mult != 1.0 or spec.rough_mult != 1.0:
        a = ws.arrays
        a["ksath"] = a["ksath"] * spec.ksat_mult
        a["ksatv"] = a["ksatv"] * spec.ksat_mult
        a["rough"] = a["rough"] * spec.rough_mult
    pcp, edir, ett = step_forcing(ws, spec.nsteps, spec.stepsize, seed=int(spec.seed) + 7)
    return dict(ws=ws, y0=W.relax_state(ws), pcp=pcp, edir=edir, ett=ett,
                outlet=int(np.where(ws.arrays["down"] < 0)[0][0]),
                ctrl=StepControl(stepsize=int(spec.stepsize)), spec=spec)


def make_cases(specs, processes: int | None = None) -> list:
    """Generate cases in parallel (spawned processes: safe after CUDA init)."""
    processes = processes or min(16, os.cpu_count() or 1)
    if processes <= 1 or len(specs) <= 1:
        return [make_case(s) for s in specs]
    with mp.get_context("spawn").Pool(processes) as pool:
        return pool.map(make_case, specs, chunksize=1)


def batched_specs(n: int = 256, lo: int = 2000, hi: int = 200000, nsteps: int = 10, seed: int = 0):
    sizes = log_uniform_sizes(n, lo, hi, seed)
    return [CaseSpec(int(s), 1000 + k, nsteps) for k, s in enumerate(sizes)]


def serving_specs(n: int, lo: int = 1000, hi: int = 500000, nsteps: int = 10, seed: int = 1,
                  stepsizes=(30.0, 60.0, 90.0, 120.0, 180.0)):
    rng = np.random.default_rng(seed)
    sizes = log_uniform_sizes(n, lo, hi, seed + 1)
    out = []
    for k, s in enumerate(sizes):
        out.append(CaseSpec(int(s), 5000 + k, nsteps, float(rng.choice(stepsizes)),
                            float(rng.uniform(0.3, 3.0)), float(rng.uniform(0.5, 2.0))))
    return out


def poisson_arrivals(n: int, rate: float, seed: int = 2) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n)) - 0.0


def fifo_latencies(arrivals, service):
    """Latencies of a single first-in-first-out server with the given service times."""
    end = 0.0
    lat = []
    for a, s in zip(arrivals, service):
        start = max(a, end)
        end = start + s
        lat.append(end - a)
    return np.array(lat), end


def run_batched(n: int, lo: int, hi: int, nsteps: int, gate: float = 1.0, profile: bool = False) -> dict:
    """Generate and integrate a batched workload; returns timings and counters."""
    import time
    from .batch import Batch, limits_for
    cases = make_cases(batched_specs(n, lo, hi, nsteps))
    b = Batch(limits_for([c["ws"] for c in cases], nsteps))
    b.set_rhs_gate(gate)
    b.set_profiling(profile)
    t0 = time.perf_counter()
    ids = b.add_many(cases)
    t1 = time.perf_counter()
    b.step()
    t2 = time.perf_counter()
    res = [b.result(i) for i in ids]
    inf = b.info()
    b.close()
    evals = sum(c["ws"].nelem * (r["stats"].nfe + r["stats"].nfes) for c, r in zip(cases, res))
    return dict(watersheds=n, elements=int(sum(c["ws"].nelem for c in cases)), admit_s=t1 - t0,
                solve_s=t2 - t1, rounds=inf.rounds, rhs_rounds=inf.rhs_rounds, launches=inf.launches,
                elem_evals=evals, host_ms=inf.host_ms, wait_ms=inf.wait_ms, program_ms=inf.program_ms,
                rhs_ms=inf.rhs_ms)


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="run a batched-watershed workload on the GPU")
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--lo", type=int, default=2000)
    ap.add_argument("--hi", type=int, default=200000)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--gate", type=float, default=1.0)
    ap.add_argument("--profile", action="store_true")
    a = ap.parse_args()
    print(json.dumps(run_batched(a.n, a.lo, a.hi, a.steps, a.gate, a.profile)))
