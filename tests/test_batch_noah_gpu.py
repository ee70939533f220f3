"""Flux-PIHM watersheds with Noah on the device in the batch engine and the
serving layer (pihm_batch_job.noah): each runs Noah() every land-surface
step, the Flux-PIHM right-hand side on Noah's outputs, and after every model
step Summary's _NOAH_ part and NoahHydrol, as the reference's _NOAH_ build
does (src/pihm.c:21-123).  Every watershed's final state, hydrograph and
integrator counters must be bit-identical to its run alone through
pihm_gpu.single.NoahWatershed, whatever else shares the arena (plain
watersheds, other Flux-PIHM watersheds)."""
import numpy as np
import pytest

import pihm_gpu.watershed as W
from pihm_gpu import noah as N
from pihm_gpu import workloads as WL

pytestmark = pytest.mark.gpu

NSTEPS, LSM = 150, 3600.0  # 2.5 hours of 60 s model steps: Noah at 0, 1 h and 2 h


def _case(ne, seed):
    ws = W.generate(ne, WL.river_count(ne), seed=seed)
    params, state = N.synthetic_noah(ws, seed=seed + 1, nlayers=4)
    forcings = [N.forcing(ws, h, seed=seed + 2) for h in range(3)]
    return dict(ws=ws, y0=W.relax_state(ws), params=params, state=state, forcings=forcings,
                outlet=int(np.where(np.asarray(ws.arrays["down"]) < 0)[0][0]))


@pytest.fixture(scope="module")
def cases():
    return [_case(3000, 40), _case(8000, 50)]


@pytest.fixture(scope="module")
def alone(cases):
    from pihm_gpu.single import NoahWatershed
    from pihm_gpu.solver import StepControl, run_steps
    out = []
    for c in cases:
        m = NoahWatershed(c["ws"], c["y0"], c["params"], c["state"], lambda h, c=c: c["forcings"][h], lsm_step=LSM)
        try:
            r = run_steps(m, StepControl(), NSTEPS, m.set_forcing, record_every=NSTEPS, outlet=c["outlet"])
        finally:
            m.close()
        out.append(dict(y=r["states"][-1], outlet=r["outlet"], stats=r["stats"]))
    return out


def _same(got, want):
    s, w = got["stats"], want["stats"]
    return (np.array_equal(got["y"], want["y"]) and np.array_equal(got["outlet"], want["outlet"]) and
            (s.nst, s.nfe, s.nni, s.ncfn, s.netf, s.nli) == (w.nst, w.nfe, w.nni, w.ncfn, w.netf, w.nli))


def test_batched_flux_pihm_matches_solo_runs(cases, alone):
    from pihm_gpu.batch import Batch, limits_for
    from pihm_gpu.solver import StepControl
    plain = W.generate(2000, WL.river_count(2000), seed=9)
    pcp, edir, ett = WL.step_forcing(plain, NSTEPS, 60.0, seed=4)
    b = Batch(limits_for([c["ws"] for c in cases] + [plain], NSTEPS, slack=1.2))
    try:
        ids = [b.add_noah(c["ws"], c["y0"], StepControl(), c["params"], c["state"], c["forcings"], LSM, NSTEPS,
                          outlet=c["outlet"]) for c in cases]
        b.add(plain, W.relax_state(plain), StepControl(), pcp, edir, ett)
        b.step()
        for k, (i, want) in enumerate(zip(ids, alone)):
            assert b.poll(i)[1] == 0, k
            got = b.result(i)
            print(f"Flux-PIHM watershed {k}: {got['stats'].nst} steps")
            assert _same(got, want), k
    finally:
        b.close()


def test_served_flux_pihm_matches_solo_runs(cases, alone):
    from pihm_gpu.batch import Batch, limits_for
    from pihm_gpu.solver import StepControl
    b = Batch(limits_for([cases[1]["ws"]], NSTEPS, slack=1.3))  # room for one at a time
    try:
        tickets = [b.submit_noah(c["ws"], c["y0"], StepControl(), c["params"], c["state"], c["forcings"], LSM,
                                 NSTEPS, arrival=0.01 * k, outlet=c["outlet"]) for k, c in enumerate(cases)]
        b.serve(workers=2)
        for k, (t, want) in enumerate(zip(tickets, alone)):
            assert b.record(t).solver_rc == 0, k
            assert _same(b.served(t), want), k
    finally:
        b.close()
