"""Input decks with their own forcing in the batch engine and the serving
layer (pihm_batch_job.deck / .land): each watershed takes its boundary
values from its deck's series every model step (ApplyBc) and runs the
land-surface step (ApplyForc + IntcpSnowEt) every LSM_STEP, as the
reference's main loop does (src/pihm.c:15-66).  Every deck's result -- final
state, hydrograph, integrator counters -- must be bit-identical to the same
deck run alone through pihm_gpu.single.run_deck, whatever else shares the
arena."""
import datetime
import os

import numpy as np
import pytest

from parity import land_deck

pytestmark = pytest.mark.gpu

NSTEPS = 150  # 2.5 simulated hours of 60 s steps: 10 land-surface steps of 900 s


def _bc_land_deck(directory, seed=6):
    """A generated 1,000-element deck with a Dirichlet and a Neumann boundary
    series on two outer edges and a seeded land-surface model."""
    import pihm_gpu.land as L
    import pihm_gpu.watershed as W
    from pihm_gpu import deck as D
    ws = W.generate(1000, 100, seed=seed)
    land = L.synthetic_land(ws, seed=seed + 1, hours=24, per_type=True)
    rng = np.random.default_rng(seed)
    lc = land.params["lc_type"]
    ws.arrays["rough"] = np.round(rng.uniform(0.02, 0.3, L.NLC), 3)[lc - 1]
    ws.arrays["rzd"] = np.round(rng.uniform(0.3, 1.5, L.NLC), 2)[lc - 1]
    bct = np.zeros((ws.nelem, 3), np.int32)
    outer = np.argwhere(np.asarray(ws.arrays["nabr"]).reshape(-1, 3) == 0)
    bct[tuple(outer[0])] = 1
    bct[tuple(outer[1])] = -2
    ws.arrays["bc_type"] = bct
    zs = float(np.asarray(ws.arrays["zmax"])[outer[0][0]])
    series = [[("2009-01-01 00:00", zs - 0.5), ("2009-01-01 12:00", zs - 0.2), ("2009-01-02 00:00", zs - 0.8)],
              [("2009-01-01 00:00", -1e-4), ("2009-01-02 00:00", -3e-4)]]
    path = os.path.join(directory, "input", "bcgen")
    end = L.epoch("2009-01-01 00:00") + 3600 * 24
    end_s = datetime.datetime.fromtimestamp(end, datetime.timezone.utc).strftime("%Y-%m-%d %H:%M")
    D.write_deck(ws, path, "bcgen", land=land, lsm_step=900, start="2009-01-01 00:00", end=end_s,
                 elem_bc_series=series)
    return path


@pytest.fixture(scope="module")
def decks(tmp_path_factory):
    from pihm_gpu import capi, deck as D
    if not os.path.exists(capi.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    t = tmp_path_factory.mktemp("decks")
    a = D.Deck.read(land_deck(str(t / "a")), "gen")
    b = D.Deck.read(_bc_land_deck(str(t / "b")), "bcgen")
    assert np.count_nonzero(b.watershed().arrays["bc_type"]) == 2
    return [a, b]


def _outlet(deck):
    return int(np.where(np.asarray(deck.watershed().arrays["down"]) < 0)[0][0])


@pytest.fixture(scope="module")
def alone(decks):
    from pihm_gpu.single import run_deck
    out = []
    for d in decks:
        r = run_deck(d, NSTEPS, record_every=NSTEPS, outlet=_outlet(d))
        out.append(dict(y=r["states"][-1], outlet=r["outlet"], stats=r["stats"]))
    return out


def _same(got, want):
    s, w = got["stats"], want["stats"]
    return (np.array_equal(got["y"], want["y"]) and np.array_equal(got["outlet"], want["outlet"]) and
            (s.nst, s.nfe, s.nni, s.ncfn, s.netf, s.nli) == (w.nst, w.nfe, w.nni, w.ncfn, w.netf, w.nli))


def test_batched_decks_match_their_solo_runs(decks, alone):
    import pihm_gpu.watershed as W
    from pihm_gpu import workloads as WL
    from pihm_gpu.batch import Batch, limits_for
    from pihm_gpu.solver import StepControl
    other = W.generate(3000, WL.river_count(3000), seed=9)
    pcp, edir, ett = WL.step_forcing(other, NSTEPS, 60.0, seed=4)
    b = Batch(limits_for([d.watershed() for d in decks] + [other], NSTEPS, slack=1.2))
    try:
        ids = [b.add_deck(d, NSTEPS, outlet=_outlet(d)) for d in decks]
        b.add(other, W.relax_state(other), StepControl(), pcp, edir, ett)
        assert all(i is not None for i in ids)
        b.step()
        for k, (i, want) in enumerate(zip(ids, alone)):
            st, rc = b.poll(i)
            assert rc == 0, (k, st, rc)
            got = b.result(i)
            print(f"deck {k}: {got['stats'].nst} steps, outlet flux {got['outlet'][-1]:.6g}")
            assert _same(got, want), k
    finally:
        b.close()


def test_served_decks_match_their_solo_runs(decks, alone):
    from pihm_gpu.batch import Batch, limits_for
    b = Batch(limits_for([decks[0].watershed()], NSTEPS, slack=1.3))  # room for one deck at a time
    try:
        tickets = [b.submit_deck(d, arrival=0.01 * k, nsteps=NSTEPS, outlet=_outlet(d)) for k, d in enumerate(decks)]
        b.serve(workers=2)
        for k, (t, want) in enumerate(zip(tickets, alone)):
            rec = b.record(t)
            assert rec.solver_rc == 0, (k, rec.solver_rc)
            assert _same(b.served(t), want), k
    finally:
        b.close()
