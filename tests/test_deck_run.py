"""An input deck run end to end the way the reference's main loop runs it,
with its own forcing (tests/golden/make_golden_deck.py): ApplyBc, ApplyForc +
IntcpSnowEt every LSM_STEP, SolveCVode, Summary, AdjCVodeMaxStep, for one
simulated day of 60 s model steps on a generated 1,000-element deck with
snow, rain, melt and interception.

On the CPU the restatements (right-hand side, land-surface step, integrator)
reproduce the reference's run bit for bit.  The GPU run is held, like the
plain two-day solve, to twice the spread of 16 runs of the restatement whose
right-hand side is perturbed by one ulp: the hydrograph relative to its
peak, the storages relative to max(|storage|, 1 mm), the step count within
one span of the perturbed runs' range, and the cumulative water-balance
residual of PrintWaterBal (src/print.c:337-542) within twice the perturbed
runs' distance from the reference's.  (That residual is large here -- about
5.5e5 m3 on a 2.5e8 m3 store after a day -- in the reference itself: it
counts the land-surface step's evaporation as a sink in full whether or not
the right-hand side can draw it from the stores.)
"""
import os

import numpy as np
import pytest

from parity import land_deck

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture():
    return np.load(os.path.join(GOLD, "deck_solve.npz"))


def _deck(tmp_path):
    from pihm_gpu import capi, deck as D
    if not os.path.exists(capi.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    return D.Deck.read(land_deck(str(tmp_path)), "gen")


def _wb_error(wb):
    src, snk, strg = wb[:, 0], wb[:, 1], wb[:, 2]
    return np.cumsum(src[1:] - snk[1:] - (strg[1:] - strg[:-1]))


def test_restated_deck_run_reproduces_the_reference(tmp_path):
    from backends import OracleDeckBackend
    from pihm_gpu.single import step_control
    from pihm_gpu.solver import run_steps
    z = _fixture()
    d = _deck(tmp_path)
    n = z["outlet_q"].shape[0]
    b = OracleDeckBackend(d)
    try:
        r = run_steps(b, step_control(d.control()), n, b.set_forcing, record_every=int(z["every"]),
                      outlet=int(z["outlet"]), water_balance=True)
    finally:
        b.close()
    s = r["stats"]
    assert (s.nst, s.nfe, s.nni, s.ncfn, s.netf) == tuple(int(v) for v in z["stats"][:5])
    assert np.array_equal(r["states"], z["states"])
    assert np.array_equal(r["outlet"], z["outlet_q"])
    assert np.array_equal(np.asarray(r["wb"]), z["wb"])


def test_deck_fixture_envelope():
    z = _fixture()
    nst = z["sens_nst"]
    assert nst.min() <= int(z["stats"][0]) <= nst.max()
    e_ref = np.abs(_wb_error(z["wb"])).max()
    assert z["sens_wb_resid"].min() <= e_ref <= z["sens_wb_resid"].max()


def _rel(a, b, floor):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


@pytest.mark.gpu
def test_gpu_deck_run_within_envelope(tmp_path):
    from pihm_gpu.single import run_deck
    z = _fixture()
    d = _deck(tmp_path)
    n = z["outlet_q"].shape[0]
    r = run_deck(d, n, record_every=int(z["every"]), outlet=int(z["outlet"]), water_balance=True)
    q_ref, fin = z["outlet_q"], z["states"][-1]
    peak = np.max(np.abs(q_ref))
    qenv = max(np.max(np.abs(q - q_ref)) / peak for q in z["sens_outlet"])
    senv = max(_rel(f, fin, 1e-3) for f in z["sens_final"])
    qerr = np.max(np.abs(r["outlet"] - q_ref)) / peak
    serr = _rel(r["states"][-1], fin, 1e-3)
    e_gpu, e_ref = np.abs(_wb_error(np.asarray(r["wb"]))).max(), np.abs(_wb_error(z["wb"])).max()
    wenv = max(abs(e - e_ref) for e in z["sens_wb_resid"])
    nmin, nmax = int(z["sens_nst"].min()), int(z["sens_nst"].max())
    print(f"GPU deck run: nst {r['stats'].nst} (reference {z['stats'][0]}, perturbed {nmin}..{nmax}); "
          f"hydrograph err {qerr:.2e} (envelope {qenv:.2e}), storage err {serr:.2e} (envelope {senv:.2e}); "
          f"water-balance residual {e_gpu:.6g} m3 (reference {e_ref:.6g}, perturbed within {wenv:.4g})")
    assert qerr <= 2 * qenv
    assert serr <= 2 * senv
    span = nmax - nmin
    assert nmin - span <= r["stats"].nst <= nmax + span
    assert abs(e_gpu - e_ref) <= 2 * wenv


class ArrayDeck:
    """A deck held as arrays (a fixture) behind the methods that
    pihm_gpu.single.DeckWatershed and tests/backends.OracleDeckBackend read,
    for the GPU machine, where the deck's files are not."""

    def __init__(self, ws, land, ctrl, y0):
        self.ws, self._land, self.ctrl, self.y0 = ws, land, ctrl, y0

    @staticmethod
    def from_fixture(z, mesh="example_watershed.npz"):
        import pihm_gpu.land as L
        import pihm_gpu.watershed as W
        from pihm_gpu.deck import DeckControl
        ws = W.Watershed.load(os.path.join(GOLD, mesh))
        step = {str(k): float(v) for k, v in zip(z["ctrl_names"], z["ctrl"])}
        step["mxstep"] = int(step.get("mxstep", 0))
        ws.surf_mode, ws.riv_mode, ws.stepsize = int(z["surf_mode"]), int(z["riv_mode"]), step["stepsize"]
        ctrl = DeckControl(int(z["surf_mode"]), int(z["riv_mode"]), 2, 0, int(z["start"]), 0, int(z["lsm_step"]),
                           step)
        land = L.Land({k: z["p_" + k] for k in L.PARAM_I32 + L.PARAM_F64}, tuple(float(c) for c in z["cal"]),
                      z["meteo_len"], z["meteo_time"], z["meteo_data"], z["lai_len"], z["lai_time"], z["lai_data"])
        return ArrayDeck(ws, land, ctrl, np.asarray(z["y0"], np.float64))

    def watershed(self):
        return self.ws

    def land(self):
        return self._land

    def control(self):
        return self.ctrl

    def initial_state(self):
        return self.y0.copy()

    def initial_storage(self):
        return np.zeros(self.ws.nelem), np.zeros(self.ws.nelem)

    def bc(self, t):
        raise AssertionError("the example deck has no boundary series")


def _example():
    path = os.path.join(GOLD, "example_run.npz")
    if not os.path.exists(path):
        pytest.skip("tests/golden/example_run.npz not generated")
    return np.load(path)


def test_restated_example_run_reproduces_the_reference():
    """The reference's bundled example deck, one simulated day with its own
    forcing: the restatements reproduce the reference's run bit for bit."""
    from pihm_gpu import capi
    if not os.path.exists(capi.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    from backends import OracleDeckBackend
    from pihm_gpu.single import step_control
    from pihm_gpu.solver import run_steps
    z = _example()
    d = ArrayDeck.from_fixture(z)
    n = z["outlet_q"].shape[0]
    b = OracleDeckBackend(d)
    try:
        r = run_steps(b, step_control(d.control()), n, b.set_forcing, record_every=int(z["every"]),
                      outlet=int(z["outlet"]), water_balance=True)
    finally:
        b.close()
    s = r["stats"]
    assert (s.nst, s.nfe, s.nni, s.ncfn, s.netf) == tuple(int(v) for v in z["stats"][:5])
    assert np.array_equal(r["states"], z["states"])
    assert np.array_equal(r["outlet"], z["outlet_q"])
    assert np.array_equal(np.asarray(r["wb"]), z["wb"])


@pytest.mark.gpu
def test_gpu_example_run_within_envelope():
    from pihm_gpu.single import DeckWatershed, step_control
    from pihm_gpu.solver import run_steps
    z = _example()
    d = ArrayDeck.from_fixture(z)
    n = z["outlet_q"].shape[0]
    b = DeckWatershed(d)
    try:
        r = run_steps(b, step_control(d.control()), n, b.set_forcing, record_every=int(z["every"]),
                      outlet=int(z["outlet"]), water_balance=True)
    finally:
        b.close()
    q_ref, fin = z["outlet_q"], z["states"][-1]
    peak = np.max(np.abs(q_ref))
    qenv = max(np.max(np.abs(q - q_ref)) / peak for q in z["sens_outlet"])
    senv = max(_rel(f, fin, 1e-3) for f in z["sens_final"])
    qerr = np.max(np.abs(r["outlet"] - q_ref)) / peak
    serr = _rel(r["states"][-1], fin, 1e-3)
    e_gpu, e_ref = np.abs(_wb_error(np.asarray(r["wb"]))).max(), np.abs(_wb_error(z["wb"])).max()
    wenv = max(abs(e - e_ref) for e in z["sens_wb_resid"])
    nmin, nmax = int(z["sens_nst"].min()), int(z["sens_nst"].max())
    print(f"GPU example run: nst {r['stats'].nst} (reference {z['stats'][0]}, perturbed {nmin}..{nmax}); "
          f"hydrograph err {qerr:.2e} (envelope {qenv:.2e}), storage err {serr:.2e} (envelope {senv:.2e}); "
          f"water-balance residual {e_gpu:.6g} m3 (reference {e_ref:.6g}, perturbed within {wenv:.4g})")
    assert qerr <= 2 * qenv + 1e-15
    assert serr <= 2 * senv + 1e-15
    span = max(nmax - nmin, 1)
    assert nmin - span <= r["stats"].nst <= nmax + span
    assert abs(e_gpu - e_ref) <= 2 * wenv + 1e-9 * max(abs(e_ref), 1.0)
