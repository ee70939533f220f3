"""End-to-end solves: the BDF integrator (include/pihm_bdf.h, a restatement of
CVODE 2.9) driving the right-hand side through the reference's model-step
loop, against the reference's own CVODE + ODE() run
(tests/golden/make_golden_solve.py: 1,000 elements, 2 days, 60 s steps).

On the CPU, with the right-hand-side restatement over host vectors, the
integrator reproduces the reference run step for step (same counters, same
states, same hydrograph, bit for bit).

A run at reltol 1e-4 is sensitive to the last bit of the right-hand side.
tests/golden/make_sensitivity.py repeats the reference run six times with
every right-hand-side output multiplied by (1 +- 2^-52) (seeded signs): the
step counts spread over 11518..11997 (reference 11752), the hydrograph moves
by up to 6.2e-3 of its peak and single storages by up to 17 % of
max(|storage|, 1 mm) after 2 days.  The GPU right-hand side differs from the
reference's by about an ulp (pow, fused multiply-adds, reciprocals, reduction
order), so its end-to-end run is held to that envelope: no farther from the
reference than the farthest perturbed run, in each measure (the GPU run sits
at about 0.6 of the hydrograph envelope and 0.3 of the storage envelope)."""
import os

import numpy as np
import pytest

import pihm_gpu.watershed as W
from backends import GpuBackend, OracleBackend
from pihm_gpu.solver import StepControl, run_steps

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden():
    z = np.load(os.path.join(GOLD, "c0_solve.npz"))
    ws = W.Watershed.load(os.path.join(GOLD, "c0_watershed.npz"))
    ctrl = StepControl(**{str(k): (int(v) if str(k) == "stepsize" else float(v))
                          for k, v in zip(z["ctrl_names"], z["ctrl"])})
    return ws, z, ctrl


def _run(backend_cls, ws, z, ctrl, deferred_scalars=None, **kw):
    nsteps = z["outlet_q"].shape[0]
    b = backend_cls(ws, z["y0"], z["pcp"], z["edir"], z["ett"], **kw)
    try:
        return run_steps(b, ctrl, nsteps, b.set_forcing, record_every=int(z["every"]),
                         outlet=int(z["outlet"]), water_balance=True, deferred_scalars=deferred_scalars)
    finally:
        b.close()


@pytest.mark.parametrize("deferred", [0, 1], ids=["plain", "deferred_scalars"])
def test_integrator_reproduces_reference_cvode_on_cpu(deferred):
    """deferred_scalars runs the GMRES iteration that keeps its norm and
    Gram-Schmidt dot products with the vectors (bdf_core.h
    atimes_gs_deferred) with the values held on the host: same operations in
    the same order, so CVODE's run is reproduced bit for bit either way."""
    ws, z, ctrl = _golden()
    res = _run(OracleBackend, ws, z, ctrl, deferred_scalars=deferred)
    assert res["deferred_scalars"] == deferred
    s = res["stats"]
    got = [s.nst, s.nfe, s.nni, s.ncfn, s.netf, s.nli, s.nfes]
    assert got == list(z["stats"]), (got, list(z["stats"]))
    assert np.array_equal(res["states"], z["states"])
    assert np.array_equal(res["outlet"], z["outlet_q"])
    # the water balance after every step: PrintWaterBal's sums, bit for bit
    assert np.array_equal(res["wb"], z["wb"])


def _wb_error(wb):
    """PrintWaterBal's cumulative error (src/print.c: from its second call)."""
    src, snk, strg = wb[:, 0], wb[:, 1], wb[:, 2]
    return np.cumsum(src[1:] - snk[1:] - (strg[1:] - strg[:-1]))


def test_reference_water_balance_fixture():
    z = np.load(os.path.join(GOLD, "c0_solve.npz"))
    err = _wb_error(z["wb"])
    # the full-precision sums round to the reference's own printed lines
    printed = z["wb_printed"]
    assert np.allclose(err, printed[:, 5], rtol=1e-5, atol=1e-6 * np.abs(err).max())
    assert np.allclose(z["wb"][1:, 0], printed[:, 1], rtol=1e-5, atol=1e-300)


def _rel(a, b, floor=1e-5):
    """Relative error with the solver's absolute tolerance as the floor
    (storages that are zero in the reference compare absolutely)."""
    den = np.maximum(np.abs(b), floor)
    return float(np.max(np.abs(a - b) / den))


def _envelope(z):
    """Largest deviation of the one-ulp-perturbed reference runs."""
    e = np.load(os.path.join(GOLD, "c0_sensitivity.npz"))
    q_ref, fin = z["outlet_q"], z["states"][-1]
    peak = np.max(np.abs(q_ref))
    qerr = max(np.max(np.abs(q - q_ref)) / peak for q in e["outlet"])
    serr = max(_rel(f, fin, floor=1e-3) for f in e["final"])
    return qerr, serr, int(e["nst"].min()), int(e["nst"].max())


def _wb_envelope(z):
    """Largest cumulative water-balance residual among the reference run and
    its one-ulp-perturbed runs: the residual is set by the integrator's
    step sequence, so it moves with last-bit noise like the storages do."""
    e = np.load(os.path.join(GOLD, "c0_sensitivity.npz"))
    runs = [float(r) for r in e["wb_resid"]]
    return max([np.abs(_wb_error(z["wb"])).max()] + runs), runs


def test_sensitivity_envelope_fixture():
    ws, z, ctrl = _golden()
    qenv, senv, nmin, nmax = _envelope(z)
    # the perturbed runs moved, but stayed close to the reference run
    assert 1e-4 < qenv < 2e-2 and 1e-3 < senv < 0.5
    assert nmin <= int(z["stats"][0]) <= nmax
    # their water-balance residuals scatter around the reference run's
    wenv, runs = _wb_envelope(z)
    e_ref = np.abs(_wb_error(z["wb"])).max()
    assert min(runs) < e_ref < max(runs) == wenv


@pytest.mark.gpu
def test_gpu_solve_hydrograph_and_storages():
    ws, z, ctrl = _golden()
    res = _run(GpuBackend, ws, z, ctrl)
    q_ref = z["outlet_q"]
    qenv, senv, nmin, nmax = _envelope(z)
    # hydrograph: relative to the peak flow, per step
    qerr = np.max(np.abs(res["outlet"] - q_ref)) / np.max(np.abs(q_ref))
    serr = _rel(res["states"][-1], z["states"][-1], floor=1e-3)
    s = res["stats"]
    print(f"GPU solve: nst {s.nst} nfe {s.nfe} (reference {z['stats'][0]} {z['stats'][1]}); "
          f"hydrograph err {qerr:.2e} (envelope {qenv:.2e}), storage err {serr:.2e} "
          f"(envelope {senv:.2e})")
    assert qerr <= qenv
    assert serr <= senv
    span = nmax - nmin
    assert nmin - span <= s.nst <= nmax + span
    # mass balance: the cumulative residual is no worse than the reference
    # gives under one-ulp noise in its right-hand side
    e_gpu, e_ref = np.abs(_wb_error(res["wb"])).max(), np.abs(_wb_error(z["wb"])).max()
    wenv, runs = _wb_envelope(z)
    print(f"water-balance residual: GPU {e_gpu:.4g} m3, reference {e_ref:.4g} m3, "
          f"perturbed reference {min(runs):.4g} .. {max(runs):.4g} m3 (storage {z['wb'][-1, 2]:.4g} m3)")
    assert e_gpu <= wenv


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["c0_golden", "generated_60k"])
def test_gpu_deferred_scalars_same_solve(case):
    """GMRES with its norm and Gram-Schmidt dot products kept on the device
    and the right-hand side's status read back with them (the default for
    pihm_gpu_ode on device vectors) makes the solve of the plain iteration
    bit for bit: every state, outlet value and counter."""
    from pihm_gpu import workloads as WL
    if case == "c0_golden":
        ws, z, ctrl = _golden()
        y0, pcp, edir, ett, nsteps = z["y0"], z["pcp"], z["edir"], z["ett"], 240
        outlet = int(z["outlet"])
    else:
        ws = W.generate(60_000, WL.river_count(60_000), seed=4)
        ctrl, nsteps = StepControl(), 6
        pcp, edir, ett = WL.step_forcing(ws, nsteps, 60.0, seed=3)
        y0 = W.relax_state(ws)
        outlet = int(np.where(np.asarray(ws.arrays["down"]) < 0)[0][0])
    res = {}
    for mode in (0, -1):
        b = GpuBackend(ws, y0, pcp, edir, ett)
        try:
            res[mode] = run_steps(b, ctrl, nsteps, b.set_forcing, record_every=nsteps // 2, outlet=outlet,
                                  deferred_scalars=mode)
        finally:
            b.close()
    assert res[0]["deferred_scalars"] == 0 and res[-1]["deferred_scalars"] == 3
    s0, s1 = res[0]["stats"], res[-1]["stats"]
    print(f"{case}: {s1.nst} steps, {s1.nli} GMRES iterations, {s1.nfe + s1.nfes} evaluations")
    assert [s0.nst, s0.nfe, s0.nni, s0.ncfn, s0.netf, s0.nli, s0.nfes] == \
        [s1.nst, s1.nfe, s1.nni, s1.ncfn, s1.netf, s1.nli, s1.nfes]
    assert np.array_equal(res[0]["states"], res[-1]["states"])
    assert np.array_equal(res[0]["outlet"], res[-1]["outlet"])


def test_deferred_scalars_follow_recoverable_rhs_failures_on_cpu():
    """A right-hand side that reports recoverable failures (return +1): the
    difference-quotient product retries with a quarter of the increment
    (CVSpilsDQJtimes), a Newton evaluation makes CVODE retry the step.  The
    GMRES iteration with its scalars kept aside (host values) must make the
    same calls and the same solve as the plain iteration."""
    import ctypes
    ws, z, ctrl = _golden()
    nsteps = 60
    RHS = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)
    out = {}
    for deferred in (0, 1):
        b = OracleBackend(ws, z["y0"], z["pcp"], z["edir"], z["ett"])
        inner = RHS(b.rhs.value)
        calls = []

        def flaky(t, y, ydot, ud, inner=inner, calls=calls):
            rc = inner(t, y, ydot, ud)
            calls.append(t)
            return 1 if len(calls) % 37 == 0 else rc

        cb = RHS(flaky)
        b.rhs = ctypes.cast(cb, ctypes.c_void_p)
        try:
            r = run_steps(b, ctrl, nsteps, b.set_forcing, record_every=nsteps, deferred_scalars=deferred)
        finally:
            b.close()
        s = r["stats"]
        out[deferred] = (r["states"], [s.nst, s.nfe, s.nni, s.ncfn, s.netf, s.nli, s.nfes], calls)
        assert r["deferred_scalars"] == deferred
    assert out[0][1] == out[1][1], (out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
    assert np.array_equal(out[0][0], out[1][0])
