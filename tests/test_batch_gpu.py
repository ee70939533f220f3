"""Batch engine (include/pihm_batch.h) on the GPU.

A watershed integrated in a batch must follow exactly the trajectory the
single-watershed path (pihm_bdf_* over device N_Vectors with pihm_gpu_ode,
driven by the reference's model-step loop) computes for it alone: same final
state, same outlet flux after every model step, same solver counters, bit for
bit -- whatever else shares the batch, whenever it was admitted and whatever
happens to its neighbours."""
import copy

import numpy as np
import pytest

import pihm_gpu.watershed as W
from backends import GpuBackend, step_forcing
from pihm_gpu.batch import DONE, FAILED, RUNNING, Batch, BatchLimits, limits_for
from pihm_gpu.solver import StepControl, run_steps

pytestmark = pytest.mark.gpu


def _case(nelem, seed, nsteps, stepsize=60):
    nriver = max(4, int(round(100 * (nelem / 1000.0) ** 0.826)))
    ws = W.generate(nelem, nriver, seed=seed)
    pcp, edir, ett = step_forcing(ws, nsteps, stepsize=stepsize, seed=seed + 2)
    # a wet start so that every branch of the right-hand side is exercised
    y0 = W.reference_state(ws, seed=seed)
    outlet = int(np.where(ws.arrays["down"] < 0)[0][0])
    return dict(ws=ws, y0=y0, pcp=pcp, edir=edir, ett=ett, outlet=outlet,
                ctrl=StepControl(stepsize=stepsize))


def _alone(c):
    """The single-watershed GPU path."""
    b = GpuBackend(c["ws"], c["y0"], c["pcp"], c["edir"], c["ett"])
    try:
        n = len(c["pcp"])
        r = run_steps(b, c["ctrl"], n, b.set_forcing, record_every=n, outlet=c["outlet"])
    finally:
        b.close()
    return dict(y=r["states"][-1], outlet=r["outlet"], stats=r["stats"])


def _add(batch, c):
    return batch.add(c["ws"], c["y0"], c["ctrl"], c["pcp"], c["edir"], c["ett"], outlet=c["outlet"])


def _same(got, want, label):
    assert np.array_equal(got["y"], want["y"]), (
        f"{label}: final state differs, max |d| {np.max(np.abs(got['y'] - want['y'])):.3e}")
    assert np.array_equal(got["outlet"], want["outlet"]), f"{label}: outlet series differs"
    gs, ws_ = got["stats"], want["stats"]
    for k in ("nst", "nfe", "nni", "ncfn", "netf", "nli", "nfes"):
        assert getattr(gs, k) == getattr(ws_, k), (label, k, getattr(gs, k), getattr(ws_, k))


@pytest.fixture(scope="module")
def cases():
    # uneven sizes, their own soils, forcing and (for the last) model step
    c = [_case(1000, 11, 90), _case(400, 12, 60), _case(2500, 13, 90)]
    c[1]["ctrl"] = StepControl(stepsize=90)
    c[1]["ws"].stepsize = 90  # the model step also caps infiltration in the right-hand side
    c[1]["pcp"], c[1]["edir"], c[1]["ett"] = step_forcing(c[1]["ws"], 60, stepsize=90, seed=14)
    return c


@pytest.fixture(scope="module")
def alone(cases):
    return [_alone(c) for c in cases]


def test_batch_is_bit_identical_to_the_single_watershed_path(cases, alone):
    b = Batch(limits_for([c["ws"] for c in cases], 90))
    ids = b.add_many(cases, threads=3)  # prepared on host threads, admitted in order
    assert None not in ids
    assert b.step() == 0
    for i, c, want in zip(ids, cases, alone):
        assert b.poll(i) == (DONE, 0)
        got = b.result(i)
        assert got["steps_done"] == len(c["pcp"])
        _same(got, want, f"watershed {c['ws'].nelem}")
    inf = b.info()
    assert inf.rounds > 0 and inf.rhs_rounds > 0
    b.close()


def test_alone_in_a_batch_and_in_a_mix_agree(cases, alone):
    b = Batch(limits_for([cases[2]["ws"]], 90))
    i = _add(b, cases[2])
    b.step()
    _same(b.result(i), alone[2], "batch of one")
    b.close()


def test_admission_by_capacity_and_reuse_of_released_ranges(cases, alone):
    # room for the largest and the smallest watershed: with the two smaller
    # ones resident the largest has to wait for a slot and a contiguous range
    lim = limits_for([cases[2]["ws"], cases[1]["ws"]], 90)
    b = Batch(lim)
    i0, i1 = _add(b, cases[0]), _add(b, cases[1])
    assert i0 is not None and i1 is not None
    assert _add(b, cases[2]) is None
    # run until one finishes, retire it, admit the waiting one mid-flight
    while b.poll(i0)[0] == RUNNING and b.poll(i1)[0] == RUNNING:
        b.step(max_rounds=50)
    first = i1 if b.poll(i1)[0] == DONE else i0
    _same(b.result(first), alone[[i0, i1].index(first)], "first finished")
    b.release(first)
    i2 = _add(b, cases[2])
    if i2 is None:  # the large one needs both slots' room
        b.step()
        other = i0 if first == i1 else i1
        _same(b.result(other), alone[[i0, i1].index(other)], "second finished")
        b.release(other)
        i2 = _add(b, cases[2])
    assert i2 is not None
    b.step()
    for i in list(b.jobs):
        idx = {i0: 0, i1: 1, i2: 2}[i]
        _same(b.result(i), alone[idx], f"job {idx}")
    b.close()


def test_a_failing_watershed_does_not_disturb_the_others(cases, alone):
    bad = dict(cases[1])
    bad["ws"] = copy.deepcopy(cases[1]["ws"])
    por = bad["ws"].arrays["porosity"].copy()
    por[5] = np.nan  # the right-hand side reports NaN derivatives
    bad["ws"].arrays["porosity"] = por
    b = Batch(limits_for([cases[0]["ws"], cases[1]["ws"]], 90))
    ig = _add(b, cases[0])
    ib = _add(b, bad)
    b.step()
    st, rc = b.poll(ib)
    assert st == FAILED and rc == -8  # CV_RHSFUNC_FAIL
    _same(b.result(ig), alone[0], "healthy neighbour")
    b.close()


def test_limits_are_validated():
    with pytest.raises(RuntimeError):
        Batch(BatchLimits(max_elem=0, max_river=1, max_edge=1, max_record=1, max_systems=1))


def _submit(b, c, arrival):
    return b.submit(c["ws"], c["y0"], c["ctrl"], c["pcp"], c["edir"], c["ett"], arrival=arrival,
                    outlet=c["outlet"])


def test_served_requests_match_their_solo_runs(cases, alone):
    # room for about two at a time: requests queue, join the rounds in
    # flight as others retire, and each still computes its solo trajectory
    b = Batch(limits_for([cases[2]["ws"], cases[1]["ws"]], 90))
    plan = [(0, 0.0), (1, 0.001), (2, 0.002), (0, 0.02), (1, 0.03)]
    tickets = [_submit(b, cases[i], t) for i, t in plan]
    b.serve(workers=2)
    for tk, (i, t) in zip(tickets, plan):
        r = b.record(tk)
        assert r.status == DONE and r.solver_rc == 0, (tk, r.status, r.solver_rc)
        assert r.t_arrival == t and r.t_admit >= r.t_arrival and r.t_done >= r.t_admit
        _same(b.served(tk), alone[i], f"request {tk}")
    b.close()


def test_serving_fails_a_request_larger_than_the_arena(cases, alone):
    b = Batch(limits_for([cases[0]["ws"]], 90))
    big = _submit(b, cases[2], 0.0)
    ok = _submit(b, cases[0], 0.0)
    b.serve(workers=1)
    assert b.record(big).status == FAILED and b.record(big).solver_rc == -5  # PIHM_GPU_ERR_NOMEM
    assert b.record(ok).status == DONE
    _same(b.served(ok), alone[0], "request behind a rejected one")
    b.close()


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_program_kernel_variants_give_the_same_bits(cases, alone, variant):
    b = Batch(limits_for([c["ws"] for c in cases], 90))
    b.set_program_variant(variant)
    ids = b.add_many(cases)
    b.step()
    assert b.info().program_variant == variant
    for i, c, want in zip(ids, cases, alone):
        _same(b.result(i), want, f"variant {variant}, watershed {c['ws'].nelem}")
    b.close()


@pytest.mark.parametrize("shape", [-1, 0, 1, 2])
def test_element_kernel_shapes_give_the_same_bits(cases, alone, shape):
    """Each forced block shape of the element kernel, and the tuner (-1),
    which rotates through them while it times evaluations, give every
    watershed the bits of its solo run."""
    b = Batch(limits_for([c["ws"] for c in cases], 90))
    b.set_rhs_shape(shape)
    ids = b.add_many(cases)
    b.step()
    inf = b.info()
    if shape >= 0:
        assert inf.rhs_shape == shape and not inf.rhs_tuning
    print(f"shape {shape}: in use {inf.rhs_shape}, tuning {inf.rhs_tuning}")
    for i, c, want in zip(ids, cases, alone):
        _same(b.result(i), want, f"shape {shape}, watershed {c['ws'].nelem}")
    b.close()
