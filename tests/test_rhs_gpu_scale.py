"""GPU right-hand side against the CPU oracle at the sizes the benchmark runs.

At 1,000 elements every kernel runs a handful of blocks; the paths that only
matter at scale -- the per-block shared-memory work queues of the edge and
element kernels, the element kernel's occupancy, the locality renumbering of
a million-element mesh, the river kernels beside the element kernels on the
second stream, the carried river-edge flux over consecutive calls -- are
compared here on:

  * the benchmark's own watershed (1,000,000 elements, 30,000 segments,
    generator seed 0) on the benchmark's own perturbed states, three
    consecutive calls through the device-pointer entry point (pihm_gpu_rhs)
    and three through the host-buffer entry point (pihm_gpu_rhs_host);
  * a 300,000-element Delaunay mesh of scattered nodes, the same way;
  * the Flux-PIHM right-hand side on a 200,000-element mesh with 4 Noah soil
    layers, the same way;
  * a batch holding a 100,000-element watershed beside small ones, bit for
    bit with its run alone.

Each row is held to the 1e-12 row-scale bar of tests/parity.py, widened only
by the reference's own last-bit envelope (rows that are differences of
nearly equal quantities, where a power one ulp away moves the result by more
than 1e-12), against the OpenMP restatement of the reference ODE()
(src/ode.c:4-399) making the same call sequence.  The worst normalised error
of each configuration, and how many rows needed the envelope, are printed
(pytest -s shows them)."""
import numpy as np
import pytest

import pihm_gpu.watershed as W
from pihm_gpu import workloads as WL
from parity import RTOL, compare, row_scales

pytestmark = pytest.mark.gpu


def _models(ws, forcing, ws0, ovl, noah=None):
    """The GPU model and three oracles: the reference's arithmetic, and the
    same with every pow()/log() result one ulp up, one ulp down (the
    envelope of tests/parity.py)."""
    import torch
    from oracle import Oracle
    from pihm_gpu.capi import GpuRhs
    g = GpuRhs(ws)
    g.set_stream(torch.cuda.current_stream().cuda_stream)
    oracles = [Oracle(ws, omp=True) for _ in range(3)]
    oracles[1].set_ulp_perturb(+1)
    oracles[2].set_ulp_perturb(-1)
    for m in [g] + oracles:
        if noah is not None:
            m.set_noah(noah)
        m.set_forcing(*forcing)
        m.set_ws0_surf(ws0)
        m.set_river_edge_ovlflow(ovl)
    return g, oracles


def _device_call(g, y):
    """One evaluation through pihm_gpu_rhs on device pointers (internal
    order), the state reordered in and the derivative out on the device."""
    import torch
    yr = torch.from_numpy(np.ascontiguousarray(y)).cuda()
    yi, ydi, ydr = torch.empty_like(yr), torch.empty_like(yr), torch.empty_like(yr)
    g.to_internal(yr.data_ptr(), yi.data_ptr())
    g.rhs_device(yi.data_ptr(), ydi.data_ptr())
    g.to_reference(ydi.data_ptr(), ydr.data_ptr())
    torch.cuda.current_stream().synchronize()
    return ydr.cpu().numpy(), g.status()


def _run_sequence(ws, states, forcing, ws0, ovl, noah, via):
    """Consecutive calls (the carried river-edge flux of one call feeds the
    next) on the GPU and in the oracles; returns the worst normalised error
    net of the last-bit envelope, the worst without it, and the number of
    rows whose error exceeds the plain 1e-12 bar."""
    g, (o, op, om) = _models(ws, forcing, ws0, ovl, noah)
    worst_all = plain_all = 0.0
    over = 0
    try:
        for k, y in enumerate(states):
            want, rc_o = o.rhs(y)
            up, rc_p = op.rhs(y)
            dn, rc_m = om.rhs(y)
            if via == "device":
                got, rc_g = _device_call(g, y)
            else:
                got, rc_g = g.rhs_host(y)
            assert rc_o == 0 and rc_p == 0 and rc_m == 0 and rc_g == 0, (via, k, rc_o, rc_g)
            scale = row_scales(ws, o.fluxes(), *forcing)
            env = np.abs(up - want) + np.abs(dn - want)
            ok, worst, idx = compare(got, want, scale, envelope=env)
            assert ok, (f"{via} call {k}: worst {worst:.3e} at row {idx}: got {got[idx]!r} want {want[idx]!r} "
                        f"envelope {env[idx]!r}")
            worst_all = max(worst_all, worst)
            _, plain, _ = compare(got, want, scale)
            plain_all = max(plain_all, plain)
            den = np.maximum(np.maximum(np.abs(want), scale), 1e-300)
            over += int(np.sum(np.abs(got - want) > RTOL * den))
    finally:
        g.close()
        for m in (o, op, om):
            m.close()
    return worst_all, plain_all, over


@pytest.fixture(scope="module")
def headline():
    ws = W.generate(WL.RHS_NELEM, WL.RHS_NRIVER, seed=WL.RHS_SEED)
    return ws, WL.rhs_base_state(ws)


@pytest.mark.parametrize("via,first", [("device", 0), ("host", 3)])
def test_headline_mesh_against_oracle(headline, via, first):
    ws, base = headline
    states = [WL.rhs_state(base, k) for k in range(first, first + 3)]
    rng = np.random.default_rng(31 + first)
    ovl = rng.normal(0.0, 1e-3, 3 * ws.nelem)
    worst, plain, over = _run_sequence(ws, states, WL.rhs_forcing(ws), base[:ws.nelem], ovl, None, via)
    print(f"\n1M-element mesh via {via}: worst normalised error {worst:.3e} net of the last-bit envelope "
          f"(bar {RTOL:.0e}); without it {plain:.3e}, {over} of {3 * ws.neq} rows above 1e-12")


@pytest.mark.parametrize("via", ["device", "host"])
def test_scattered_point_mesh_against_oracle(via):
    """A 300,000-element Delaunay mesh of scattered nodes (irregular node
    degrees and element sizes, as a mesh generator's output), so the
    renumbering and the per-block queues are exercised on an unstructured
    adjacency."""
    ne = 300_000
    ws = W.generate(ne, WL.river_count(ne), seed=5, mesh="scattered")
    base = W.reference_state(ws, 6)
    states = [W.jitter(base, 600 + k) for k in range(3)]
    forcing = W.random_forcing(ws, 7)
    ovl = np.random.default_rng(78).normal(0.0, 1e-3, 3 * ne)
    worst, plain, over = _run_sequence(ws, states, forcing, base[:ne], ovl, None, via)
    print(f"\n300k-element scattered-node mesh via {via}: worst normalised error {worst:.3e} net of the last-bit "
          f"envelope (bar {RTOL:.0e}); without it {plain:.3e}, {over} of {3 * ws.neq} rows above 1e-12")


@pytest.mark.parametrize("via", ["device", "host"])
def test_flux_pihm_200k_against_oracle(via):
    ne = 200_000
    ws = W.generate(ne, WL.river_count(ne), seed=2)
    base = W.reference_state(ws, 3)
    states = [W.jitter(base, 500 + k) for k in range(3)]
    pcpdrp, edir, ett = W.random_forcing(ws, 5)
    rng = np.random.default_rng(77)
    ett = np.where(rng.random(ne) < 0.15, 0.0, ett)  # some elements without transpiration
    noah = W.noah_inputs(ws, 2, nlayers=4)
    ovl = rng.normal(0.0, 1e-3, 3 * ne)
    worst, plain, over = _run_sequence(ws, states, (pcpdrp, edir, ett), base[:ne], ovl, noah, via)
    print(f"\n200k-element Flux-PIHM mesh via {via}: worst normalised error {worst:.3e} net of the last-bit "
          f"envelope (bar {RTOL:.0e}); without it {plain:.3e}, {over} of {3 * ws.neq} rows above 1e-12")


def test_batch_with_a_large_watershed_matches_its_solo_runs():
    """A 100,000-element watershed beside two small ones: every watershed's
    trajectory in the batch is its solo trajectory on the single-watershed
    GPU path, bit for bit."""
    from backends import GpuBackend
    from pihm_gpu.batch import DONE, Batch, limits_for
    from pihm_gpu.solver import StepControl, run_steps
    nsteps = 3
    cases = []
    for ne, seed in ((100_000, 21), (1000, 22), (400, 23)):
        ws = W.generate(ne, WL.river_count(ne), seed=seed)
        pcp, edir, ett = WL.step_forcing(ws, nsteps, 60.0, seed=seed + 2)
        # the large one from the relaxed initial condition (RelaxIc), the
        # small ones from a wet perturbed state
        y0 = W.relax_state(ws) if ne > 10_000 else W.reference_state(ws, seed=seed)
        cases.append(dict(ws=ws, y0=y0, pcp=pcp, edir=edir, ett=ett,
                          outlet=int(np.where(ws.arrays["down"] < 0)[0][0]), ctrl=StepControl()))
    alone = []
    for c in cases:
        b = GpuBackend(c["ws"], c["y0"], c["pcp"], c["edir"], c["ett"])
        try:
            r = run_steps(b, c["ctrl"], nsteps, b.set_forcing, record_every=nsteps, outlet=c["outlet"])
        finally:
            b.close()
        alone.append(r)
    bt = Batch(limits_for([c["ws"] for c in cases], nsteps))
    try:
        ids = bt.add_many(cases, threads=3)
        assert None not in ids
        assert bt.step() == 0
        for i, c, want in zip(ids, cases, alone):
            assert bt.poll(i) == (DONE, 0)
            got = bt.result(i)
            assert np.array_equal(got["y"], want["states"][-1]), c["ws"].nelem
            assert np.array_equal(got["outlet"], want["outlet"]), c["ws"].nelem
            for k in ("nst", "nfe", "nni", "nli", "nfes"):
                assert getattr(got["stats"], k) == getattr(want["stats"], k), (c["ws"].nelem, k)
    finally:
        bt.close()
    print(f"\nbatch with 100,000 + 1,000 + 400 elements: bit-identical to solo runs "
          f"({int(alone[0]['stats'].nst)} integrator steps for the large one)")
