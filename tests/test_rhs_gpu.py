"""GPU right-hand side against the CPU oracle (same inputs, reference order)."""
import numpy as np
import pytest

import pihm_gpu.watershed as W
from parity import RTOL, apply, compare, row_scales, scenario

pytestmark = pytest.mark.gpu


def _pair(ws, order=1):
    from oracle import Oracle
    from pihm_gpu.capi import GpuRhs
    return Oracle(ws), GpuRhs(ws, order=order)


def _check_call(o, g, ws, sc, calls=3, label=""):
    y = sc["y"]
    for k in range(calls):
        yk = W.jitter(y, 77 + k) if k else y
        want, rc_o = o.rhs(yk)
        got, rc_g = g.rhs_host(yk)
        assert rc_o == 0 and rc_g == 0
        fx = o.fluxes()
        scale = row_scales(ws, fx, sc["pcpdrp"], sc["edir"], sc["ett"])
        ok, worst, idx = compare(got, want, scale)
        assert ok, f"{label} call {k}: worst {worst:.3e} at {idx} got {got[idx]!r} want {want[idx]!r}"


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_c0_parity(seed, order):
    ws = W.generate(1000, 100, seed=seed)
    ws, sc = scenario(ws, seed)
    o, g = _pair(ws, order)
    apply(o, sc)
    apply(g, sc)
    _check_call(o, g, ws, sc, label=f"seed {seed}")


def test_boundary_conditions():
    ws = W.generate(1000, 100, seed=5)
    ws, sc = scenario(ws, 5, bc=True)
    o, g = _pair(ws)
    apply(o, sc)
    apply(g, sc)
    _check_call(o, g, ws, sc, label="bc")


@pytest.mark.parametrize("surf_mode,riv_mode", [(1, 1), (1, 2), (2, 1)])
def test_kinematic_modes(surf_mode, riv_mode):
    ws = W.generate(1000, 100, seed=7)
    ws.surf_mode, ws.riv_mode = surf_mode, riv_mode
    ws, sc = scenario(ws, 7)
    o, g = _pair(ws)
    apply(o, sc)
    apply(g, sc)
    _check_call(o, g, ws, sc, label=f"modes {surf_mode}{riv_mode}")


def test_fluxes_match():
    ws = W.generate(1000, 100, seed=3)
    ws, sc = scenario(ws, 3)
    o, g = _pair(ws)
    apply(o, sc)
    apply(g, sc)
    g.set_diagnostics(True)
    o.rhs(sc["y"])
    g.rhs_host(sc["y"])
    fo, fg = o.fluxes(), g.fluxes()
    for k in fo:
        a, b = fg[k], fo[k]
        den = np.maximum(np.abs(b), np.abs(b).max() * 1e-3)
        err = np.abs(a - b) / np.where(den > 0, den, 1)
        assert err.max() <= 1e-11, (k, err.max(), int(err.argmax()))


def test_device_path_internal_order():
    """pihm_gpu_rhs on device pointers in internal order agrees with the
    host-buffer path after reordering."""
    import torch
    ws = W.generate(1000, 100, seed=11)
    ws, sc = scenario(ws, 11)
    o, g = _pair(ws)
    apply(o, sc)
    apply(g, sc)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    g.set_stream(stream.cuda_stream)
    y_ref = torch.from_numpy(sc["y"]).to(dev)
    y_int = torch.empty_like(y_ref)
    yd_int = torch.empty_like(y_ref)
    yd_ref = torch.empty_like(y_ref)
    g.to_internal(y_ref.data_ptr(), y_int.data_ptr())
    g.rhs_device(y_int.data_ptr(), yd_int.data_ptr())
    g.to_reference(yd_int.data_ptr(), yd_ref.data_ptr())
    assert g.status() == 0
    got = yd_ref.cpu().numpy()
    want, _ = o.rhs(sc["y"])
    scale = row_scales(ws, o.fluxes(), sc["pcpdrp"], sc["edir"], sc["ett"])
    ok, worst, idx = compare(got, want, scale)
    assert ok, (worst, idx)
    # permutation round trip is exact
    back = torch.empty_like(y_ref)
    g.to_reference(y_int.data_ptr(), back.data_ptr())
    assert torch.equal(back, y_ref)


def test_nan_reports_error_without_exit():
    """An upstream Dirichlet head above the water surface makes the
    reference's BoundFluxRiver take sqrt of a negative gradient
    (src/river_flow.c:410-413) and exit through CheckDy; the library reports
    PIHM_GPU_ERR_NAN and stays usable."""
    import copy
    ws = copy.deepcopy(W.generate(1000, 100, seed=2))
    ws.arrays["riverbc_type"][0] = 1
    river_bc = np.zeros(ws.nriver)
    river_bc[0] = ws.arrays["riv_zbed"][0] + 50.0
    ws, sc = scenario(ws, 2)
    o, g = _pair(ws)
    apply(o, sc)
    apply(g, sc)
    o.set_bc(None, river_bc)
    g.set_bc(None, river_bc)
    _, rc_o = o.rhs(sc["y"])
    _, rc_g = g.rhs_host(sc["y"])
    assert rc_o == -3 and rc_g == -3
    # context still usable: clear the bad boundary and evaluate again
    o.set_bc(None, np.zeros(ws.nriver))
    g.set_bc(None, np.zeros(ws.nriver))
    want, rc_o = o.rhs(sc["y"])
    got, rc_g = g.rhs_host(sc["y"])
    assert rc_o == 0 and rc_g == 0


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_flux_pihm_noah_variant(seed):
    """Flux-PIHM right-hand side (Noah's per-step inputs) against the oracle,
    which is pinned bit for bit to the reference built with _NOAH_."""
    ws = W.generate(1000, 100, seed=seed)
    ws, sc = scenario(ws, seed, noah=True)
    o, g = _pair(ws)
    apply(o, sc)
    apply(g, sc)
    _check_call(o, g, ws, sc, label=f"noah seed {seed}")


def test_flux_pihm_noah_reference_goldens():
    """The GPU Flux-PIHM right-hand side against the reference's own _NOAH_
    build (tests/golden/c0_noah_calls.npz)."""
    import os
    from oracle import Oracle
    from pihm_gpu.capi import GpuRhs
    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    ws = W.Watershed.load(os.path.join(gold, "c0_watershed.npz"))
    z = np.load(os.path.join(gold, "c0_noah_calls.npz"))
    for seed in range(3):
        tag = f"n{seed}"
        noah = {k: z[f"{tag}_noah_{k}"] for k in ("et", "nwtbl", "nroot", "sh2o0", "smcmin", "smcmax", "fcr")}
        g, o = GpuRhs(ws), Oracle(ws)
        for m in (g, o):
            m.set_noah(noah)
            m.set_forcing(z[f"{tag}_pcpdrp"], z[f"{tag}_edir"], z[f"{tag}_ett"])
            m.set_ws0_surf(z[f"{tag}_ws0"])
            m.set_river_edge_ovlflow(z[f"{tag}_ovl"])
        for c in range(3):
            y = z[f"{tag}_call{c}_y"]
            got, rc = g.rhs_host(y)
            _, _ = o.rhs(y)
            assert rc == 0
            scale = row_scales(ws, o.fluxes(), z[f"{tag}_pcpdrp"], z[f"{tag}_edir"], z[f"{tag}_ett"])
            ok, worst, idx = compare(got, z[f"{tag}_call{c}_ydot"], scale)
            assert ok, f"{tag} call {c}: worst {worst:.3e} at {idx}"


def test_host_path_direct_equals_copy():
    """pihm_gpu_rhs_host on pinned host buffers: the reordering kernels read y
    from and write ydot to host memory directly, and the result is the copy
    path's bit for bit and meets the oracle.  Pageable arrays take the direct
    path only on a device with pageable-memory access, with the same bits."""
    import torch
    ws = W.generate(1000, 100, seed=4)
    ws, sc = scenario(ws, 4)
    o, g = _pair(ws)
    y = torch.from_numpy(sc["y"]).pin_memory()
    out = {}
    for mode in (0, 1):
        apply(g, sc)  # the same carried river-edge flux before each call
        res = torch.empty_like(y).pin_memory()
        g.set_host_path(mode)
        assert g.rhs_host_ptr(y.data_ptr(), res.data_ptr()) == 0
        direct, pageable = g.host_path_info()
        assert direct == (mode == 0)  # pinned buffers are always addressable
        out[mode] = res.numpy().copy()
    assert np.array_equal(out[0], out[1])
    apply(o, sc)
    want, rc = o.rhs(sc["y"])
    assert rc == 0
    ok, worst, idx = compare(out[0], want, row_scales(ws, o.fluxes(), sc["pcpdrp"], sc["edir"], sc["ett"]))
    assert ok, (worst, idx)
    apply(g, sc)
    g.set_host_path(0)
    got, rc = g.rhs_host(sc["y"])  # pageable numpy arrays
    assert rc == 0 and g.host_path_info()[0] == pageable
    assert np.array_equal(got, out[1])


def test_deck_mesh_straight_to_gpu(tmp_path):
    """A deck read by the library, its pihm_gpu_mesh handed straight to
    pihm_gpu_create as a C caller does, evaluated at the deck's initial
    state: the oracle's result on the same arrays, within the parity bar."""
    import ctypes
    from oracle import Oracle
    from pihm_gpu import capi, deck
    from pihm_gpu.meshdesc import MeshDesc, f64p
    d = tmp_path / "input" / "gen"
    deck.write_deck(W.generate(1000, 100, seed=9), str(d), "gen")
    dk = deck.Deck.read(str(d), "gen")
    ws = dk.watershed()
    y0 = dk.initial_state()
    pcpdrp, edir, ett = W.random_forcing(ws, 9)
    ws0 = np.ascontiguousarray(y0[:ws.nelem])
    lib = capi.load()
    m = MeshDesc()
    assert dk.lib.pihm_deck_mesh(dk.h, ctypes.byref(m)) == 0
    h = ctypes.c_void_p()
    assert lib.pihm_gpu_create(ctypes.byref(m), ws.surf_mode, ws.riv_mode, ws.stepsize, capi.ORDER_RCM,
                               ctypes.byref(h)) == 0
    try:
        assert lib.pihm_gpu_set_forcing(h, f64p(pcpdrp), f64p(edir), f64p(ett)) == 0
        assert lib.pihm_gpu_set_ws0_surf(h, f64p(ws0)) == 0
        got = np.empty_like(y0)
        assert lib.pihm_gpu_rhs_host(h, 0.0, f64p(y0), f64p(got)) == 0
    finally:
        lib.pihm_gpu_destroy(h)
    o = Oracle(ws)
    o.set_forcing(pcpdrp, edir, ett)
    o.set_ws0_surf(ws0)
    want, rc = o.rhs(y0)
    assert rc == 0
    ok, worst, idx = compare(got, want, row_scales(ws, o.fluxes(), pcpdrp, edir, ett))
    assert ok, (worst, idx)


def test_element_kernel_shapes_give_the_same_bits():
    """k_elem_main's three block shapes (512 x 2, 256 x 4, 128 x 8 per SM)
    evaluate identical derivatives, over three consecutive calls (the carried
    river-edge flux included), on a 60,000-element mesh."""
    import torch
    from pihm_gpu import workloads as WL
    from pihm_gpu.capi import GpuRhs
    ws = W.generate(60_000, WL.river_count(60_000), seed=12)
    y0 = W.reference_state(ws, 12)
    pcp, edir, ett = W.random_forcing(ws, 12)
    dev = torch.device("cuda", 0)
    out = []
    for shape in (0, 1, 2):
        g = GpuRhs(ws)
        g.set_kernel_shape(shape)
        g.set_forcing(pcp, edir, ett)
        g.set_ws0_surf(y0[:ws.nelem])
        y_ref = torch.from_numpy(y0).to(dev)
        y = torch.empty_like(y_ref)
        g.to_internal(y_ref.data_ptr(), y.data_ptr())
        calls = []
        for k in range(3):
            yk = y * (1.0 + 0.01 * k)
            yd = torch.empty_like(y)
            torch.cuda.synchronize()
            g.rhs_device(yk.data_ptr(), yd.data_ptr())
            torch.cuda.synchronize()
            calls.append(yd.cpu().numpy())
        assert g.status() == 0
        g.close()
        out.append(calls)
    for shape in (1, 2):
        for k in range(3):
            assert np.array_equal(out[shape][k], out[0][k]), (shape, k)


@pytest.mark.parametrize("depth", [1, 3])
@pytest.mark.parametrize("host_path", [0, 1])
def test_async_host_evaluations_on_two_contexts_match_sync(depth, host_path):
    """pihm_gpu_rhs_host_async on two contexts of one mesh, each on its own
    stream, alternating states (pinned buffers; the direct host path, or the
    copy path with its alternating staging pairs and copy streams), with one
    or several evaluations queued per context before a wait: each derivative
    equals the synchronous evaluation of the same state on a context with the
    same call history."""
    import ctypes
    import torch
    from pihm_gpu import workloads as WL
    from pihm_gpu.capi import GpuRhs
    ws = W.generate(20_000, WL.river_count(20_000), seed=14)
    base = W.reference_state(ws, 14)
    forcing = W.random_forcing(ws, 14)
    states = [W.jitter(base, 900 + k) for k in range(6)]
    f64p = ctypes.POINTER(ctypes.c_double)

    def ctx(stream=None):
        g = GpuRhs(ws, stream=stream)
        g.set_forcing(*forcing)
        g.set_ws0_surf(base[:ws.nelem])
        return g

    # synchronous reference: context k % 2 evaluates states k in order
    want = []
    refs = [ctx(), ctx()]
    for k, y in enumerate(states):
        got, rc = refs[k % 2].rhs_host(y)
        assert rc == 0
        want.append(got)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    gs = [ctx(s1.cuda_stream), ctx(s2.cuda_stream)]
    for g in gs:
        g.set_host_path(host_path)
    yh = [torch.from_numpy(y).pin_memory() for y in states]
    ydh = [torch.empty(ws.neq, dtype=torch.float64).pin_memory() for _ in states]
    lib = gs[0].lib
    queued = [0, 0]
    for k in range(len(states)):
        if queued[k % 2] >= depth:
            assert lib.pihm_gpu_wait(gs[k % 2].h) == 0
            queued[k % 2] = 0
        queued[k % 2] += 1
        assert lib.pihm_gpu_rhs_host_async(gs[k % 2].h, 0.0, ctypes.cast(yh[k].data_ptr(), f64p),
                                           ctypes.cast(ydh[k].data_ptr(), f64p)) == 0
    for g in gs:
        assert lib.pihm_gpu_wait(g.h) == 0
    for k in range(len(states)):
        assert np.array_equal(ydh[k].numpy(), want[k]), k
    for g in gs + refs:
        g.close()


def test_async_host_paths_switched_with_evaluations_in_flight():
    """One context queues evaluations on the copy path, switches to the
    direct path and queues more before waiting: the copy path stages through
    buffers of its own, so every derivative equals the synchronous
    evaluation of the same state in the same order."""
    import ctypes
    import torch
    from pihm_gpu import workloads as WL
    from pihm_gpu.capi import GpuRhs
    ws = W.generate(20_000, WL.river_count(20_000), seed=15)
    base = W.reference_state(ws, 15)
    forcing = W.random_forcing(ws, 15)
    states = [W.jitter(base, 950 + k) for k in range(6)]
    f64p = ctypes.POINTER(ctypes.c_double)

    def ctx(stream=None):
        g = GpuRhs(ws, stream=stream)
        g.set_forcing(*forcing)
        g.set_ws0_surf(base[:ws.nelem])
        return g

    ref = ctx()
    want = []
    for y in states:
        got, rc = ref.rhs_host(y)
        assert rc == 0
        want.append(got)
    st = torch.cuda.Stream()
    g = ctx(st.cuda_stream)
    yh = [torch.from_numpy(y).pin_memory() for y in states]
    ydh = [torch.empty(ws.neq, dtype=torch.float64).pin_memory() for _ in states]
    for k in range(len(states)):
        g.set_host_path(1 if k % 3 != 2 else 0)
        assert g.lib.pihm_gpu_rhs_host_async(g.h, 0.0, ctypes.cast(yh[k].data_ptr(), f64p),
                                             ctypes.cast(ydh[k].data_ptr(), f64p)) == 0
    assert g.lib.pihm_gpu_wait(g.h) == 0
    for k in range(len(states)):
        assert np.array_equal(ydh[k].numpy(), want[k]), k
    for c in (g, ref):
        c.close()
