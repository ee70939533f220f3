"""The land-surface step on the GPU (pihm_gpu_land_*) against the reference's
golden vectors and the CPU restatement, and wired into the right-hand side
and the water balance.

Tolerance.  The kernel rounds every product and sum where the reference's C
does and evaluates exp, log and pow to about 0.51 ulp (almost always the
correctly rounded value the C library returns); cos is CUDA's (documented
within 2 ulp).  A field is compared element by element against

    |gpu - ref| <= LAND_RTOL * max(|ref|, LAND_FLOOR * max_k |ref_k|)

with LAND_RTOL = 1e-12: relative to the value, or, for values far below the
field's largest in the watershed (soil evaporation with the soil's
transpiration factor clamped at 1e-4, a canopy nearly dry), to a thousandth
of that largest value.  The share of elements that agree to the last bit is
reported as well.
"""
import numpy as np
import pytest

import pihm_gpu.land as L
import pihm_gpu.watershed as W
from parity import land_states
from test_land import FIELDS, _bits, golden_land, golden_steps

pytestmark = pytest.mark.gpu

LAND_RTOL = 1e-12
LAND_FLOOR = 1e-3


def _torch():
    import torch
    assert torch.cuda.is_available()
    return torch


def _state_on_device(g, ws, unsat, gw):
    """y with the given unsat and gw, on the device in internal order."""
    torch = _torch()
    y = np.zeros(ws.neq)
    ne = ws.nelem
    y[ne:2 * ne] = unsat
    y[2 * ne:3 * ne] = gw
    yr = torch.from_numpy(y).cuda()
    yi = torch.empty_like(yr)
    g.to_internal(yr.data_ptr(), yi.data_ptr())
    return yi, yr


def _check(got, want, label, stats):
    got, want = np.asarray(got), np.asarray(want)
    assert np.all(np.isfinite(want)), f"{label}: the expected values hold NaN or infinity"
    floor = LAND_FLOOR * np.max(np.abs(want)) if want.size else 0.0
    err = np.abs(got - want)
    lim = LAND_RTOL * np.maximum(np.abs(want), floor)
    bad = np.flatnonzero(~(err <= lim))
    exact = int(np.count_nonzero(_bits(got) == _bits(want)))
    stats["exact"] = stats.get("exact", 0) + exact
    stats["n"] = stats.get("n", 0) + got.size
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(lim > 0, err / np.maximum(np.abs(want), floor), np.where(err > 0, np.inf, 0.0))
    stats["worst"] = max(stats.get("worst", 0.0), float(np.max(rel)) if rel.size else 0.0)
    assert bad.size == 0, f"{label}: {bad.size} elements off, first {bad[0]}: got {got[bad[0]]!r} want {want[bad[0]]!r}"


def test_land_step_against_reference_golden():
    """48 land-surface steps from the reference's golden run (snow, rain,
    melt, interception, 14 land types, LAI series and monthly LAI)."""
    from pihm_gpu.capi import GpuRhs
    ws, land, z = golden_land()
    g = GpuRhs(ws)
    g.land_init(land)
    want_at = set(golden_steps(z))
    t, dt = int(z["start"]), float(z["lsm_step"])
    stats = {}
    for s, (unsat, gw) in enumerate(land_states(ws.arrays["depth"], 7, max(want_at))):
        yi, _ = _state_on_device(g, ws, unsat, gw)
        g.land_step(t, dt, yi.data_ptr())
        if s + 1 in want_at:
            for k in FIELDS:
                _check(g.land_get(k), z[f"s{s + 1}_{k}"], f"step {s + 1} {k}", stats)
        t += int(dt)
    print(f"land step vs reference: {stats['exact']}/{stats['n']} values bit-identical, "
          f"worst {stats['worst']:.2e} of the tolerance scale")


@pytest.mark.parametrize("seed", [0, 1])
def test_land_step_matches_oracle(seed):
    """A 40,000-element watershed with per-element parameters, 8 stations and 3
    LAI series over a day of steps, every field every step."""
    import oracle
    from pihm_gpu.capi import GpuRhs
    ws = W.generate(40000, 1000, seed=seed)
    land = L.synthetic_land(ws, seed=seed, hours=30, nstations=8, nlai=3)
    g = GpuRhs(ws)
    g.land_init(land)
    o = oracle.OracleLand(land, ws)
    t = L.epoch("2009-01-01 00:00")
    stats = {}
    for s, (unsat, gw) in enumerate(land_states(ws.arrays["depth"], 10 + seed, 96)):
        yi, _ = _state_on_device(g, ws, unsat, gw)
        g.land_step(t, 900.0, yi.data_ptr())
        assert o.step(t, 900.0, unsat, gw) == 0
        for k in FIELDS:
            _check(g.land_get(k), o.get(k), f"step {s} {k}", stats)
        t += 900
    print(f"land step vs restatement: {stats['exact']}/{stats['n']} values bit-identical, "
          f"worst {stats['worst']:.2e} of the tolerance scale")


def test_land_step_feeds_the_right_hand_side():
    """After a land-surface step the right-hand side reads its pcpdrp, edir and
    ett: the GPU evaluation equals the restatement given the same forcing,
    within the 1e-12 row bar net of the reference's own last-bit envelope
    (tests/parity.py: the restatement with every pow and log moved one ulp
    up plus the same moved down, as the scale tests take it).  The relaxed state puts full soil columns next to a water
    table at the column's top, where Psi's pow(1/satn, m) - 1 cancels: one
    ulp of pow moves such a row by up to 5e-8 of its terms in the reference
    itself."""
    import oracle
    from parity import compare, row_scales
    from pihm_gpu.capi import GpuRhs
    ws = W.generate(5000, 300, seed=3)
    land = L.synthetic_land(ws, seed=3, hours=24)
    g = GpuRhs(ws)
    g.land_init(land)
    t = L.epoch("2009-01-01 06:00")
    ne = ws.nelem
    y = W.relax_state(ws)
    yi, yr = _state_on_device(g, ws, y[ne:2 * ne], y[2 * ne:3 * ne])
    # the full state, not only unsat and gw
    torch = _torch()
    yr.copy_(torch.from_numpy(y))
    g.to_internal(yr.data_ptr(), yi.data_ptr())
    g.land_step(t, 900.0, yi.data_ptr())
    forcing = {k: g.land_get(k) for k in ("pcpdrp", "edir", "ett")}
    outs = {}
    for p in (0, 1, -1):
        o = oracle.Oracle(ws)
        o.set_ulp_perturb(p)
        o.set_forcing(forcing["pcpdrp"], forcing["edir"], forcing["ett"])
        outs[p], rc = o.rhs(y)
        assert rc == 0
        if p == 0:
            scale = row_scales(ws, o.fluxes(), forcing["pcpdrp"], forcing["edir"], forcing["ett"])
        o.close()
    want = outs[0]
    env = np.abs(outs[1] - want) + np.abs(outs[-1] - want)
    got, rc = g.rhs_host(y)
    assert rc == 0
    ok, worst, idx = compare(got, want, scale, envelope=env)
    plain = compare(got, want, scale)[1]
    print(f"land-forced right-hand side: worst {worst:.3e} net of the envelope, {plain:.3e} without it")
    assert ok, f"worst {worst:.3e} at {idx} (envelope {env[idx]:.3e})"
    assert np.count_nonzero(forcing["pcpdrp"]) > 0 and np.count_nonzero(forcing["edir"]) > 0


def test_water_balance_counts_canopy_and_snow():
    """With the land-surface model attached the water balance takes
    precipitation, canopy evaporation, canopy storage and snow from it."""
    from pihm_gpu.capi import GpuRhs
    ws = W.generate(5000, 300, seed=4)
    land = L.synthetic_land(ws, seed=4, hours=48)
    g = GpuRhs(ws)
    g.land_init(land)
    ne, nr = ws.nelem, ws.nriver
    y = W.relax_state(ws)
    yi, yr = _state_on_device(g, ws, y[ne:2 * ne], y[2 * ne:3 * ne])
    torch = _torch()
    yr.copy_(torch.from_numpy(y))
    g.to_internal(yr.data_ptr(), yi.data_ptr())
    t = L.epoch("2009-01-01 00:00")
    for s in range(24):  # build up canopy storage and snow
        g.land_step(t + 900 * s, 900.0, yi.data_ptr())
    f = {k: g.land_get(k) for k in FIELDS}
    assert np.count_nonzero(f["sneqv"]) > 0 and np.count_nonzero(f["cmc"]) > 0
    _, rc = g.rhs_host(y)  # river fluxes for the outlet term
    assert rc == 0
    wb = g.water_balance(yi.data_ptr(), 60.0)
    a = ws.arrays
    area, por = np.asarray(a["area"]), np.asarray(a["porosity"])
    src = np.sum(f["prcp"] * area * 60.0)
    rivflow = g.fluxes()["rivflow"].reshape(nr, 11)  # DOWN_CHANL2CHANL is slot 1
    outlet = np.asarray(a["down"]) < 0
    snk = np.sum((f["edir"] + f["ett"] + f["ec"]) * area * 60.0) + np.sum(rivflow[outlet, 1] * 60.0)
    strg = np.sum((f["cmc"] + f["sneqv"] + y[:ne] + (y[ne:2 * ne] + y[2 * ne:3 * ne]) * por) * area)
    strg += np.sum((y[3 * ne:3 * ne + nr] + y[3 * ne + nr:] * np.asarray(a["riv_porosity"])) *
                   np.asarray(a["riv_area"]))
    assert np.allclose(wb, [src, snk, strg], rtol=1e-12, atol=0.0), (wb, (src, snk, strg))


def test_land_errors():
    from pihm_gpu.capi import GpuRhs, PihmGpuError
    ws = W.generate(1000, 100, seed=2)
    land = L.synthetic_land(ws, seed=2, hours=24)
    g = GpuRhs(ws)
    torch = _torch()
    y = torch.zeros(ws.neq, dtype=torch.float64, device="cuda")
    with pytest.raises(PihmGpuError):  # no model attached
        g.land_step(L.epoch("2009-01-01 00:00"), 900.0, y.data_ptr())
    bad = L.synthetic_land(ws, seed=2, hours=24)
    bad.params["lc_type"] = bad.params["lc_type"].copy()
    bad.params["lc_type"][5] = L.NLC + 1
    with pytest.raises(PihmGpuError):
        g.land_init(bad)
    bad = L.synthetic_land(ws, seed=2, hours=24)
    bad.meteo_time = bad.meteo_time.copy()
    bad.meteo_time[3], bad.meteo_time[4] = bad.meteo_time[4], bad.meteo_time[3]
    with pytest.raises(PihmGpuError):
        g.land_init(bad)
    g.land_init(land)
    lo, hi = land.time_range()
    with pytest.raises(PihmGpuError):
        g.land_step(hi + 1, 900.0, y.data_ptr())
    with pytest.raises(PihmGpuError):
        g.land_step(lo - 1, 900.0, y.data_ptr())
    g.land_step(hi, 900.0, y.data_ptr())
    assert g.status() == 0
