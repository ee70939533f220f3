"""Shared helpers of the parity tests: scenarios and the tolerance.

Tolerance.  The target is ydot within 1e-12 relative of the reference.  A
derivative is a sum of fluxes that can cancel, and two correct libms differ by
an ulp or two, so each row is compared against the magnitude of the terms that
make it up (the row's "scale"):

    |gpu - ref| <= RTOL * max(|ref|, scale),   RTOL = 1e-12

with scale = sum of |terms| of that row, e.g. for the surface row
|pcpdrp| + |infil| + |edir_surf| + sum_j |ovlflow_j| / area
(src/ode.c:111-209 and :228-300 for the row definitions).

Recharge is itself a difference: kavg (0.5 deficit + Psi) / (0.5 depth)
(src/vert_flow.c:132-170), and near equilibrium 0.5 deficit + Psi cancels by
up to four orders of magnitude.  A Psi one ulp away from the reference's --
what two correct libms' pow can give -- then moves the unsaturated and
groundwater rows by up to 3.4e-12 of their terms on the 1M-element benchmark
mesh (measured by perturbing the restatement's Psi by one ulp).  When the
state is passed, Recharge's term therefore counts with the magnitude of its
two addends, kavg (0.5 deficit + |Psi|) / (0.5 depth) (recharge_magnitude);
everywhere else the scale is unchanged.
"""
from __future__ import annotations

import numpy as np

RTOL = 1e-12


SATMIN = 0.1  # src/include/pihm_const.h


def recharge_magnitude(ws, y, rechg):
    """|Recharge| counted by its two addends where Recharge evaluates its
    own gradient: kavg (0.5 deficit + |Psi|) / (0.5 depth), with Psi,
    KrFunc and AvgKv (arithmetic mean) as src/vert_flow.c:132-209 and
    src/soil.c:8-13 form them (numpy's pow: this is a tolerance scale, not
    a result); |rechg| elsewhere (water table within the infiltration
    depth, where Recharge equals Infil)."""
    a = ws.arrays
    ne = ws.nelem
    y = np.asarray(y, np.float64)
    unsat = np.maximum(y[ne:2 * ne], 0.0)
    gw = np.maximum(y[2 * ne:3 * ne], 0.0)
    depth, dinf, beta, alpha = a["depth"], a["dinf"], a["beta"], a["alpha"]
    ksatv, dmac, kmacv, areafh = a["ksatv"], a["dmac"], a["kmacv"], a["areafh"]
    own = ~(gw > depth - dinf)
    deficit = depth - gw
    with np.errstate(all="ignore"):
        satn = np.clip(unsat / deficit, SATMIN, 1.0)
        m = beta / (beta - 1.0)
        psi = -np.power(np.power(1.0 / satn, m) - 1.0, 1.0 / beta) / alpha
        kr = np.sqrt(satn) * (1.0 - np.power(1.0 - np.power(satn, m), (beta - 1.0) / beta)) ** 2
        deep = deficit > dmac
        k2 = np.where(deep, kr * ksatv, np.where(areafh > 0.0, kmacv * areafh + ksatv * (1.0 - areafh), ksatv))
        d1 = np.where(deep, dmac, deficit)
        d2 = np.where(deep, deficit - dmac, dmac - deficit)
        d3 = np.where(deep, gw, gw - (dmac - deficit))
        kavg = (kr * ksatv * d1 + k2 * d2 + ksatv * d3) / (d1 + d2 + d3)
        mag = np.abs(kavg) * (0.5 * deficit + np.abs(psi)) / (0.5 * depth)
    mag = np.where(np.isfinite(mag), mag, 0.0)
    r = np.abs(np.asarray(rechg, np.float64))
    return np.where(own, np.maximum(r, mag), r)


def row_scales(ws, fx, pcpdrp, edir, ett, y=None):
    """Sum of |terms| of every ydot row, from a flux set (oracle diagnostics);
    with the state y, Recharge counts by its addends (recharge_magnitude)."""
    a = ws.arrays
    ne, nr = ws.nelem, ws.nriver
    area = a["area"]
    por = a["porosity"]
    ovl = np.abs(fx["ovlflow"].reshape(ne, 3)).sum(1)
    sub = np.abs(fx["subsurf"].reshape(ne, 3)).sum(1)
    et = np.abs(fx["et_split"].reshape(ne, 5))
    infil = np.abs(fx["infil"])
    rechg = np.abs(fx["rechg"]) if y is None else recharge_magnitude(ws, y, fx["rechg"])
    s_surf = np.abs(pcpdrp) + infil + et[:, 0] + ovl / area
    s_unsat = (infil + rechg + et[:, 1] + et[:, 3]) / por
    s_gw = (rechg + et[:, 2] + et[:, 4] + sub / area) / por
    rf = np.abs(fx["rivflow"].reshape(nr, 11))
    s_stage = rf[:, 0:7].sum(1) / a["riv_area"]
    s_rgw = (rf[:, 7] + rf[:, 8] + rf[:, 9] + rf[:, 10] + rf[:, 6]) / (
        a["riv_porosity"] * a["riv_area"])
    return np.concatenate([s_surf, s_unsat, s_gw, s_stage, s_rgw])


def compare(got, want, scale, rtol=RTOL):
    """Returns (ok, worst normalised error, index)."""
    den = np.maximum(np.abs(want), scale)
    den = np.where(den > 0, den, 1.0)
    err = np.abs(got - want) / den
    err = np.where(got == want, 0.0, err)
    k = int(np.argmax(err)) if err.size else 0
    worst = float(err[k]) if err.size else 0.0
    return bool(worst <= rtol and np.all(np.isfinite(got) == np.isfinite(want))), worst, k


def scenario(ws, seed: int, bc: bool = False, noah: bool = False):
    """A reproducible single-call scenario: state, forcing, carried values and
    (optionally) Dirichlet / Neumann boundary edges and river inflow BCs.
    Returns (watershed, scenario); with bc=True the watershed is a copy whose
    boundary types were changed."""
    import copy
    import pihm_gpu.watershed as W
    if bc:
        ws = copy.deepcopy(ws)
    rng = np.random.default_rng(1000 + seed)
    y = W.jitter(W.reference_state(ws, seed), seed + 1)
    pcpdrp, edir, ett = W.random_forcing(ws, seed + 2)
    ne = ws.nelem
    ws0 = y[:ne] * rng.uniform(0.5, 1.5, ne)
    ovl = rng.normal(0.0, 1e-3, 3 * ne)
    elem_bc = None
    river_bc = None
    if bc:
        elem_bc = np.zeros(3 * ne)
        nabr = ws.arrays["nabr"]
        bct = ws.arrays["bc_type"].reshape(-1)
        bnd = np.where(nabr.reshape(-1) == 0)[0]
        kind = rng.integers(0, 3, bnd.size)  # 0 no-flow, 1 Dirichlet, 2 Neumann
        bct[bnd] = np.where(kind == 1, 1, np.where(kind == 2, -1, 0))
        zmin = np.repeat(ws.arrays["zmin"], 3)
        depth = np.repeat(ws.arrays["depth"], 3)
        elem_bc[bnd] = np.where(kind == 1, zmin[bnd] + depth[bnd] * rng.uniform(0.1, 1.0, bnd.size),
                                np.where(kind == 2, rng.normal(0, 1e-4, bnd.size), 0.0))
        rbct = ws.arrays["riverbc_type"]
        nr = ws.nriver
        rk = rng.integers(0, 3, nr)
        rbct[:] = np.where(rk == 1, 1, np.where(rk == 2, -1, 0))
        # Dirichlet heads stay below the bed: the reference's BoundFluxRiver
        # takes sqrt of the head gradient (src/river_flow.c:410-413), which is
        # NaN for inflow, and the reference then exits
        river_bc = np.where(rk == 1, ws.arrays["riv_zbed"] - rng.uniform(0.1, 1.0, nr),
                            np.where(rk == 2, rng.normal(0, 0.01, nr), 0.0))
    sc = dict(y=y, pcpdrp=pcpdrp, edir=edir, ett=ett, ws0=ws0, ovl=ovl,
              elem_bc=elem_bc, river_bc=river_bc)
    if noah:
        # Flux-PIHM: Noah's per-step inputs; some elements without transpiration
        sc["noah"] = W.noah_inputs(ws, seed)
        sc["ett"] = np.where(rng.random(ne) < 0.15, 0.0, ett)
    return ws, sc


def apply(model, sc):
    if sc.get("noah") is not None:
        model.set_noah(sc["noah"])
    model.set_forcing(sc["pcpdrp"], sc["edir"], sc["ett"])
    model.set_ws0_surf(sc["ws0"])
    model.set_river_edge_ovlflow(sc["ovl"])
    if sc["elem_bc"] is not None or sc["river_bc"] is not None:
        model.set_bc(sc["elem_bc"], sc["river_bc"])


def land_states(depth, seed: int, nsteps: int):
    """Soil states (unsat, gw) for a sequence of land-surface steps: the water
    table anywhere in the column, the unsaturated store from slightly negative
    to above the column's capacity, so that every branch of the soil
    saturation in IntcpSnowEt (src/is_sm_et.c:103-118) is taken."""
    depth = np.asarray(depth, np.float64)
    rng = np.random.default_rng(seed)
    for _ in range(nsteps):
        gw = depth * rng.uniform(0.0, 1.0, depth.size)
        unsat = (depth - gw) * rng.uniform(-0.1, 1.2, depth.size)
        yield unsat, gw


def land_deck(directory: str, seed: int = 11, land_seed: int = 5, hours: int = 96):
    """Write a generated 1,000-element deck with a seeded land-surface model
    (pihm_gpu.land.synthetic_land, per-type canopy parameters, hourly forcing
    with snow, rain and melt, LSM_STEP 900 s) to <directory>/input/gen; returns
    that path."""
    import datetime
    import os

    import pihm_gpu.land as L
    import pihm_gpu.watershed as W
    from pihm_gpu import deck as D
    ws = W.generate(1000, 100, seed=seed)
    land = L.synthetic_land(ws, seed=land_seed, hours=hours, per_type=True)
    rng = np.random.default_rng(0)
    lc = land.params["lc_type"]
    rough_t = np.round(rng.uniform(0.02, 0.3, L.NLC), 3)
    rzd_t = np.round(rng.uniform(0.3, 1.5, L.NLC), 2)
    ws.arrays["rough"] = rough_t[lc - 1]
    ws.arrays["rzd"] = rzd_t[lc - 1]
    path = os.path.join(directory, "input", "gen")
    end = L.epoch("2009-01-01 00:00") + 3600 * hours
    end_s = datetime.datetime.fromtimestamp(end, datetime.timezone.utc).strftime("%Y-%m-%d %H:%M")
    D.write_deck(ws, path, "gen", land=land, lsm_step=900, start="2009-01-01 00:00", end=end_s)
    return path
