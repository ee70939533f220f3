"""Shared helpers of the parity tests: scenarios and the tolerance.

Tolerance.  The target is ydot within 1e-12 relative of the reference.  A
derivative is a sum of fluxes that can cancel, and two correct libms differ by
an ulp or two, so each row is compared against the magnitude of the terms that
make it up (the row's "scale"):

    |gpu - ref| <= RTOL * max(|ref|, scale),   RTOL = 1e-12

with scale = sum of |terms| of that row, e.g. for the surface row
|pcpdrp| + |infil| + |edir_surf| + sum_j |ovlflow_j| / area
(src/ode.c:111-209 and :228-300 for the row definitions).

Some terms are themselves computed as differences that cancel: Recharge's
head gradient 0.5 deficit + Psi near equilibrium (src/vert_flow.c:132-170),
KrFunc's 1 - (1 - satn^m)^e at low saturation (src/soil.c:8-13), Infil's
surfh + zmax - (Psi + zmax - 0.5 dinf).  There the reference's own roundings
fix the result only to a few parts in 1e12: a power one ulp away from
glibc's -- what any other correct libm may return -- moves such a row by up to
a few times 1e-12 of its terms on the 1M-element benchmark mesh.  Where a test
passes an envelope, the bar of each row is widened by it:

    |gpu - ref| <= RTOL * max(|ref|, scale) + envelope,

envelope = |ref(+1 ulp) - ref| + |ref(-1 ulp) - ref|, the movement of the
reference's result when every pow() and log() it evaluates is moved by one
unit in the last place up, then down (Oracle.set_ulp_perturb, the same
calls, the same state).  Rows that are not sensitive keep the 1e-12 bar.
"""
from __future__ import annotations

import numpy as np

RTOL = 1e-12


def row_scales(ws, fx, pcpdrp, edir, ett):
    """Sum of |terms| of every ydot row, from a flux set (oracle diagnostics)."""
    a = ws.arrays
    ne, nr = ws.nelem, ws.nriver
    area = a["area"]
    por = a["porosity"]
    ovl = np.abs(fx["ovlflow"].reshape(ne, 3)).sum(1)
    sub = np.abs(fx["subsurf"].reshape(ne, 3)).sum(1)
    et = np.abs(fx["et_split"].reshape(ne, 5))
    infil = np.abs(fx["infil"])
    rechg = np.abs(fx["rechg"])
    s_surf = np.abs(pcpdrp) + infil + et[:, 0] + ovl / area
    s_unsat = (infil + rechg + et[:, 1] + et[:, 3]) / por
    s_gw = (rechg + et[:, 2] + et[:, 4] + sub / area) / por
    rf = np.abs(fx["rivflow"].reshape(nr, 11))
    s_stage = rf[:, 0:7].sum(1) / a["riv_area"]
    s_rgw = (rf[:, 7] + rf[:, 8] + rf[:, 9] + rf[:, 10] + rf[:, 6]) / (
        a["riv_porosity"] * a["riv_area"])
    return np.concatenate([s_surf, s_unsat, s_gw, s_stage, s_rgw])


def compare(got, want, scale, rtol=RTOL, envelope=None):
    """Returns (ok, worst normalised error, index).  With an envelope (the
    reference's last-bit movement, see above) a row's error is counted net
    of it."""
    den = np.maximum(np.abs(want), scale)
    den = np.where(den > 0, den, 1.0)
    diff = np.abs(got - want)
    if envelope is not None:
        diff = np.maximum(diff - envelope, 0.0)
    err = diff / den
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
