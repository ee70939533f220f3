"""Golden vectors of the land-surface step from the reference itself: its
ReadAlloc + Initialize on a generated deck with a seeded land-surface model
(tests/parity.py land_deck: hourly forcing with snow, rain and melt, 14 land
types, LAI series and monthly LAI, LSM_STEP 900 s), then its ApplyForc +
IntcpSnowEt (src/forcing.c:44-87, src/is_sm_et.c:5-226) for 48 steps from
the deck's start, the soil state of every step from tests/parity.py
land_states(depth, seed 7).

    python tests/golden/make_golden_land.py [--reference /path/to/PIHM-CUDA]

writes tests/golden/land_watershed.npz (the deck's mesh as the library's
reader gives it, bit for bit the reference's) and tests/golden/land_calls.npz:
the land-surface parameters as the reference's Initialize leaves them, the
forcing series, and after every 4th step the reference's prcp, pcpdrp, edir,
ett, ec, drip, cmc and sneqv.
"""
import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "pihm-cuda_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import pihm_gpu.land as L  # noqa: E402
from parity import land_deck, land_states  # noqa: E402

NSTEPS, EVERY, STATE_SEED = 48, 4, 7


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "pihm-cuda_gb300")], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.reference}"], check=True)
    from oracle import Reference
    from pihm_gpu import deck as D
    tmp = tempfile.mkdtemp()
    path = land_deck(tmp)
    d = D.Deck.read(path, "gen")
    ws, land, ctrl = d.watershed(), d.land(), d.control()
    ref = Reference()
    ref.load_deck(tmp, "gen")
    ne = ws.nelem
    out = {"start": np.int64(ctrl.start), "lsm_step": np.int64(ctrl.lsm_step), "cal": np.array(land.cal),
           "meteo_len": land.meteo_len, "meteo_time": land.meteo_time, "meteo_data": land.meteo_data,
           "lai_len": land.lai_len, "lai_time": land.lai_time, "lai_data": land.lai_data}
    for k in L.PARAM_I32 + L.PARAM_F64:
        want = ref.export(k, ne, np.int32 if k in L.PARAM_I32 else np.float64)
        assert np.array_equal(np.asarray(land.params[k]), want), k
        out["p_" + k] = want
    ws.save(os.path.join(HERE, "land_watershed.npz"))
    ref.land_set_state(None, None, np.zeros(ne), np.zeros(ne))
    t = ctrl.start
    for s, (unsat, gw) in enumerate(land_states(ws.arrays["depth"], STATE_SEED, NSTEPS)):
        ref.land_set_state(unsat, gw, None, None)
        ref.land_step(t, ctrl.lsm_step)
        if (s + 1) % EVERY == 0:
            for k, v in ref.land_fields().items():
                out[f"s{s + 1}_{k}"] = v
        t += ctrl.lsm_step
    np.savez_compressed(os.path.join(HERE, "land_calls.npz"), **out)
    print("wrote land_watershed.npz, land_calls.npz")


if __name__ == "__main__":
    main()
