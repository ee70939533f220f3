"""Golden run of the reference's bundled example deck (benchmark/input/example:
535 elements, 20 segments, its own meteorological and LAI records) through
the reference's own main loop with its own forcing for one simulated day
(ApplyBc, ApplyForc + IntcpSnowEt every LSM_STEP, SolveCVode, Summary,
AdjCVodeMaxStep; oracle/ref_harness.c ref_run_deck), and a one-ulp
sensitivity ensemble of that run from the CPU restatements.

    python tests/golden/make_golden_example_run.py [--steps 1440] [--runs 16]

writes tests/golden/example_run.npz: the deck as the library's reader gives
it (bit for bit the reference's: tests/test_deck.py, tests/test_land.py) --
the land-surface parameters, the forcing records the day needs (the knots
around it; interpolation inside the day reads no others), the solver
controls and start time -- and the reference run's outlet flux after every
step, its state every 360 steps, PrintWaterBal's sums and CVODE's counters,
with the ensemble's final states, outlet series, step counts and
water-balance residuals.  The mesh itself is example_watershed.npz.
"""
import argparse
import ctypes
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "pihm-cuda_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

EVERY = 360
_P = ctypes.POINTER(ctypes.c_double)


def _deck(reference):
    from pihm_gpu import deck as D
    ex = os.path.join(reference, "benchmark", "input")
    return D.Deck.read(os.path.join(ex, "example"), "example", lc_table=os.path.join(ex, "vegprmt.tbl"))


def reference_run(reference, steps, out):
    from oracle import Reference
    d = _deck(reference)
    ws = d.watershed()
    outlet = int(np.flatnonzero(np.asarray(ws.arrays["down"]) < 0)[0])
    ref = Reference()
    y = ref.load_deck(os.path.join(reference, "benchmark"), "example")
    lib = ref.lib
    lib.ref_run_deck.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P,
                                 ctypes.POINTER(ctypes.c_long)]
    q, wb = np.zeros(steps), np.zeros((steps, 3))
    ys = np.zeros((steps // EVERY, ws.neq))
    st = np.zeros(7, np.int64)
    assert lib.ref_run_deck(y.ctypes.data_as(_P), steps, outlet, EVERY, ys.ctypes.data_as(_P), q.ctypes.data_as(_P),
                            wb.ctypes.data_as(_P), st.ctypes.data_as(ctypes.POINTER(ctypes.c_long))) == 0
    np.savez(out, outlet=np.int64(outlet), every=np.int64(EVERY), states=ys, outlet_q=q, wb=wb, stats=st)


def window(lens, times, data, t0, t1):
    """The knots of each series that interpolation over [t0, t1] reads."""
    nl, tt, dd = [], [], []
    o = 0
    for n in lens:
        t = times[o:o + n]
        a = max(int(np.searchsorted(t, t0, side="right")) - 1, 0)
        b = min(int(np.searchsorted(t, t1, side="left")) + 1, n)
        nl.append(b - a)
        tt.append(t[a:b])
        dd.append(data[o + a:o + b])
        o += n
    return np.array(nl, np.int32), np.concatenate(tt), np.concatenate(dd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1440)
    ap.add_argument("--runs", type=int, default=16)
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--child", default=None)
    args = ap.parse_args()
    if args.child:
        reference_run(args.reference, args.steps, args.child)
        return
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "pihm-cuda_gb300")], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.reference}"], check=True)
    child = os.path.join(tempfile.mkdtemp(), "ref.npz")
    subprocess.run([sys.executable, os.path.abspath(__file__), "--steps", str(args.steps), "--child", child,
                    "--reference", args.reference], check=True)
    z = dict(np.load(child))
    d = _deck(args.reference)
    c, land = d.control(), d.land()
    t0, t1 = int(c.start), int(c.start) + args.steps * int(c.step["stepsize"])
    ml, mt, md = window(land.meteo_len, land.meteo_time, land.meteo_data, t0, t1)
    ll, lt, ld = window(land.lai_len, land.lai_time, land.lai_data, t0, t1)
    fix = {"start": np.int64(c.start), "lsm_step": np.int64(c.lsm_step), "surf_mode": np.int64(c.surf_mode),
           "riv_mode": np.int64(c.riv_mode), "ctrl_names": np.array(list(c.step.keys())),
           "ctrl": np.array([float(v) for v in c.step.values()]), "y0": d.initial_state(),
           "cal": np.array(land.cal), "meteo_len": ml, "meteo_time": mt, "meteo_data": md,
           "lai_len": ll, "lai_time": lt, "lai_data": ld}
    for k, v in land.params.items():
        fix["p_" + k] = v
    # the ensemble, from the restatements over the same arrays
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_deck_run import ArrayDeck
    from make_golden_deck import noisy_run
    ad = ArrayDeck.from_fixture(fix)
    finals, outs, nst, wbs = [], [], [], []
    for s in range(args.runs):
        r = noisy_run(ad, args.steps, int(z["outlet"]), s)
        finals.append(r["states"][-1])
        outs.append(r["outlet"])
        nst.append(r["stats"].nst)
        wb = r["wb"]
        resid = np.cumsum(wb[1:, 0] - wb[1:, 1] - (wb[1:, 2] - wb[:-1, 2]))
        wbs.append(np.abs(resid).max())
        print("seed", s, "nst", r["stats"].nst, "water-balance residual", wbs[-1])
    np.savez_compressed(os.path.join(HERE, "example_run.npz"), **fix, **z, sens_final=np.array(finals),
                        sens_outlet=np.array(outs), sens_nst=np.array(nst), sens_wb_resid=np.array(wbs))
    print("reference: nst", z["stats"][0], "nfe", z["stats"][1])


if __name__ == "__main__":
    main()
