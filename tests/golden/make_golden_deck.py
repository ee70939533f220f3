"""Golden run of the reference's own main loop on an input deck with its own
forcing: the generated 1,000-element deck of tests/parity.py land_deck
(hourly forcing with snow, rain and melt, LSM_STEP 900 s) read by the
reference's ReadAlloc/Initialize, then one simulated day of 60 s model steps
with ApplyBc, ApplyForc + IntcpSnowEt every 900 s, SolveCVode, Summary and
AdjCVodeMaxStep (src/main.c:217-254, src/pihm.c:7-187; oracle/ref_harness.c
ref_run_deck), and a one-ulp sensitivity ensemble of that run.

    python tests/golden/make_golden_deck.py [--steps 1440] [--runs 16]

writes tests/golden/deck_solve.npz: the outlet segment, the state every 360
steps, the outlet flux (rivflow DOWN_CHANL2CHANL) after every step,
PrintWaterBal's three sums (src/print.c:337-542) at full precision after every
step, CVODE's counters; and, from `runs` repetitions with the CPU
restatements (right-hand side, land-surface step, integrator -- which
together reproduce the reference run bit for bit) with every right-hand-side
output multiplied by (1 +- 2^-52): their final states, outlet series, step
counts and largest cumulative water-balance residuals.  The reference keeps
solver state in statics (src/ode.c:416,609-611), so its run is made in a
child process.
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

from parity import land_deck  # noqa: E402

EVERY = 360
_P = ctypes.POINTER(ctypes.c_double)


def reference_run(steps: int, out: str):
    from oracle import Reference
    from pihm_gpu import deck as D
    tmp = tempfile.mkdtemp()
    path = land_deck(tmp)
    ws = D.Deck.read(path, "gen").watershed()
    outlet = int(np.flatnonzero(np.asarray(ws.arrays["down"]) < 0)[0])
    ref = Reference()
    y = ref.load_deck(tmp, "gen")
    lib = ref.lib
    lib.ref_run_deck.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P,
                                 ctypes.POINTER(ctypes.c_long)]
    q, wb = np.zeros(steps), np.zeros((steps, 3))
    ys = np.zeros((steps // EVERY, ws.neq))
    st = np.zeros(7, np.int64)
    assert lib.ref_run_deck(y.ctypes.data_as(_P), steps, outlet, EVERY, ys.ctypes.data_as(_P), q.ctypes.data_as(_P),
                            wb.ctypes.data_as(_P), st.ctypes.data_as(ctypes.POINTER(ctypes.c_long))) == 0
    np.savez(out, outlet=np.int64(outlet), every=np.int64(EVERY), states=ys, outlet_q=q, wb=wb, stats=st)


def noisy_run(d, steps, outlet, seed):
    from backends import OracleDeckBackend
    from pihm_gpu.single import step_control
    from pihm_gpu.solver import RHS_FN, run_steps
    rng = np.random.default_rng(seed)
    b = OracleDeckBackend(d)
    base = b.model.lib.oracle_cvrhs
    base.argtypes = [ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    base.restype = ctypes.c_int
    n = b.ws.neq

    def f(t, y, ydot, ud):
        rc = base(t, y, ydot, ud)
        content = ctypes.cast(ctypes.cast(ydot, ctypes.POINTER(ctypes.c_void_p))[0], ctypes.POINTER(ctypes.c_void_p))
        a = np.ctypeslib.as_array(ctypes.cast(content[2], _P), shape=(n,))
        a *= 1.0 + 2.0 ** -52 * rng.choice([-1.0, 1.0], n)
        return rc

    b._cb = RHS_FN(f)
    b.rhs = ctypes.cast(b._cb, ctypes.c_void_p)
    try:
        return run_steps(b, step_control(d.control()), steps, b.set_forcing, record_every=steps, outlet=outlet,
                         water_balance=True)
    finally:
        b.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1440)
    ap.add_argument("--runs", type=int, default=16)
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--child", default=None)
    args = ap.parse_args()
    if args.child:
        reference_run(args.steps, args.child)
        return
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "pihm-cuda_gb300")], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.reference}"], check=True)
    tmp = tempfile.mkdtemp()
    child = os.path.join(tmp, "ref.npz")
    subprocess.run([sys.executable, os.path.abspath(__file__), "--steps", str(args.steps), "--child", child],
                   check=True)
    z = dict(np.load(child))
    from pihm_gpu import deck as D
    d = D.Deck.read(land_deck(tempfile.mkdtemp()), "gen")
    finals, outs, nst, wbs = [], [], [], []
    for s in range(args.runs):
        r = noisy_run(d, args.steps, int(z["outlet"]), s)
        finals.append(r["states"][-1])
        outs.append(r["outlet"])
        nst.append(r["stats"].nst)
        wb = r["wb"]
        resid = np.cumsum(wb[1:, 0] - wb[1:, 1] - (wb[1:, 2] - wb[:-1, 2]))
        wbs.append(np.abs(resid).max())
        print("seed", s, "nst", r["stats"].nst, "water-balance residual", wbs[-1])
    np.savez_compressed(os.path.join(HERE, "deck_solve.npz"), **z, sens_final=np.array(finals),
                        sens_outlet=np.array(outs), sens_nst=np.array(nst), sens_wb_resid=np.array(wbs),
                        sens_seeds=np.arange(args.runs))
    print("reference: nst", z["stats"][0], "nfe", z["stats"][1])


if __name__ == "__main__":
    main()
