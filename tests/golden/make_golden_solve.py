"""Golden end-to-end run of the reference: its own CVODE 2.9 and ODE() on the
1,000-element synthetic watershed, 2 simulated days of 60 s model steps with
the reference's per-step loop (SolveCVode / Summary / AdjCVodeMaxStep,
src/main.c:217-254), driven through oracle/ref_harness.c::ref_run_pihm.

    python tests/golden/make_golden_solve.py [--days 2]

writes tests/golden/c0_solve.npz: the initial state, the per-step forcing,
the state every 6 hours, the outlet flux (rivflow DOWN_CHANL2CHANL of the
outlet segment as left by the last right-hand-side call, what PIHM prints as
rivflx1) after every step, CVODE's counters, and the water balance after
every step: the sums of PrintWaterBal (src/print.c:337-542: sources, sinks,
storage) at full precision in `wb` and the reference's own printed lines in
`wb_printed`.  Runs in its own process:
the reference keeps solver state in statics (src/ode.c:416,609-611).
"""
import argparse
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "pihm-cuda_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pihm_gpu.watershed as W  # noqa: E402

CTRL = dict(stepsize=60, reltol=1e-4, abstol=1e-5, initstep=5e-5, nncfn=0.0, nnimax=3.0,
            nnimin=1.0, decr=1.2, incr=1.2, stmin=1.0)
EVERY = 360


def step_forcing(ws, nsteps, stepsize=60):
    hours = (nsteps * stepsize + 3599) // 3600
    p, e, t = W.hourly_forcing(ws, hours, seed=2)
    k = (np.arange(nsteps) * stepsize) // 3600
    return p[k].copy(), e[k].copy(), t[k].copy()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--days", type=float, default=2.0)
    ap.add_argument("--out", default=os.path.join(HERE, "c0_solve.npz"))
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref",
                    f"REF={args.reference}"], check=True)
    from oracle import Reference
    ws = W.Watershed.load(os.path.join(HERE, "c0_watershed.npz"))
    nsteps = int(round(args.days * 86400 / CTRL["stepsize"]))
    pcp, edir, ett = step_forcing(ws, nsteps, CTRL["stepsize"])
    y0 = W.relax_state(ws)
    outlet = int(np.where(ws.arrays["down"] < 0)[0][0])
    ref = Reference()
    ref.build(ws)
    f = ref.lib.ref_run_pihm
    D = ctypes.c_double
    P = ctypes.POINTER(D)
    f.argtypes = [P, ctypes.c_int, ctypes.c_int] + [D] * 9 + [P, P, P, ctypes.c_int, ctypes.c_int,
                                                             P, P, ctypes.POINTER(ctypes.c_long)]
    # the watershed water balance per step: the reference's own PrintWaterBal
    # (6 printed digits) and its sums at full precision
    wb = np.zeros((nsteps, 3))
    wb_path = os.path.join(HERE, "_wb_tmp.txt")
    ref.lib.ref_set_water_balance.argtypes = [ctypes.c_char_p, P]
    ref.lib.ref_set_water_balance(wb_path.encode(), wb.ctypes.data_as(P))
    y = y0.copy()
    nrec = nsteps // EVERY
    ys = np.zeros((nrec, ws.neq))
    q = np.zeros(nsteps)
    stats = (ctypes.c_long * 7)()
    c = CTRL
    rc = f(y.ctypes.data_as(P), nsteps, c["stepsize"], c["reltol"], c["abstol"], c["initstep"],
           c["nncfn"], c["nnimax"], c["nnimin"], c["decr"], c["incr"], c["stmin"],
           pcp.ctypes.data_as(P), edir.ctypes.data_as(P), ett.ctypes.data_as(P), outlet, EVERY,
           ys.ctypes.data_as(P), q.ctypes.data_as(P), stats)
    assert rc == 0
    ref.lib.ref_close_water_balance()
    printed = np.loadtxt(wb_path, skiprows=1)  # t, src, snk, dstrg, src - snk - dstrg, cumulative
    os.remove(wb_path)
    np.savez_compressed(args.out, y0=y0, pcp=pcp, edir=edir, ett=ett, wb=wb, wb_printed=printed,
                        states=ys, outlet_q=q, outlet=outlet, every=EVERY,
                        stats=np.array(list(stats)), ctrl=np.array([c[k] for k in CTRL]),
                        ctrl_names=np.array(list(CTRL)))
    print("steps", nsteps, "stats nst nfe nni ncfn netf nli nfes:", list(stats))


if __name__ == "__main__":
    main()
