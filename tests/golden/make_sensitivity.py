"""Sensitivity envelope of the 2-day, 1,000-element golden solve
(c0_solve.npz) to one-ulp noise in the right-hand side.

Each run repeats the golden solve with the CPU restatement of the right-hand
side (oracle/) and the integrator over host vectors -- which together
reproduce the reference run bit for bit -- except that every right-hand-side
output entry is multiplied by (1 +- 2^-52), the sign drawn per entry and call
from a seeded generator.  The spread of these runs around the golden run is
how far any right-hand side that differs from the reference's in the last
bit (another libm, fused multiply-adds, another reduction order) can be
expected to land; the GPU end-to-end test is held to it.

    python tests/golden/make_sensitivity.py [--runs 24]

writes tests/golden/c0_sensitivity.npz: final states [runs, neq], outlet
flux series [runs, nsteps], step counts [runs], the largest cumulative
water-balance residual of PrintWaterBal (src/print.c:337-542) over the run
[runs], seeds.  The residual is heavy-tailed under this noise (six runs
spread from 13 to 96 m3 around the unperturbed 35 m3), so the default is
24 runs.
"""
import argparse
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "pihm-cuda_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import pihm_gpu.watershed as W  # noqa: E402
from backends import OracleBackend  # noqa: E402
from pihm_gpu.solver import RHS_FN, StepControl, run_steps  # noqa: E402


def noisy_run(ws, z, ctrl, seed):
    rng = np.random.default_rng(seed)
    b = OracleBackend(ws, z["y0"], z["pcp"], z["edir"], z["ett"])
    base = b.model.lib.oracle_cvrhs
    base.argtypes = [ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    base.restype = ctypes.c_int
    n = ws.neq

    def f(t, y, ydot, ud):
        rc = base(t, y, ydot, ud)
        # host N_Vector content: length, own_data, data
        content = ctypes.cast(ctypes.cast(ydot, ctypes.POINTER(ctypes.c_void_p))[0],
                              ctypes.POINTER(ctypes.c_void_p))
        a = np.ctypeslib.as_array(ctypes.cast(content[2], ctypes.POINTER(ctypes.c_double)), shape=(n,))
        a *= 1.0 + 2.0 ** -52 * rng.choice([-1.0, 1.0], n)
        return rc

    b._cb = RHS_FN(f)
    b.rhs = ctypes.cast(b._cb, ctypes.c_void_p)
    try:
        return run_steps(b, ctrl, z["outlet_q"].shape[0], b.set_forcing, record_every=int(z["every"]),
                         outlet=int(z["outlet"]), water_balance=True)
    finally:
        b.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=24)
    ap.add_argument("--out", default=os.path.join(HERE, "c0_sensitivity.npz"))
    args = ap.parse_args()
    z = np.load(os.path.join(HERE, "c0_solve.npz"))
    ws = W.Watershed.load(os.path.join(HERE, "c0_watershed.npz"))
    ctrl = StepControl(**{str(k): (int(v) if str(k) == "stepsize" else float(v))
                          for k, v in zip(z["ctrl_names"], z["ctrl"])})
    seeds = list(range(args.runs))
    finals, outs, nst, wbs = [], [], [], []
    for s in seeds:
        r = noisy_run(ws, z, ctrl, s)
        finals.append(r["states"][-1])
        outs.append(r["outlet"])
        nst.append(r["stats"].nst)
        wb = r["wb"]
        resid = np.cumsum(wb[1:, 0] - wb[1:, 1] - (wb[1:, 2] - wb[:-1, 2]))
        wbs.append(np.abs(resid).max())
        print("seed", s, "nst", r["stats"].nst, "water-balance residual", wbs[-1])
    np.savez_compressed(args.out, final=np.array(finals), outlet=np.array(outs), nst=np.array(nst),
                        wb_resid=np.array(wbs), seeds=np.array(seeds))


if __name__ == "__main__":
    main()
