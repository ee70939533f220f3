"""Golden vectors of the Noah land-surface model of Flux-PIHM from the
reference itself: its Noah(), Summary() and NoahHydrol() built with -D_NOAH_
(oracle/Makefile target `ref`, oracle/_ref/libpihm_ref_noah.so, the harness
filling the element records from the same parameter, state and forcing
structs the GPU library takes).

    python tests/golden/make_golden_noah_lsm.py [--reference /path/to/PIHM-CUDA]

writes tests/golden/noah_lsm.npz: a generated 400-element watershed with
generated Noah inputs (pihm_gpu.noah), its initial state y0, and 4
land-surface steps of 1,800 s with per-element forcing drawn to take
snowfall, melt, freezing rain and frozen soil in the same step
(pihm_gpu.noah.forcing(..., diverse=True)), each followed by 2 model steps of
900 s ending at perturbed states: the right-hand side at each state (the
Flux-PIHM ODE reading Noah's outputs), then Summary and NoahHydrol.  After
every Noah() and every NoahHydrol() every readable field is recorded.
"""
import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "pihm-cuda_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import pihm_gpu.watershed as W  # noqa: E402
from pihm_gpu import noah as N  # noqa: E402
from pihm_gpu import workloads as WL  # noqa: E402

NELEM, SEED, NOAH_SEED, FORCING_SEED = 400, 31, 5, 9
NLSM, NMODEL, DT_LSM, DT_MODEL = 4, 2, 1800.0, 900.0


def fields():
    return list(N.LAYER_FIELDS) + list(N.SCALAR_FIELDS)


def model_state(y0, s, m):
    return W.jitter(y0, 100 + 10 * s + m)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.reference}"], check=True)
    from oracle import Reference
    ws = W.generate(NELEM, WL.river_count(NELEM), seed=SEED)
    p, st = N.synthetic_noah(ws, seed=NOAH_SEED)
    y0 = W.reference_state(ws, NOAH_SEED)
    ref = Reference(noah=True)
    ref.build(ws)
    ref.noah_load(p, st, y0)
    out = {"y0": y0}
    for k, v in p.items():
        out["p_" + k] = v
    for k, v in st.items():
        out["s_" + k] = v
    for s in range(NLSM):
        f = N.forcing(ws, s, seed=FORCING_SEED, diverse=True)
        for k, v in f.items():
            out[f"f{s}_{k}"] = v
        ref.noah_forcing(f)
        ref.noah_step(DT_LSM)
        for k in fields():
            out[f"lsm{s}_{k}"] = ref.noah_get(k)
        for m in range(NMODEL):
            y = model_state(y0, s, m)
            ydot, rc = ref.rhs(y)
            assert rc == 0
            out[f"post{s}_{m}_y"] = y
            out[f"post{s}_{m}_ydot"] = ydot
            ref.noah_post(y, DT_MODEL)
            for k in fields():
                out[f"post{s}_{m}_{k}"] = ref.noah_get(k)
    ws.save(os.path.join(HERE, "noah_lsm_watershed.npz"))
    np.savez_compressed(os.path.join(HERE, "noah_lsm.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
