"""Golden vectors of the Flux-PIHM (_NOAH_) right-hand side from the
reference itself: its ODE() built with -D_NOAH_ (oracle/Makefile target
`ref`, library oracle/_ref/libpihm_ref_noah.so), whose EtExtract splits
transpiration with Noah's per-layer transpiration (GwTransp), whose Infil
takes its saturation from Noah's top-layer moisture and scales infiltration
by the frozen-soil factor (src/hydrol.c:43-55,79-83, src/vert_flow.c:16-19,
94-98).

    python tests/golden/make_golden_noah.py [--reference /path/to/PIHM-CUDA]

writes tests/golden/c0_noah_calls.npz: for three scenarios on the
1,000-element watershed (tests/parity.py scenario(..., noah=True)), the Noah
inputs, forcing and carried values, three consecutive calls' y and ydot, the
fluxes of the first call, and GwTransp's fraction gwet per element.
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
from parity import apply, scenario  # noqa: E402

FLUX_KEYS = ("ovlflow", "subsurf", "infil", "rechg", "et_split", "rivflow")
NOAH_KEYS = ("et", "nwtbl", "nroot", "sh2o0", "smcmin", "smcmax", "fcr")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.reference}"], check=True)
    from oracle import Reference
    ws = W.Watershed.load(os.path.join(HERE, "c0_watershed.npz"))
    out = {"digest": np.frombuffer(ws.digest().encode(), np.uint8)}
    for seed in range(3):
        tag = f"n{seed}"
        w2, sc = scenario(ws, seed, noah=True)
        ref = Reference(noah=True)
        ref.build(w2)
        apply(ref, sc)
        for k in ("y", "pcpdrp", "edir", "ett", "ws0", "ovl"):
            out[f"{tag}_{k}"] = sc[k]
        for k in NOAH_KEYS:
            out[f"{tag}_noah_{k}"] = sc["noah"][k]
        for c in range(3):
            y = sc["y"] if c == 0 else W.jitter(sc["y"], 77 + c)
            ydot, rc = ref.rhs(y)
            assert rc == 0
            out[f"{tag}_call{c}_y"] = y
            out[f"{tag}_call{c}_ydot"] = ydot
            if c == 0:
                fx = ref.fluxes()
                for k in FLUX_KEYS:
                    out[f"{tag}_call{c}_{k}"] = fx[k]
                gwet = np.zeros(ws.nelem)
                ref.lib.ref_get_gwet(gwet.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_double)))
                out[f"{tag}_call{c}_gwet"] = gwet
    np.savez_compressed(os.path.join(HERE, "c0_noah_calls.npz"), **out)
    print("wrote c0_noah_calls.npz")


if __name__ == "__main__":
    main()
