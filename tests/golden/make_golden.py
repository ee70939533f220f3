"""Generate the golden vectors of the right-hand side from the reference itself.

Run in a container that has the reference sources (it builds
oracle/_ref/libpihm_ref.so from them through oracle/Makefile):

    python tests/golden/make_golden.py [--reference /path/to/PIHM-CUDA]

It writes, next to this script:

  c0_watershed.npz       the 1,000-element / 100-segment synthetic watershed
                         (seed 0), in the reference's field layout
  c0_calls.npz           two scenarios x three consecutive ODE() calls each
                         (the river-edge overland flux carries from call to
                         call), a boundary-condition scenario (two calls) and
                         the three kinematic-wave mode pairs: inputs, ydot,
                         and the fluxes of the first call of s0 and bc
  example_watershed.npz  the bundled benchmark/input/example deck (535
                         elements, 20 segments) as read and initialised by the
                         reference's own ReadAlloc/Initialize
  example_calls.npz      ODE() on its initial state with the forcing of its
                         first step (ApplyBc/ApplyForc/IntcpSnowEt), and on a
                         wet perturbed state

Every expected ydot comes from the reference's ODE() (src/ode.c:4) compiled
from its sources; nothing here comes from the restatement or the GPU library.
"""
import argparse
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "pihm-cuda_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import pihm_gpu.watershed as W  # noqa: E402
from parity import scenario  # noqa: E402

FLUX_KEYS = ("ovlflow", "subsurf", "infil", "rechg", "et_split", "rivflow")


def run_calls(ref, ws, sc, ncalls, tag, out, fluxes=False):
    ref.build(ws)
    ref.set_forcing(sc["pcpdrp"], sc["edir"], sc["ett"])
    ref.set_ws0_surf(sc["ws0"])
    ref.set_river_edge_ovlflow(sc["ovl"])
    if sc["elem_bc"] is not None or sc["river_bc"] is not None:
        ref.set_bc(sc["elem_bc"], sc["river_bc"])
    for k in ("y", "pcpdrp", "edir", "ett", "ws0", "ovl"):
        out[f"{tag}_{k}"] = sc[k]
    if sc["elem_bc"] is not None:
        out[f"{tag}_elem_bc"] = sc["elem_bc"]
        out[f"{tag}_river_bc"] = sc["river_bc"]
        out[f"{tag}_bc_type"] = ws.arrays["bc_type"]
        out[f"{tag}_riverbc_type"] = ws.arrays["riverbc_type"]
    out[f"{tag}_modes"] = np.array([ws.surf_mode, ws.riv_mode])
    for c in range(ncalls):
        y = sc["y"] if c == 0 else W.jitter(sc["y"], 500 + c)
        ydot, rc = ref.rhs(y)
        assert rc == 0
        out[f"{tag}_call{c}_y"] = y
        out[f"{tag}_call{c}_ydot"] = ydot
        if fluxes and c == 0:
            fx = ref.fluxes()
            for k in FLUX_KEYS:
                out[f"{tag}_call{c}_{k}"] = fx[k]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    import subprocess
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref",
                    f"REF={args.reference}"], check=True)
    from oracle import Reference
    ref = Reference()

    # ---- synthetic c0 ----
    ws = W.generate(1000, 100, seed=0)
    ws.save(os.path.join(HERE, "c0_watershed.npz"))
    out = {"digest": np.frombuffer(ws.digest().encode(), np.uint8)}
    for seed in (0, 1):
        w2, sc = scenario(ws, seed)
        run_calls(ref, w2, sc, 3, f"s{seed}", out, fluxes=(seed == 0))
    w2, sc = scenario(ws, 5, bc=True)
    run_calls(ref, w2, sc, 2, "bc", out, fluxes=True)
    for sm, rm in ((1, 1), (1, 2), (2, 1)):
        w2, sc = scenario(ws, 7)
        w2.surf_mode, w2.riv_mode = sm, rm
        run_calls(ref, w2, sc, 1, f"k{sm}{rm}", out)
    np.savez_compressed(os.path.join(HERE, "c0_calls.npz"), **out)

    # ---- bundled example deck, read by the reference itself ----
    with tempfile.TemporaryDirectory() as tmp:
        os.symlink(os.path.join(args.reference, "benchmark", "input"),
                   os.path.join(tmp, "input"))
        y0 = ref.load_deck(tmp, "example")
    ne, nr = ref.ne, ref.nr
    arrays = {}
    for k in W.MESH_FIELDS:
        n = (3 * ne if k in W.PER_EDGE else (ne if not k.startswith("riv")
             and k not in W.RIVER_INT_FIELDS else nr))
        kind = np.int32 if (k in W.ELEM_INT_FIELDS or k in W.RIVER_INT_FIELDS) else np.float64
        arrays[k] = ref.export(k, n, kind)
    ex = W.Watershed(ne, nr, arrays, ref.surf_mode, ref.riv_mode, float(ref.stepsize))
    ex.save(os.path.join(HERE, "example_watershed.npz"))
    import ctypes
    st, en, et, ns = (ctypes.c_int() for _ in range(4))
    ref.lib.ref_model_times(ctypes.byref(st), ctypes.byref(en), ctypes.byref(et), ctypes.byref(ns))
    assert ref.lib.ref_apply_forcing(st.value) == 0
    pcpdrp = ref.export("pcpdrp", ne)
    edir = ref.export("edir", ne)
    ett = ref.export("ett", ne)
    ws0 = ref.export("ws0_surf", ne)
    eout = {"y0": y0, "pcpdrp": pcpdrp, "edir": edir, "ett": ett, "ws0": ws0,
            "times": np.array([st.value, en.value, et.value, ns.value])}
    states = [y0, W.jitter(W.reference_state(ex, 11), 12)]
    for c, y in enumerate(states):
        ydot, rc = ref.rhs(y)
        assert rc == 0
        eout[f"call{c}_y"] = y
        eout[f"call{c}_ydot"] = ydot
        fx = ref.fluxes()
        for k in FLUX_KEYS:
            eout[f"call{c}_{k}"] = fx[k]
    np.savez_compressed(os.path.join(HERE, "example_calls.npz"), **eout)
    print("wrote golden vectors to", HERE)


if __name__ == "__main__":
    main()
