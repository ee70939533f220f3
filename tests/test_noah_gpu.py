"""The Noah land-surface model of Flux-PIHM on the GPU (include/pihm_noah.h)
against the reference's own Noah(), Summary() and NoahHydrol()
(tests/golden/noah_lsm.npz, tests/golden/make_golden_noah_lsm.py): the same
400-element watershed, parameters, initial state and forcing, 4
land-surface steps each followed by 2 model steps -- the Flux-PIHM right-hand
side on the device reading Noah's outputs, then the post-step -- with every
readable field compared after each Noah step and each NoahHydrol.

Tolerance: each field within 1e-10 relative to max(|reference|, 1e-3 of
the field's largest magnitude).  The arithmetic follows the reference's
operations without contraction, so the differences are those of the
elementary functions (CUDA's exp, log, log10 and atan against glibc's, the
power within 0.502 ulp) carried through the coupled steps; measured on GB300:
96 % of the values identical to the last bit, the worst field 3.4e-12."""
import os

import numpy as np
import pytest

import pihm_gpu.watershed as W
from pihm_gpu import noah as N

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-10


def _err(got, want):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    scale = np.max(np.abs(want)) if want.size else 0.0
    den = np.maximum(np.abs(want), 1e-3 * scale)
    den = np.where(den > 0, den, 1.0)
    e = np.abs(got - want) / den
    return np.where(got == want, 0.0, e)


def test_noah_against_reference_goldens():
    import torch
    from pihm_gpu.capi import GpuRhs
    z = np.load(os.path.join(GOLD, "noah_lsm.npz"))
    ws = W.Watershed.load(os.path.join(GOLD, "noah_lsm_watershed.npz"))
    ne = ws.nelem
    p = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    st = {k[2:]: z[k] for k in z.files if k.startswith("s_")}
    g = GpuRhs(ws)
    g.set_stream(torch.cuda.current_stream().cuda_stream)
    g.noah_init(p, st)
    y0 = z["y0"]
    g.set_ws0_surf(y0[:ne])

    def to_dev(y):
        yr = torch.from_numpy(np.ascontiguousarray(y)).cuda()
        yi = torch.empty_like(yr)
        g.to_internal(yr.data_ptr(), yi.data_ptr())
        return yi

    y0i = to_dev(y0)
    g.noah_begin(y0i.data_ptr())
    worst, same, total = {}, 0, 0

    def check(prefix):
        nonlocal same, total
        for k in list(N.LAYER_FIELDS) + list(N.SCALAR_FIELDS):
            want = z[f"{prefix}_{k}"]
            got = g.noah_get(k)
            e = _err(got, want)
            worst[k] = max(worst.get(k, 0.0), float(e.max()))
            same += int(np.sum(got == want))
            total += got.size

    for s in range(4):
        g.noah_set_forcing({k: z[f"f{s}_{k}"] for k in N.FORCING_FIELDS})
        g.noah_step(1800.0)
        check(f"lsm{s}")
        for m in range(2):
            y = z[f"post{s}_{m}_y"]
            yi = to_dev(y)
            ydi, ydr = torch.empty_like(yi), torch.empty_like(yi)
            g.rhs_device(yi.data_ptr(), ydi.data_ptr())
            g.to_reference(ydi.data_ptr(), ydr.data_ptr())
            torch.cuda.current_stream().synchronize()
            assert g.status() == 0
            want = z[f"post{s}_{m}_ydot"]
            ydot_err = 0.0
            for b in range(3):  # the element blocks of ydot
                ydot_err = max(ydot_err, float(_err(ydr.cpu().numpy()[b * ne:(b + 1) * ne],
                                                    want[b * ne:(b + 1) * ne]).max()))
            worst["ydot"] = max(worst.get("ydot", 0.0), ydot_err)
            g.noah_post_step(yi.data_ptr(), 900.0)
            g.post_step(yi.data_ptr())
            check(f"post{s}_{m}")
    g.close()
    bad = {k: v for k, v in worst.items() if v > TOL}
    print("\nNoah against the reference: %d of %d values identical to the last bit; worst per field: %s"
          % (same, total, ", ".join(f"{k} {v:.1e}" for k, v in sorted(worst.items(), key=lambda x: -x[1])[:12])))
    assert not bad, bad
