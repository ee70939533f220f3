"""The Noah golden vectors (tests/golden/noah_lsm.npz) are the reference's
own results: rerun here through the reference built with -D_NOAH_, the same
sequence gives every recorded array bit for bit."""
import os

import numpy as np
import pytest

import pihm_gpu.watershed as W
from pihm_gpu import noah as N

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_noah_goldens_are_the_references_own():
    import oracle
    if not os.path.exists(os.path.join(os.path.dirname(oracle.__file__), "_ref", "libpihm_ref_noah.so")):
        pytest.skip("the reference build is not here")
    z = np.load(os.path.join(GOLD, "noah_lsm.npz"))
    ws = W.Watershed.load(os.path.join(GOLD, "noah_lsm_watershed.npz"))
    p = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    st = {k[2:]: z[k] for k in z.files if k.startswith("s_")}
    ref = oracle.Reference(noah=True)
    ref.build(ws)
    ref.noah_load(p, st, z["y0"])
    names = list(N.LAYER_FIELDS) + list(N.SCALAR_FIELDS)
    for s in range(4):
        ref.noah_forcing({k: z[f"f{s}_{k}"] for k in N.FORCING_FIELDS})
        ref.noah_step(1800.0)
        for k in names:
            assert np.array_equal(ref.noah_get(k), z[f"lsm{s}_{k}"]), (s, k)
        for m in range(2):
            y = z[f"post{s}_{m}_y"]
            ydot, rc = ref.rhs(y)
            assert rc == 0 and np.array_equal(ydot, z[f"post{s}_{m}_ydot"])
            ref.noah_post(y, 900.0)
            for k in names:
                assert np.array_equal(ref.noah_get(k), z[f"post{s}_{m}_{k}"]), (s, m, k)


def test_generated_inputs_take_the_models_branches():
    """The fixture's forcing takes snowfall, melt, frozen soil and every
    water-table position."""
    z = np.load(os.path.join(GOLD, "noah_lsm.npz"))
    assert (z["lsm3_sneqv"] > 0).sum() > 50 and (z["lsm0_snomlt"] > 0).sum() > 0
    assert (z["post3_1_fcr"] < 1.0).sum() > 50
    assert len(np.unique(z["post3_1_nwtbl"])) >= 4
