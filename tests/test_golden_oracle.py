"""The CPU restatement (oracle/pihm_oracle.c) against golden vectors that the
reference's own ODE() produced (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

import pihm_gpu.watershed as W
from parity import compare, row_scales

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load_ws(name):
    return W.Watershed.load(os.path.join(GOLD, name))


def _scenario_tags(z):
    return sorted({k.split("_")[0] for k in z.files if k.endswith("_modes")})


def _run(model_cls, ws, z, tag):
    import copy
    w2 = copy.deepcopy(ws)
    if f"{tag}_bc_type" in z.files:
        w2.arrays["bc_type"] = z[f"{tag}_bc_type"]
        w2.arrays["riverbc_type"] = z[f"{tag}_riverbc_type"]
    w2.surf_mode, w2.riv_mode = (int(v) for v in z[f"{tag}_modes"])
    m = model_cls(w2)
    m.set_forcing(z[f"{tag}_pcpdrp"], z[f"{tag}_edir"], z[f"{tag}_ett"])
    m.set_ws0_surf(z[f"{tag}_ws0"])
    m.set_river_edge_ovlflow(z[f"{tag}_ovl"])
    if f"{tag}_elem_bc" in z.files:
        m.set_bc(z[f"{tag}_elem_bc"], z[f"{tag}_river_bc"])
    return w2, m


def test_generator_reproduces_c0():
    ws = W.generate(1000, 100, seed=0)
    ref = _load_ws("c0_watershed.npz")
    assert ws.digest() == ref.digest()
    z = np.load(os.path.join(GOLD, "c0_calls.npz"))
    assert bytes(z["digest"]).decode() == ws.digest()


def test_oracle_matches_reference_goldens():
    from oracle import Oracle
    ws = _load_ws("c0_watershed.npz")
    z = np.load(os.path.join(GOLD, "c0_calls.npz"))
    tags = _scenario_tags(z)
    assert {"s0", "s1", "bc", "k11", "k12", "k21"} <= set(tags)
    for tag in tags:
        w2, o = _run(Oracle, ws, z, tag)
        c = 0
        while f"{tag}_call{c}_y" in z.files:
            got, rc = o.rhs(z[f"{tag}_call{c}_y"])
            want = z[f"{tag}_call{c}_ydot"]
            assert rc == 0
            fx = o.fluxes()
            scale = row_scales(w2, fx, z[f"{tag}_pcpdrp"], z[f"{tag}_edir"], z[f"{tag}_ett"])
            ok, worst, idx = compare(got, want, scale)
            assert ok, (tag, c, worst, idx)
            if f"{tag}_call{c}_rivflow" in z.files:
                for k in ("ovlflow", "subsurf", "infil", "rechg", "et_split", "rivflow"):
                    ref = z[f"{tag}_call{c}_{k}"]
                    den = np.maximum(np.abs(ref), 1e-30)
                    assert np.max(np.abs(fx[k] - ref) / den) <= 1e-12, (tag, k)
            c += 1


def test_oracle_matches_reference_example_deck():
    """The bundled 535-element example, read and initialised by the
    reference's own readers."""
    from oracle import Oracle
    ws = _load_ws("example_watershed.npz")
    assert ws.nelem == 535 and ws.nriver == 20
    z = np.load(os.path.join(GOLD, "example_calls.npz"))
    o = Oracle(ws)
    o.set_forcing(z["pcpdrp"], z["edir"], z["ett"])
    o.set_ws0_surf(z["ws0"])
    for c in range(2):
        got, rc = o.rhs(z[f"call{c}_y"])
        assert rc == 0
        fx = o.fluxes()
        scale = row_scales(ws, fx, z["pcpdrp"], z["edir"], z["ett"])
        ok, worst, idx = compare(got, z[f"call{c}_ydot"], scale)
        assert ok, (c, worst, idx)


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference not built here")
def test_oracle_bit_exact_with_reference_build():
    """Where the reference compiles (same compiler and libm), the restatement
    agrees with it bit for bit, fluxes included."""
    from oracle import Oracle, Reference
    from parity import apply, scenario
    for seed, bc in ((0, False), (4, True), (9, False)):
        ws, sc = scenario(W.generate(1000, 100, seed=seed), seed, bc=bc)
        o = Oracle(ws)
        r = Reference()
        r.build(ws)
        apply(o, sc)
        apply(r, sc)
        for k in range(3):
            y = W.jitter(sc["y"], 900 + k)
            a, _ = o.rhs(y)
            b, _ = r.rhs(y)
            assert np.array_equal(a, b), (seed, k)
            fa, fb = o.fluxes(), r.fluxes()
            for key in fa:
                assert np.array_equal(fa[key], fb[key]), (seed, k, key)


def _noah_inputs(z, tag):
    return {k: z[f"{tag}_noah_{k}"] for k in ("et", "nwtbl", "nroot", "sh2o0", "smcmin", "smcmax", "fcr")}


def test_oracle_matches_reference_noah_goldens():
    """Flux-PIHM (_NOAH_) variant: bit for bit with the reference built with
    -D_NOAH_ (tests/golden/make_golden_noah.py)."""
    from oracle import Oracle
    ws = _load_ws("c0_watershed.npz")
    z = np.load(os.path.join(GOLD, "c0_noah_calls.npz"))
    assert bytes(z["digest"]).decode() == ws.digest()
    for seed in range(3):
        tag = f"n{seed}"
        o = Oracle(ws)
        o.set_noah(_noah_inputs(z, tag))
        o.set_forcing(z[f"{tag}_pcpdrp"], z[f"{tag}_edir"], z[f"{tag}_ett"])
        o.set_ws0_surf(z[f"{tag}_ws0"])
        o.set_river_edge_ovlflow(z[f"{tag}_ovl"])
        for c in range(3):
            got, rc = o.rhs(z[f"{tag}_call{c}_y"])
            assert rc == 0
            assert np.array_equal(got, z[f"{tag}_call{c}_ydot"]), (tag, c)
            if c == 0:
                fx = o.fluxes()
                for k in ("ovlflow", "subsurf", "infil", "rechg", "et_split", "rivflow"):
                    assert np.array_equal(fx[k], z[f"{tag}_call0_{k}"]), (tag, k)
        # the variant is live: the plain right-hand side differs on these inputs
        o2 = Oracle(ws)
        o2.set_forcing(z[f"{tag}_pcpdrp"], z[f"{tag}_edir"], z[f"{tag}_ett"])
        o2.set_ws0_surf(z[f"{tag}_ws0"])
        o2.set_river_edge_ovlflow(z[f"{tag}_ovl"])
        plain, _ = o2.rhs(z[f"{tag}_call0_y"])
        assert not np.array_equal(plain, z[f"{tag}_call0_ydot"])
