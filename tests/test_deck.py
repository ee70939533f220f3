"""Input decks (include/pihm_deck.h, pihm_gpu/deck.py): the reference's text
input files read and initialised by the library, against the generator that
wrote them, against the reference's own ReadAlloc + Initialize on the same
files, and against the bundled example deck as the reference reads it."""
import os

import numpy as np
import pytest

import pihm_gpu.watershed as W

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _example_dir():
    """benchmark/input of the reference checkout ($PIHM_REFERENCE_SRC, or the
    one the reference harness was built from); skips when there is none."""
    import oracle
    src = oracle.reference_src()
    if src is None or not os.path.isdir(os.path.join(src, "benchmark", "input", "example")):
        pytest.skip("the reference's example deck is not here")
    return os.path.join(src, "benchmark", "input")


def _deck_mod():
    from pihm_gpu import capi
    if not os.path.exists(capi.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    from pihm_gpu import deck
    return deck


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def _write(deck, tmp_path, ws, name="gen", **kw):
    d = tmp_path / "input" / name
    deck.write_deck(ws, str(d), name, **kw)
    return str(d)


@pytest.mark.parametrize("seed,shapes", [(3, "mixed"), (4, "rectangle")])
def test_generated_deck_reads_back_bit_for_bit(tmp_path, seed, shapes):
    deck = _deck_mod()
    ws = W.generate(1000, 100, seed=seed, shapes=shapes)
    d = deck.Deck.read(_write(deck, tmp_path, ws), "gen")
    got = d.watershed()
    assert (got.nelem, got.nriver) == (ws.nelem, ws.nriver)
    for k in W.MESH_FIELDS:
        assert _same(np.asarray(got.arrays[k]).reshape(np.shape(ws.arrays[k])), ws.arrays[k]), k
    assert _same(d.initial_state(), W.relax_state(ws))
    c = d.control()
    assert (c.surf_mode, c.riv_mode, c.init_mode) == (ws.surf_mode, ws.riv_mode, 0)
    assert c.step["stepsize"] == ws.stepsize and c.step["reltol"] == 1e-4 and c.step["abstol"] == 1e-5
    assert c.end - c.start == 2 * 86400


def test_reference_reads_the_written_deck_alike(tmp_path):
    """The reference's own readers and Initialize on the same files give the
    same arrays and the same initial state."""
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference build is not here")
    deck = _deck_mod()
    ws = W.generate(1000, 100, seed=5)
    d = deck.Deck.read(_write(deck, tmp_path, ws), "gen")
    got = d.watershed()
    ref = oracle.Reference()
    y0 = ref.load_deck(str(tmp_path), "gen")
    assert (ref.ne, ref.nr) == (ws.nelem, ws.nriver)
    for k in W.MESH_FIELDS:
        n = np.size(ws.arrays[k])
        kind = np.int32 if (k in W.ELEM_INT_FIELDS or k in W.RIVER_INT_FIELDS) else np.float64
        want = ref.export(k, n, kind)
        assert _same(np.asarray(got.arrays[k]).ravel(), want), k
    assert _same(d.initial_state(), y0)


def test_bundled_example_deck():
    """The reference's bundled 535-element example (benchmark/input/example)
    against the arrays and initial state its own readers produce
    (tests/golden/example_watershed.npz, example_calls.npz)."""
    REF_EXAMPLE = _example_dir()
    deck = _deck_mod()
    d = deck.Deck.read(os.path.join(REF_EXAMPLE, "example"), "example",
                       lc_table=os.path.join(REF_EXAMPLE, "vegprmt.tbl"))
    got = d.watershed()
    want = W.Watershed.load(os.path.join(GOLD, "example_watershed.npz"))
    assert (got.nelem, got.nriver) == (535, 20) == (want.nelem, want.nriver)
    for k in W.MESH_FIELDS:
        assert _same(np.asarray(got.arrays[k]).ravel(), np.asarray(want.arrays[k]).ravel()), k
    z = np.load(os.path.join(GOLD, "example_calls.npz"))
    assert _same(d.initial_state(), z["y0"])
    c = d.control()
    assert (c.surf_mode, c.riv_mode, c.step["stepsize"]) == (2, 2, 60.0)
    assert (c.step["reltol"], c.step["abstol"], c.lsm_step) == (1e-3, 1e-4, 900)


def _bc_deck(deck, tmp_path, seed):
    """A generated deck with a Dirichlet and a Neumann boundary series on two
    outer edges, and uniform land cover (one type)."""
    ws = W.generate(1000, 100, seed=seed)
    ws.arrays["rough"] = np.full(ws.nelem, 0.05)
    ws.arrays["rzd"] = np.full(ws.nelem, 1.0)
    bct = np.zeros((ws.nelem, 3), np.int32)
    outer = np.argwhere(np.asarray(ws.arrays["nabr"]).reshape(-1, 3) == 0)
    bct[tuple(outer[0])] = 1
    bct[tuple(outer[1])] = -2
    ws.arrays["bc_type"] = bct
    series = [[("2009-01-01 00:00", 300.0), ("2009-01-02 00:00", 310.0), ("2009-01-03 00:00", 290.0)],
              [("2009-01-01 00:00", 1e-3), ("2009-01-03 00:00", 3e-3)]]
    path = _write(deck, tmp_path, ws, elem_bc_series=series)
    k1, k2 = 3 * outer[0][0] + outer[0][1], 3 * outer[1][0] + outer[1][1]
    return ws, path, k1, k2


def test_boundary_values_match_reference_applybc(tmp_path):
    """ApplyBc (src/forcing.c:127-249) of the reference on the same deck: the
    library's boundary values at the same times, bit for bit."""
    import ctypes
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference build is not here")
    deck = _deck_mod()
    ws, path, k1, k2 = _bc_deck(deck, tmp_path, 6)
    d = deck.Deck.read(path, "gen")
    ref = oracle.Reference()
    ref.load_deck(str(tmp_path), "gen")
    st, en, et, ns = (ctypes.c_int() for _ in range(4))
    ref.lib.ref_model_times(ctypes.byref(st), ctypes.byref(en), ctypes.byref(et), ctypes.byref(ns))
    assert (st.value, en.value) == (d.control().start, d.control().end)
    for t in (st.value, st.value + 6 * 3600 + 60, st.value + 86400, en.value - 7):
        assert ref.lib.ref_apply_forcing(t) == 0
        e, _ = d.bc(t)
        want = ref.export("bc", 3 * ws.nelem)
        assert _same(e[[k1, k2]], want[[k1, k2]]), t
        assert np.count_nonzero(e) == 2


def test_boundary_series_interpolate(tmp_path):
    """Dirichlet and Neumann series: linear between knots, exact at knots,
    refused outside the series."""
    deck = _deck_mod()
    ws, path, k1, k2 = _bc_deck(deck, tmp_path, 6)
    d = deck.Deck.read(path, "gen")
    t0 = d.control().start
    e, _ = d.bc(t0 + 6 * 3600)
    assert e[k1] == (18 * 3600 * 300.0 + 6 * 3600 * 310.0) / 86400.0
    assert e[k2] == ((2 * 86400 - 6 * 3600) * 1e-3 + 6 * 3600 * 3e-3) / (2 * 86400.0)
    assert np.count_nonzero(e) == 2
    assert d.bc(t0 + 86400)[0][k1] == 310.0
    with pytest.raises(deck.DeckError):
        d.bc(t0 + 3 * 86400 + 1)


def test_malformed_and_missing_decks(tmp_path):
    deck = _deck_mod()
    ws = W.generate(1000, 100, seed=7)
    path = _write(deck, tmp_path, ws)
    with pytest.raises(deck.DeckError) as e:
        deck.Deck.read(str(tmp_path / "nowhere"), "gen")
    assert e.value.code == -20 and "gen.riv" in str(e.value)
    mesh = os.path.join(path, "gen.mesh")
    lines = open(mesh).read().splitlines()
    lines[5] = "5 1 2"  # an element line cut short
    open(mesh, "w").write("\n".join(lines) + "\n")
    with pytest.raises(deck.DeckError) as e:
        deck.Deck.read(path, "gen")
    assert e.value.code == -21 and "gen.mesh" in str(e.value) and "line 6" in str(e.value)


def test_comments_blank_lines_and_case(tmp_path):
    """Lines that are blank or start with '#' are skipped and keywords compare
    without case, as the reference's NextLine / ReadKeyword do."""
    deck = _deck_mod()
    ws = W.generate(1000, 100, seed=8)
    path = _write(deck, tmp_path, ws)
    para = os.path.join(path, "gen.para")
    text = open(para).read().replace("SURF_MODE", "\n# a comment\n\n   surf_mode")
    open(para, "w").write(text)
    d = deck.Deck.read(path, "gen")
    assert d.control().surf_mode == ws.surf_mode
