"""Land-surface step (include/pihm_land.h) on the CPU side: the deck's
land-surface parameters and forcing series against the reference's own
Initialize, the restatement (oracle/land_oracle.c) against the reference's
own ApplyForc + IntcpSnowEt and against its golden vectors, and the writer's
round trip."""
import os

import numpy as np
import pytest

import pihm_gpu.land as L
from parity import land_deck, land_states

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _example_dir():
    """benchmark/input of the reference checkout ($PIHM_REFERENCE_SRC, or the
    one the reference harness was built from); skips when there is none."""
    import oracle
    src = oracle.reference_src()
    if src is None or not os.path.isdir(os.path.join(src, "benchmark", "input", "example")):
        pytest.skip("the reference's example deck is not here")
    return os.path.join(src, "benchmark", "input")
FIELDS = ("prcp", "pcpdrp", "edir", "ett", "ec", "drip", "cmc", "sneqv")


def _have_lib():
    from pihm_gpu import capi
    if not os.path.exists(capi.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")


def _ref():
    import oracle
    if not oracle.ref_available():
        pytest.skip("the reference build is not here")
    return oracle.Reference()


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def golden_land():
    """(watershed, Land, fixture) of tests/golden/land_calls.npz."""
    import pihm_gpu.watershed as W
    z = np.load(os.path.join(GOLD, "land_calls.npz"))
    ws = W.Watershed.load(os.path.join(GOLD, "land_watershed.npz"))
    params = {k: z["p_" + k] for k in L.PARAM_I32 + L.PARAM_F64}
    land = L.Land(params, tuple(z["cal"]), z["meteo_len"], z["meteo_time"], z["meteo_data"], z["lai_len"],
                  z["lai_time"], z["lai_data"])
    return ws, land, z


def golden_steps(z):
    return sorted(int(k[1:].split("_")[0]) for k in z.files if k.startswith("s") and k.endswith("_prcp"))


def test_oracle_land_against_golden():
    """The restatement reproduces the reference's 48 land-surface steps bit for
    bit (the fixture holds every 4th); runs where the reference is absent."""
    import oracle
    ws, land, z = golden_land()
    o = oracle.OracleLand(land, ws)
    o.set_state(None, None)
    want_at = set(golden_steps(z))
    t, dt = int(z["start"]), float(z["lsm_step"])
    for s, (unsat, gw) in enumerate(land_states(ws.arrays["depth"], 7, max(want_at))):
        assert o.step(t, dt, unsat, gw) == 0
        if s + 1 in want_at:
            for k in FIELDS:
                assert np.array_equal(_bits(o.get(k)), _bits(z[f"s{s + 1}_{k}"])), (s + 1, k)
        t += int(dt)
    # the steps exercised snow, canopy storage, drip and both ET branches
    for k in ("sneqv", "cmc", "drip", "ec", "ett"):
        assert any(np.count_nonzero(z[f"s{s}_{k}"]) for s in want_at), k


def test_oracle_land_refuses_times_outside_the_series():
    import oracle
    ws, land, z = golden_land()
    o = oracle.OracleLand(land, ws)
    lo, hi = land.time_range()
    ne = ws.nelem
    assert o.step(lo - 1, 900.0, np.zeros(ne), np.zeros(ne)) == -1
    assert o.step(hi + 1, 900.0, np.zeros(ne), np.zeros(ne)) == -1
    assert o.step(hi, 900.0, np.zeros(ne), np.zeros(ne)) == 0


def test_monthly_tables_match_reference():
    """MonthlyLai, MonthlyRl and MonthlyMf for all 40 land types and 12 months."""
    import oracle
    ref = _ref()
    _have_lib()
    ws, land, _ = golden_land()
    o = oracle.OracleLand(land, ws)
    for month in range(12):
        t = L.epoch(f"2009-{month + 1:02d}-15 12:00")
        for lc in range(1, L.NLC + 1):
            assert np.array_equal(o.monthly(t, lc), ref.monthly(t, lc)), (month, lc)


def test_deck_land_matches_reference_initialize(tmp_path):
    """The library's reader gives the land-surface parameters the reference's
    InitSoil / InitLc / InitForc leave (FieldCapacity and WiltingPoint
    included) and the forcing series as written."""
    _have_lib()
    ref = _ref()
    from pihm_gpu import deck as D
    path = land_deck(str(tmp_path))
    d = D.Deck.read(path, "gen")
    land = d.land()
    ref.load_deck(str(tmp_path), "gen")
    ne = d.watershed().nelem
    for k in L.PARAM_I32 + L.PARAM_F64:
        want = ref.export(k, ne, np.int32 if k in L.PARAM_I32 else np.float64)
        assert np.array_equal(np.asarray(land.params[k]), want), k


def test_bundled_example_land_matches_reference():
    _have_lib()
    REF_EXAMPLE = _example_dir()
    ref = _ref()
    import oracle
    from pihm_gpu import deck as D
    d = D.Deck.read(os.path.join(REF_EXAMPLE, "example"), "example", lc_table=os.path.join(REF_EXAMPLE, "vegprmt.tbl"))
    land, ws, c = d.land(), d.watershed(), d.control()
    y0 = ref.load_deck(os.path.join(REF_EXAMPLE, ".."), "example")
    ne = ws.nelem
    for k in L.PARAM_I32 + L.PARAM_F64:
        want = ref.export(k, ne, np.int32 if k in L.PARAM_I32 else np.float64)
        assert np.array_equal(np.asarray(land.params[k]), want), k
    assert (land.meteo_len.size, land.lai_len.size) == (1, 1)
    # a day of land-surface steps from the relaxed state, bit for bit
    o = oracle.OracleLand(land, ws)
    unsat, gw = y0[ne:2 * ne], y0[2 * ne:3 * ne]
    ref.land_set_state(unsat, gw, np.zeros(ne), np.zeros(ne))
    t = c.start
    for _ in range(96):
        ref.land_step(t, c.lsm_step)
        assert o.step(t, c.lsm_step, unsat, gw) == 0
        t += c.lsm_step
    for k, v in ref.land_fields().items():
        assert np.array_equal(_bits(o.get(k)), _bits(v)), k


def test_oracle_land_bit_exact_with_reference(tmp_path):
    """Four days of land-surface steps on a live deck, every step compared."""
    _have_lib()
    ref = _ref()
    import oracle
    from pihm_gpu import deck as D
    path = land_deck(str(tmp_path))
    d = D.Deck.read(path, "gen")
    land, ws, c = d.land(), d.watershed(), d.control()
    ref.load_deck(str(tmp_path), "gen")
    o = oracle.OracleLand(land, ws)
    ne = ws.nelem
    ref.land_set_state(None, None, np.zeros(ne), np.zeros(ne))
    t = c.start
    for s, (unsat, gw) in enumerate(land_states(ws.arrays["depth"], 3, 4 * 96 - 1)):
        ref.land_set_state(unsat, gw, None, None)
        ref.land_step(t, c.lsm_step)
        assert o.step(t, c.lsm_step, unsat, gw) == 0
        for k, v in ref.land_fields().items():
            assert np.array_equal(_bits(o.get(k)), _bits(v)), (s, k)
        t += c.lsm_step


def test_written_forcing_reads_back(tmp_path):
    """write_deck's .meteo/.lai/.att and land-cover rows read back as written."""
    _have_lib()
    from pihm_gpu import deck as D
    import pihm_gpu.watershed as W
    path = land_deck(str(tmp_path))
    d = D.Deck.read(path, "gen")
    got = d.land()
    ws = W.generate(1000, 100, seed=11)
    want = L.synthetic_land(ws, seed=5, hours=96, per_type=True)
    for k in ("meteo_len", "meteo_time", "meteo_data", "lai_len", "lai_time", "lai_data"):
        assert np.array_equal(getattr(got, k), getattr(want, k)), k
    for k in ("lc_type", "meteo_type", "lai_type", "shdfac", "albedomin", "albedomax", "rsmin", "rgl"):
        assert np.array_equal(got.params[k], want.params[k]), k
    assert got.cal == (1.0, 1.0, 1.0)
    assert d.control().lsm_step == 900


def test_hot_start_restores_canopy_and_snow(tmp_path):
    """INIT_MODE 1: the restart file's state, canopy storage and snow, as the
    reference's ReadIc + InitVar leave them (ws.cmc, ws.sneqv)."""
    import ctypes
    _have_lib()
    ref = _ref()
    from pihm_gpu import capi, deck as D
    path = land_deck(str(tmp_path))
    d0 = D.Deck.read(path, "gen")
    ws = d0.watershed()
    ne, nr = ws.nelem, ws.nriver
    rng = np.random.default_rng(4)
    y = d0.initial_state() * rng.uniform(0.5, 1.5, ws.neq)
    cmc, sneqv = rng.uniform(0.0, 5e-4, ne), rng.uniform(0.0, 2e-2, ne)
    lib = capi.load()
    P = ctypes.POINTER(ctypes.c_double)
    lib.pihm_ic_write.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, P, P, P]
    assert lib.pihm_ic_write(os.path.join(path, "gen.ic").encode(), ne, nr, y.ctypes.data_as(P),
                             cmc.ctypes.data_as(P), sneqv.ctypes.data_as(P)) == 0
    para = os.path.join(path, "gen.para")
    text = open(para).read()
    open(para, "w").write(text.replace("INIT_MODE 0", "INIT_MODE 1"))
    d = D.Deck.read(path, "gen")
    got_c, got_s = d.initial_storage()
    assert np.array_equal(d.initial_state(), y)
    y_ref = ref.load_deck(str(tmp_path), "gen")
    assert np.array_equal(y_ref, y)
    assert np.array_equal(got_c, ref.export("cmc", ne)) and np.array_equal(got_c, cmc)
    assert np.array_equal(got_s, ref.export("sneqv", ne)) and np.array_equal(got_s, sneqv)


def test_malformed_forcing_files(tmp_path):
    """A missing .meteo, a record cut short and an element naming a station
    the file does not hold come back as errors naming the file (the reference
    exits there)."""
    _have_lib()
    from pihm_gpu import deck as D
    path = land_deck(str(tmp_path))
    meteo = os.path.join(path, "gen.meteo")
    text = open(meteo).read()
    os.remove(meteo)
    with pytest.raises(D.DeckError) as e:
        D.Deck.read(path, "gen")
    assert e.value.code == -20 and "gen.meteo" in str(e.value)
    lines = text.splitlines()
    lines[5] = " ".join(lines[5].split()[:5])  # a record with three of its seven values
    open(meteo, "w").write("\n".join(lines) + "\n")
    with pytest.raises(D.DeckError) as e:
        D.Deck.read(path, "gen")
    assert e.value.code == -21 and "gen.meteo" in str(e.value) and "line 6" in str(e.value)
    open(meteo, "w").write(text)
    att = os.path.join(path, "gen.att")
    rows = open(att).read().splitlines()
    f = rows[1].split()
    f[4] = "99"  # METEO column: a station the file does not hold
    rows[1] = " ".join(f)
    open(att, "w").write("\n".join(rows) + "\n")
    with pytest.raises(D.DeckError) as e:
        D.Deck.read(path, "gen")
    assert e.value.code == -22 and "station 99" in str(e.value)
