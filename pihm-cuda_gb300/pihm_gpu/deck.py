"""PIHM input decks through the library's reader (include/pihm_deck.h), and a
writer that stores a generated watershed as a deck.

    d = Deck.read("input/example", "example")       # .riv .mesh .att .soil ...
    ws = d.watershed()                              # the initialised mesh
    y0 = d.initial_state()                          # RelaxIc or the .ic file
    elem_bc, river_bc = d.bc(t)                     # ApplyBc at time t

A deck is the reference's input set (src/read_alloc.c:3-162): <proj>.riv,
.mesh, .att, .soil, .para, .bc, <project>.calib (and <project>.ic for a hot
start) in one directory, plus the land-cover table vegprmt.tbl in its parent
(the reference's input/vegprmt.tbl).  `write_deck` writes that set for a
watershed from `watershed.generate`, one soil row and one land-cover row per
element, every number with 17 significant digits, so that reading it back
gives the generator's arrays bit for bit.
"""
from __future__ import annotations

import ctypes
import dataclasses
import datetime
import os

import numpy as np

from . import capi
from . import land as land_mod
from .batch import StepControlC
from .meshdesc import MeshDesc, _INTS, _ORDER
from .watershed import Watershed

_VP = ctypes.c_void_p


class DeckControlC(ctypes.Structure):
    _fields_ = [("surf_mode", ctypes.c_int32), ("riv_mode", ctypes.c_int32), ("unsat_mode", ctypes.c_int32),
                ("init_mode", ctypes.c_int32), ("start", ctypes.c_int64), ("end", ctypes.c_int64),
                ("lsm_step", ctypes.c_int32), ("step", StepControlC)]


def _lib():
    lib = capi.load()
    if not getattr(lib, "_deck_sigs", False):
        lib.pihm_deck_read.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                       ctypes.POINTER(_VP)]
        lib.pihm_deck_read.restype = ctypes.c_int
        lib.pihm_deck_error.argtypes = []
        lib.pihm_deck_error.restype = ctypes.c_char_p
        lib.pihm_deck_free.argtypes = [_VP]
        lib.pihm_deck_free.restype = None
        lib.pihm_deck_mesh.argtypes = [_VP, ctypes.POINTER(MeshDesc)]
        lib.pihm_deck_mesh.restype = ctypes.c_int
        lib.pihm_deck_control_get.argtypes = [_VP, ctypes.POINTER(DeckControlC)]
        lib.pihm_deck_control_get.restype = ctypes.c_int
        lib.pihm_deck_initial_state.argtypes = [_VP, ctypes.POINTER(ctypes.c_double)]
        lib.pihm_deck_initial_state.restype = ctypes.c_int
        lib.pihm_deck_bc.argtypes = [_VP, ctypes.c_int64, ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double)]
        lib.pihm_deck_bc.restype = ctypes.c_int
        lib.pihm_deck_land.argtypes = [_VP, ctypes.POINTER(land_mod.LandParamsC),
                                       ctypes.POINTER(land_mod.ForcingSeriesC)]
        lib.pihm_deck_land.restype = ctypes.c_int
        lib.pihm_deck_initial_storage.argtypes = [_VP, ctypes.POINTER(ctypes.c_double),
                                                  ctypes.POINTER(ctypes.c_double)]
        lib.pihm_deck_initial_storage.restype = ctypes.c_int
        lib._deck_sigs = True
    return lib


class DeckError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"pihm_deck_read: {message} (code {code})")
        self.code = code


@dataclasses.dataclass
class DeckControl:
    surf_mode: int
    riv_mode: int
    unsat_mode: int
    init_mode: int
    start: int
    end: int
    lsm_step: int
    step: dict


class Deck:
    """One deck read and initialised by the library."""

    CORR_ELEV = 1

    def __init__(self, handle, lib):
        self.h = handle
        self.lib = lib

    @staticmethod
    def read(directory: str, project: str, lc_table: str | None = None, corr_elev: bool = False) -> "Deck":
        lib = _lib()
        h = _VP()
        rc = lib.pihm_deck_read(directory.encode(), project.encode(),
                                lc_table.encode() if lc_table else None,
                                Deck.CORR_ELEV if corr_elev else 0, ctypes.byref(h))
        if rc != 0:
            raise DeckError(rc, lib.pihm_deck_error().decode())
        return Deck(h, lib)

    def close(self):
        if self.h:
            self.lib.pihm_deck_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def control(self) -> DeckControl:
        c = DeckControlC()
        capi._check("pihm_deck_control_get", self.lib.pihm_deck_control_get(self.h, ctypes.byref(c)))
        step = {n: getattr(c.step, n) for n, _ in StepControlC._fields_}
        return DeckControl(c.surf_mode, c.riv_mode, c.unsat_mode, c.init_mode, c.start, c.end, c.lsm_step, step)

    def watershed(self) -> Watershed:
        """The initialised mesh as a Watershed (copies, reference order)."""
        m = MeshDesc()
        capi._check("pihm_deck_mesh", self.lib.pihm_deck_mesh(self.h, ctypes.byref(m)))
        ne, nr = m.nelem, m.nriver
        per_edge = {"nabr", "bc_type", "edge", "nabrdist", "nabr_x", "nabr_y"}
        river = {"down", "leftele", "rightele", "intrpl_ord", "riverbc_type"}
        arrays = {}
        for name in _ORDER:
            n = nr if (name in river or name.startswith("riv_")) else (3 * ne if name in per_edge else ne)
            ptr = getattr(m, name)
            if n == 0:
                arrays[name] = np.zeros(0, np.int32 if name in _INTS else np.float64)
                continue
            a = np.ctypeslib.as_array(ptr, shape=(n,)).copy()
            arrays[name] = a.reshape(ne, 3) if name in per_edge else a
        ctrl = self.control()
        return Watershed(ne, nr, arrays, surf_mode=ctrl.surf_mode, riv_mode=ctrl.riv_mode,
                         stepsize=float(ctrl.step["stepsize"]))

    def initial_state(self) -> np.ndarray:
        m = MeshDesc()
        capi._check("pihm_deck_mesh", self.lib.pihm_deck_mesh(self.h, ctypes.byref(m)))
        y = np.empty(3 * m.nelem + 2 * m.nriver)
        capi._check("pihm_deck_initial_state",
                    self.lib.pihm_deck_initial_state(self.h, y.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return y

    def initial_storage(self):
        """(cmc, sneqv) at the start: zeros after RelaxIc, the .ic file's values
        on a hot start."""
        m = MeshDesc()
        capi._check("pihm_deck_mesh", self.lib.pihm_deck_mesh(self.h, ctypes.byref(m)))
        cmc, sneqv = np.zeros(m.nelem), np.zeros(m.nelem)
        P = ctypes.POINTER(ctypes.c_double)
        capi._check("pihm_deck_initial_storage",
                    self.lib.pihm_deck_initial_storage(self.h, cmc.ctypes.data_as(P), sneqv.ctypes.data_as(P)))
        return cmc, sneqv

    def land(self) -> "land_mod.Land":
        """The land-surface model (parameters and forcing series, copies)."""
        p, s = land_mod.LandParamsC(), land_mod.ForcingSeriesC()
        capi._check("pihm_deck_land", self.lib.pihm_deck_land(self.h, ctypes.byref(p), ctypes.byref(s)))
        ne = p.nelem

        def arr(ptr, n, shape=None):
            if n == 0:
                return np.zeros(shape or (0,))
            a = np.ctypeslib.as_array(ptr, shape=(n,)).copy()
            return a.reshape(shape) if shape else a
        params = {k: arr(getattr(p, k), ne) for k in land_mod.PARAM_I32 + land_mod.PARAM_F64}
        ml = arr(s.meteo_len, s.nmeteo).astype(np.int32)
        nmk = int(ml.sum())
        ll = arr(s.lai_len, s.nlai).astype(np.int32) if s.nlai else np.zeros(0, np.int32)
        nlk = int(ll.sum())
        return land_mod.Land(params, (p.cal_edir, p.cal_ec, p.cal_ett), ml, arr(s.meteo_time, nmk).astype(np.int64),
                             arr(s.meteo_data, nmk * land_mod.NVAR, (nmk, land_mod.NVAR)), ll,
                             arr(s.lai_time, nlk).astype(np.int64) if nlk else np.zeros(0, np.int64),
                             arr(s.lai_data, nlk) if nlk else np.zeros(0))

    def bc(self, t: int):
        """(elem_bc [nelem*3], river_bc [nriver]) at time t (s since 1970 UTC)."""
        m = MeshDesc()
        capi._check("pihm_deck_mesh", self.lib.pihm_deck_mesh(self.h, ctypes.byref(m)))
        e = np.zeros(3 * m.nelem)
        r = np.zeros(m.nriver)
        P = ctypes.POINTER(ctypes.c_double)
        rc = self.lib.pihm_deck_bc(self.h, int(t), e.ctypes.data_as(P), r.ctypes.data_as(P))
        if rc != 0:
            raise DeckError(rc, self.lib.pihm_deck_error().decode())
        return e, r


# ----------------------------------------------------------------------------
# writer
# ----------------------------------------------------------------------------

def _num(v) -> str:
    return repr(float(v))


PRINT_CTRL = ("SURF", "UNSAT", "GW", "RIVSTG", "RIVGW", "SNOW", "CMC", "INFIL", "RECHARGE", "EC", "ETT",
              "EDIR", "RIVFLX0", "RIVFLX1", "RIVFLX2", "RIVFLX3", "RIVFLX4", "RIVFLX5", "RIVFLX6", "RIVFLX7",
              "RIVFLX8", "RIVFLX9", "RIVFLX10", "SUBFLX", "SURFFLX", "IC")


def write_deck(ws: Watershed, directory: str, project: str, *, start: str = "2009-01-01 00:00",
               end: str = "2009-01-03 00:00", reltol: float = 1e-4, abstol: float = 1e-5,
               initstep: float = 5e-5, elem_bc_series=None, lc_table: str | None = None,
               land: "land_mod.Land | None" = None, lsm_step: int | None = None) -> None:
    """Write `ws` (from watershed.generate, which keeps its node mesh) as a deck
    in `directory`, and the land-cover table to `lc_table` (default
    <directory>/../vegprmt.tbl).  elem_bc_series: optional list of
    [(YYYY-MM-DD hh:mm, value), ...] series that ws.arrays["bc_type"] names
    (1-based, positive Dirichlet head, negative Neumann flux).

    land: a land.Land whose element land types, stations and LAI series go to
    the .att file, its series to .meteo and .lai, and its per-type canopy
    parameters (shdfac, albedo, rsmin, rgl; rsmax, topt, cfactr shared) with
    the watershed's roughness and root depth to the land-cover table; every
    element of a type must carry the same values.  Its soil moistures are not
    written: the reader derives them from the soil rows.  Without it, one
    station with a two-knot mild record and one LAI series are written.
    lsm_step: LSM_STEP (default the model step)."""
    if ws.nodes is None:
        raise ValueError("the watershed carries no node mesh (watershed.generate keeps it)")
    a, nd = ws.arrays, ws.nodes
    ne, nr = ws.nelem, ws.nriver
    os.makedirs(directory, exist_ok=True)
    proj = project.split(".")[0]
    base = os.path.join(directory, proj)
    nabr = np.asarray(a["nabr"]).reshape(ne, 3).copy()
    # element neighbours before InitRiver marked the river edges (src/init_river.c:25-35)
    for s in range(nr):
        L, R = int(a["leftele"][s]) - 1, int(a["rightele"][s]) - 1
        nabr[L][nabr[L] == -(s + 1)] = R + 1
        nabr[R][nabr[R] == -(s + 1)] = L + 1
    tri = np.asarray(nd["tri"])
    with open(base + ".mesh", "w") as f:
        f.write(f"NUMELE {ne}\nINDEX NODE1 NODE2 NODE3 NABR1 NABR2 NABR3\n")
        for i in range(ne):
            f.write(f"{i + 1} {tri[i, 0] + 1} {tri[i, 1] + 1} {tri[i, 2] + 1} {nabr[i, 0]} {nabr[i, 1]} {nabr[i, 2]}\n")
        nn = len(nd["x"])
        f.write(f"NUMNODE {nn}\nINDEX X Y ZMIN ZMAX\n")
        for k in range(nn):
            f.write(f"{k + 1} {_num(nd['x'][k])} {_num(nd['y'][k])} {_num(nd['zmin'][k])} {_num(nd['zmax'][k])}\n")
    bct = np.asarray(a["bc_type"]).reshape(ne, 3)
    # one land-cover type when roughness and root depth are uniform (the
    # reference's forcing code indexes fixed 40-row tables by type), else one
    # per element
    uniform_lc = bool(np.all(a["rough"] == a["rough"][0]) and np.all(a["rzd"] == a["rzd"][0]))
    nlc = 1 if uniform_lc else ne
    if land is not None:
        lc_of = np.asarray(land.params["lc_type"], np.int64)
        met_of = np.asarray(land.params["meteo_type"], np.int64)
        lai_of = np.asarray(land.params["lai_type"], np.int64)
        nlc = int(lc_of.max())
    else:
        lc_of = np.ones(ne, np.int64) if uniform_lc else np.arange(1, ne + 1)
        met_of = np.ones(ne, np.int64)
        lai_of = np.ones(ne, np.int64)
    with open(base + ".att", "w") as f:
        f.write("INDEX SOIL GEOL LC METEO LAI SS BC0 BC1 BC2\n")
        for i in range(ne):
            f.write(f"{i + 1} {i + 1} 1 {lc_of[i]} {met_of[i]} {lai_of[i]} 0 {bct[i, 0]} {bct[i, 1]} {bct[i, 2]}\n")
    kmacv_ro, kmach_ro, dinf = 100.0, 1000.0, 0.1
    if not (np.array_equal(a["kmacv"], kmacv_ro * a["kinfv"]) and np.array_equal(a["kmach"], kmach_ro * a["ksath"])
            and np.all(a["dinf"] == dinf)):
        raise ValueError("the deck format holds one macropore ratio and one DINF for all elements")
    with open(base + ".soil", "w") as f:
        f.write(f"NUMSOIL {ne}\nINDEX SILT CLAY OM BD KINF KSATV KSATH MAXSMC MINSMC ALPHA BETA MACHF MACVF DMAC QTZ\n")
        for i in range(ne):
            f.write(" ".join([str(i + 1), "40.0", "20.0", "2.5", "1.3"] + [_num(a[k][i]) for k in (
                "kinfv", "ksatv", "ksath", "porosity")] + ["0.0"] + [_num(a[k][i]) for k in (
                    "alpha", "beta", "areafh", "areafv", "dmac")] + ["0.5"]) + "\n")
        f.write(f"DINF {_num(dinf)}\nKMACV_RO {_num(kmacv_ro)}\nKMACH_RO {_num(kmach_ro)}\n")
    lc = lc_table or os.path.join(directory, "..", "vegprmt.tbl")
    shared = {"topt": 298.0, "cfactr": 0.5, "rsmax": 5000.0}
    rows = []
    if land is not None:
        P = land.params
        for k in shared:
            v = np.asarray(P[k])
            if not np.all(v == v[0]):
                raise ValueError(f"the land-cover table holds one {k} for all types")
            shared[k] = float(v[0])
        for t in range(1, nlc + 1):
            idx = np.flatnonzero(lc_of == t)
            if idx.size == 0:  # an unused type: any valid row
                rows.append((0.5, 1.0, 100.0, 30.0, 0.15, 0.2, 0.1))
                continue
            row = tuple(np.asarray(v)[idx] for v in (P["shdfac"], a["rzd"], P["rsmin"], P["rgl"],
                                                     P["albedomin"], P["albedomax"], a["rough"]))
            if any(not np.all(v == v[0]) for v in row):
                raise ValueError(f"elements of land type {t} differ in a land-cover table value")
            rows.append(tuple(float(v[0]) for v in row))
    else:
        for i in range(nlc):
            rows.append((0.8, float(a["rzd"][i]), 100.0, 30.0, 0.15, 0.2, float(a["rough"][i])))
    with open(lc, "w") as f:
        f.write(f"NUMLC {nlc}\nINDEX SHDFAC DROOT RS RGL HS SNUP LAIMIN LAIMAX EMISMIN EMISMAX ALBMIN ALBMAX "
                "Z0MIN Z0MAX ROUGH\n")
        for i, (veg, rzd, rs, rgl, amin, amax, rough) in enumerate(rows):
            f.write(f"{i + 1} {_num(veg)} {_num(rzd)} {_num(rs)} {_num(rgl)} 47.35 0.08 1.0 4.0 0.93 0.97 "
                    f"{_num(amin)} {_num(amax)} 0.1 0.5 {_num(rough)}\n")
        f.write(f"TOPT_DATA {_num(shared['topt'])}\nCFACTR_DATA {_num(shared['cfactr'])}\n"
                f"RSMAX_DATA {_num(shared['rsmax'])}\nBARE 19\nNATURAL 5\n")
    with open(base + ".riv", "w") as f:
        f.write(f"NUMRIV {nr}\nINDEX FROM TO DOWN LEFT RIGHT SHAPE MATL BC RES\n")
        for s in range(nr):
            f.write(f"{s + 1} {nd['from_n'][s] + 1} {nd['to_n'][s] + 1} {a['down'][s]} {a['leftele'][s]} "
                    f"{a['rightele'][s]} {s + 1} {s + 1} {a['riverbc_type'][s]} 0\n")
        f.write(f"SHAPE {nr}\nINDEX DPTH OINT CWID\n")
        for s in range(nr):
            f.write(f"{s + 1} {_num(a['riv_depth'][s])} {a['intrpl_ord'][s]} {_num(a['riv_coeff'][s])}\n")
        f.write(f"MATERIAL {nr}\nINDEX ROUGH CWR KH KV BEDTHCK\n")
        for s in range(nr):
            f.write(f"{s + 1} {_num(a['riv_rough'][s])} {_num(a['riv_cwr'][s])} {_num(a['riv_ksath'][s])} "
                    f"{_num(a['riv_ksatv'][s])} {_num(a['riv_bedthick'][s])}\n")
        f.write("BC 0\nRES 0\n")
    step = int(ws.stepsize)
    with open(base + ".para", "w") as f:
        f.write(f"SIMULATION_MODE 0\nINIT_MODE 0\nASCII_OUTPUT 0\nWATBAL_OUTPUT 0\nWRITE_IC 0\n"
                f"UNSAT_MODE 2\nSURF_MODE {ws.surf_mode}\nRIV_MODE {ws.riv_mode}\nSTART {start}\nEND {end}\n"
                f"MAX_SPINUP_YEAR 0\nMODEL_STEPSIZE {step}\nLSM_STEP {lsm_step or step}\n"
                f"ABSTOL {_num(abstol)}\nRELTOL {_num(reltol)}\nINIT_SOLVER_STEP {_num(initstep)}\n"
                "NUM_NONCOV_FAIL 0.0\nMAX_NONLIN_ITER 3.0\nMIN_NONLIN_ITER 1.0\nDECR_FACTOR 1.2\n"
                "INCR_FACTOR 1.2\nMIN_MAXSTEP 1.0\n")
        for k in PRINT_CTRL:
            f.write(f"{k} 0\n")
    with open(os.path.join(directory, project + ".calib"), "w") as f:
        cal = dict(zip(("EDIR", "EC", "ETT"), land.cal)) if land is not None else {}
        for k in ("KSATH", "KSATV", "KINF", "KMACSATH", "KMACSATV", "DINF", "DROOT", "DMAC", "POROSITY",
                  "ALPHA", "BETA", "MACVF", "MACHF", "VEGFRAC", "ALBEDO", "ROUGH", "EC", "ETT", "EDIR",
                  "ROUGH_RIV", "KRIVH", "KRIVV", "BEDTHCK", "RIV_DPTH", "RIV_WDTH"):
            f.write(f"{k} {_num(cal.get(k, 1.0))}\n")
        f.write("SCENARIO\nPRCP 1.0\nSFCTMP 0.0\n")
    # forcing files (src/read_forc.c, src/read_lai.c)
    def stamp(t):
        return datetime.datetime.fromtimestamp(int(t), datetime.timezone.utc).strftime("%Y-%m-%d %H:%M")
    with open(base + ".meteo", "w") as f:
        if land is None:
            f.write("METEO_TS 1 WIND_LVL 10.0\nTIME PRCP SFCTMP RH SFCSPD SOLAR LONGWV PRES\n"
                    "TS kg/m2/s K % m/s W/m2 W/m2 Pa\n")
            for when in (start, end):
                f.write(f"{when} 0.0 283.15 80.0 2.0 0.0 300.0 100000.0\n")
        else:
            o = 0
            for k, n in enumerate(np.asarray(land.meteo_len)):
                at = np.flatnonzero(met_of == k + 1)
                zl = float(land.params["zlvl_wind"][at[0]]) if at.size else 10.0
                f.write(f"METEO_TS {k + 1} WIND_LVL {_num(zl)}\nTIME PRCP SFCTMP RH SFCSPD SOLAR LONGWV PRES\n"
                        "TS kg/m2/s K % m/s W/m2 W/m2 Pa\n")
                for j in range(o, o + int(n)):
                    f.write(stamp(land.meteo_time[j]) + " " + " ".join(_num(v) for v in land.meteo_data[j]) + "\n")
                o += int(n)
    with open(base + ".lai", "w") as f:
        if land is None:
            f.write("LAI_TS 1\nTIME LAI\nTS m2/m2\n")
            for when in (start, end):
                f.write(f"{when} 1.0\n")
        else:
            o = 0
            for k, n in enumerate(np.asarray(land.lai_len)):
                f.write(f"LAI_TS {k + 1}\nTIME LAI\nTS m2/m2\n")
                for j in range(o, o + int(n)):
                    f.write(f"{stamp(land.lai_time[j])} {_num(land.lai_data[j])}\n")
                o += int(n)
    if elem_bc_series:
        with open(base + ".bc", "w") as f:
            for k, series in enumerate(elem_bc_series):
                f.write(f"BC_TS {k + 1}\nTIME VALUE\nTS m\n")
                for when, v in series:
                    f.write(f"{when} {_num(v)}\n")
