"""The land-surface step on the GPU (include/pihm_land.h): forcing series
interpolated at the step's time and interception, snow and
evapotranspiration, writing the right-hand side's forcing in place.

    land = deck.land()                       # or synthetic_land(ws, ...)
    gpu = capi.GpuRhs(ws)
    gpu.land_init(land)
    gpu.land_step(t, lsm_step, y_internal_ptr)   # every LSM_STEP seconds
    gpu.land_get(FIELDS["cmc"])

`Land` holds the per-element parameters and the series as numpy arrays in
reference order; `synthetic_land` makes a seeded one for a generated
watershed (hourly station records with rain, snow and melt, land types with
and without leaf-area series), for tests and benchmarks.
"""
from __future__ import annotations

import ctypes
import dataclasses
import datetime

import numpy as np

from . import capi

_F64P = ctypes.POINTER(ctypes.c_double)
_I32P = ctypes.POINTER(ctypes.c_int32)
_I64P = ctypes.POINTER(ctypes.c_int64)
_VP = ctypes.c_void_p

NVAR = 7  # PRCP SFCTMP RH SFCSPD SOLAR LONGWV PRES
NLC = 40
FIELDS = {"prcp": 0, "pcpdrp": 1, "edir": 2, "ett": 3, "ec": 4, "drip": 5, "cmc": 6, "sneqv": 7}
PARAM_F64 = ("albedomin", "albedomax", "shdfac", "cmcfactr", "cfactr", "rgl", "rsmin", "rsmax", "topt",
             "smcmin", "smcwlt", "smcref", "zlvl_wind")
PARAM_I32 = ("lc_type", "meteo_type", "lai_type")


class LandParamsC(ctypes.Structure):
    _fields_ = ([("nelem", ctypes.c_int32)] + [(k, _I32P) for k in PARAM_I32] + [(k, _F64P) for k in PARAM_F64]
                + [("cal_edir", ctypes.c_double), ("cal_ec", ctypes.c_double), ("cal_ett", ctypes.c_double)])


class ForcingSeriesC(ctypes.Structure):
    _fields_ = [("nmeteo", ctypes.c_int32), ("meteo_len", _I32P), ("meteo_time", _I64P), ("meteo_data", _F64P),
                ("nlai", ctypes.c_int32), ("lai_len", _I32P), ("lai_time", _I64P), ("lai_data", _F64P)]


def _p(a, t):
    return None if a is None or a.size == 0 else a.ctypes.data_as(t)


@dataclasses.dataclass
class Land:
    """Per-element parameters (reference order) and forcing series."""
    params: dict            # PARAM_I32 -> int32 [ne], PARAM_F64 -> float64 [ne]
    cal: tuple              # (EDIR, EC, ETT) calibration factors
    meteo_len: np.ndarray   # int32 [nmeteo]
    meteo_time: np.ndarray  # int64 [knots]
    meteo_data: np.ndarray  # float64 [knots, 7], climate scenario applied
    lai_len: np.ndarray     # int32 [nlai]
    lai_time: np.ndarray    # int64 [knots]
    lai_data: np.ndarray    # float64 [knots]

    @property
    def nelem(self) -> int:
        return int(self.params["lc_type"].size)

    def structs(self):
        """(LandParamsC, ForcingSeriesC) pointing into this object's arrays."""
        for k in PARAM_I32:
            self.params[k] = np.ascontiguousarray(self.params[k], np.int32)
        for k in PARAM_F64:
            self.params[k] = np.ascontiguousarray(self.params[k], np.float64)
        self.meteo_len = np.ascontiguousarray(self.meteo_len, np.int32)
        self.meteo_time = np.ascontiguousarray(self.meteo_time, np.int64)
        self.meteo_data = np.ascontiguousarray(self.meteo_data, np.float64)
        self.lai_len = np.ascontiguousarray(self.lai_len, np.int32)
        self.lai_time = np.ascontiguousarray(self.lai_time, np.int64)
        self.lai_data = np.ascontiguousarray(self.lai_data, np.float64)
        p = LandParamsC(self.nelem, *[_p(self.params[k], _I32P) for k in PARAM_I32],
                        *[_p(self.params[k], _F64P) for k in PARAM_F64], *[float(c) for c in self.cal])
        s = ForcingSeriesC(self.meteo_len.size, _p(self.meteo_len, _I32P), _p(self.meteo_time, _I64P),
                           _p(self.meteo_data, _F64P), self.lai_len.size, _p(self.lai_len, _I32P),
                           _p(self.lai_time, _I64P), _p(self.lai_data, _F64P))
        return p, s

    def time_range(self) -> tuple[int, int]:
        """Model times every series covers."""
        lo, hi = -(1 << 62), 1 << 62
        for lens, tt in ((self.meteo_len, self.meteo_time), (self.lai_len, self.lai_time)):
            o = 0
            for n in np.asarray(lens):
                lo, hi = max(lo, int(tt[o])), min(hi, int(tt[o + n - 1]))
                o += int(n)
        return lo, hi

    def save(self, path: str):
        np.savez_compressed(path, cal=np.array(self.cal), meteo_len=self.meteo_len, meteo_time=self.meteo_time,
                            meteo_data=self.meteo_data, lai_len=self.lai_len, lai_time=self.lai_time,
                            lai_data=self.lai_data, **{"p_" + k: v for k, v in self.params.items()})

    @staticmethod
    def load(path: str) -> "Land":
        z = np.load(path)
        params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
        return Land(params, tuple(float(c) for c in z["cal"]), z["meteo_len"], z["meteo_time"], z["meteo_data"],
                    z["lai_len"], z["lai_time"], z["lai_data"])


def _lib():
    lib = capi.load()
    if not getattr(lib, "_land_sigs", False):
        lib.pihm_gpu_land_init.argtypes = [_VP, ctypes.POINTER(LandParamsC), ctypes.POINTER(ForcingSeriesC)]
        lib.pihm_gpu_land_init.restype = ctypes.c_int
        lib.pihm_gpu_land_set_state.argtypes = [_VP, _F64P, _F64P]
        lib.pihm_gpu_land_set_state.restype = ctypes.c_int
        lib.pihm_gpu_land_step.argtypes = [_VP, ctypes.c_int64, ctypes.c_double, _VP]
        lib.pihm_gpu_land_step.restype = ctypes.c_int
        lib.pihm_gpu_land_get.argtypes = [_VP, ctypes.c_int, _F64P]
        lib.pihm_gpu_land_get.restype = ctypes.c_int
        lib._land_sigs = True
    return lib


# Land types the synthetic generator draws from: MODIS classes whose monthly
# roughness length is positive (the reference's ra divides by it), with
# deciduous ones whose monthly LAI drops to 0 in winter.
SYNTH_LC = (1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 13, 14, 16)


def epoch(when: str) -> int:
    """'YYYY-MM-DD hh:mm' (UTC) as seconds since 1970."""
    d = datetime.datetime.strptime(when, "%Y-%m-%d %H:%M").replace(tzinfo=datetime.timezone.utc)
    return int(d.timestamp())


def synthetic_meteo(start: str, hours: int, nstations: int, seed: int):
    """Hourly records for `nstations` stations from `start` over `hours` + 1
    knots: air temperature swinging through the snow/rain thresholds (-3 to
    +1 C) on a daily cycle, rain and snow events, humidity 35-100 %, wind
    0.3-9 m/s, solar radiation on a daytime arc.  Returns (len, time, data)."""
    rng = np.random.default_rng(seed)
    t0 = epoch(start)
    n = hours + 1
    times = t0 + 3600 * np.arange(n, dtype=np.int64)
    lens, tt, dd = [], [], []
    for _ in range(nstations):
        hr = np.arange(n)
        day = np.sin(2 * np.pi * (hr % 24 - 9) / 24.0)
        base = rng.uniform(-4.0, 6.0)
        tmp = 273.15 + base + 6.0 * day + rng.normal(0.0, 0.8, n)
        wet = rng.random(n) < 0.25
        prcp = np.where(wet, rng.exponential(4e-4, n), 0.0)  # kg m-2 s-1
        rh = np.clip(70.0 + 20.0 * (-day) + rng.normal(0.0, 8.0, n) + 15.0 * wet, 35.0, 100.0)
        wind = rng.uniform(0.3, 9.0, n)
        solar = np.maximum(0.0, 650.0 * day + rng.normal(0.0, 40.0, n))
        lw = 280.0 + rng.normal(0.0, 10.0, n)
        pres = 97000.0 + rng.normal(0.0, 300.0, n)
        # rounded to the digits a forcing file carries
        cols = [np.round(prcp, 7)] + [np.round(c, 2) for c in (tmp, rh, wind, solar, lw, pres)]
        d = np.stack(cols, axis=1)
        lens.append(n)
        tt.append(times)
        dd.append(d)
    return np.array(lens, np.int32), np.concatenate(tt), np.concatenate(dd)


def synthetic_land(ws, *, start: str = "2009-01-01 00:00", hours: int = 72, nstations: int = 4, nlai: int = 2,
                   seed: int = 0, per_type: bool = False) -> Land:
    """A seeded land-surface model for watershed `ws`: per-element land types
    from SYNTH_LC, stations and LAI series assigned in spatial blocks, soil
    moistures consistent with the porosity, canopy parameters in the
    ranges of the reference's land-cover table.  per_type: canopy parameters
    (shdfac, albedo, rsmin, rgl) by land type, as a land-cover table holds
    them (what a deck can store), instead of per element."""
    rng = np.random.default_rng(seed + 1)
    ne = ws.nelem
    block = np.arange(ne) * max(nstations, 1) // max(ne, 1)
    lc = rng.choice(np.array(SYNTH_LC, np.int32), ne)
    lai_type = np.where(rng.random(ne) < 0.5, rng.integers(1, nlai + 1, ne), 0).astype(np.int32) if nlai else \
        np.zeros(ne, np.int32)
    por = np.asarray(ws.arrays["porosity"], np.float64)
    smcmin = rng.uniform(0.02, 0.08, ne)
    smcwlt = smcmin + por * rng.uniform(0.05, 0.2, ne)
    smcref = smcwlt + por * rng.uniform(0.2, 0.5, ne)
    albmin = rng.uniform(0.1, 0.2, ne)
    params = {
        "lc_type": lc, "meteo_type": (block + 1).astype(np.int32), "lai_type": lai_type,
        "albedomin": albmin, "albedomax": albmin + rng.uniform(0.0, 0.1, ne),
        # (no bare soil: with shdfac 0 and a positive LAI the canopy capacity is
        # 0 and the reference's canopy evaporation is 0/0, src/is_sm_et.c:128)
        "shdfac": rng.uniform(0.3, 0.95, ne),
        "cmcfactr": np.full(ne, 2e-4), "cfactr": np.full(ne, 0.5),
        "rgl": rng.uniform(30.0, 100.0, ne), "rsmin": rng.uniform(40.0, 300.0, ne), "rsmax": np.full(ne, 5000.0),
        "topt": np.full(ne, 298.0), "smcmin": smcmin, "smcwlt": smcwlt, "smcref": smcref,
        "zlvl_wind": np.full(ne, 10.0),
    }
    if per_type:
        t_shd = np.round(rng.uniform(0.3, 0.95, NLC), 3)
        t_amin = np.round(rng.uniform(0.1, 0.2, NLC), 3)
        t_amax = t_amin + np.round(rng.uniform(0.0, 0.1, NLC), 3)
        t_rgl = np.round(rng.uniform(30.0, 100.0, NLC), 1)
        t_rs = np.round(rng.uniform(40.0, 300.0, NLC), 1)
        for k, v in (("shdfac", t_shd), ("albedomin", t_amin), ("albedomax", t_amax), ("rgl", t_rgl),
                     ("rsmin", t_rs)):
            params[k] = v[lc - 1]
    ml, mt, md = synthetic_meteo(start, hours, nstations, seed)
    ll, lt, ld = [], [], []
    t0 = epoch(start)
    for k in range(nlai):
        n = hours // 24 + 2
        ll.append(n)
        lt.append(t0 + 86400 * np.arange(n, dtype=np.int64))
        ld.append(np.round(rng.uniform(0.2, 5.0, n), 4))
    return Land(params, (1.0, 1.0, 1.0), ml, mt, md, np.array(ll, np.int32),
                np.concatenate(lt) if lt else np.zeros(0, np.int64), np.concatenate(ld) if ld else np.zeros(0))
