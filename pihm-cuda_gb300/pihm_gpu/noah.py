"""The Noah land-surface model of Flux-PIHM (include/pihm_noah.h): ctypes
structs, the binding on a GpuRhs context, and a seeded generator of Noah's
parameters, initial state and forcing for generated watersheds.

Generated inputs (the Flux-PIHM configuration of the benchmark: 4 soil
layers per element, hourly forcing):

  layers     thicknesses 0.1, 0.3, 0.6 m and the rest of the soil column
             (the element's depth, 2..10 m); root layers from the element's
             root depth (FindLayer), root distribution by thickness
             (RootDist, src/noah/lsm_func.c:187-205)
  soil       residual moisture U(0.02, 0.08) with saturation = residual +
             porosity; wilting point and reference moisture at U(0.05, 0.2)
             and U(0.5, 0.8) of the porosity above the residual; quartz
             U(0.1, 0.9); the mesh's van Genuchten alpha, beta and Ksatv
  land cover vegetation fraction U(0.3, 0.95), LAI range, emissivity,
             albedo and roughness ranges, canopy resistance parameters drawn
             per element from the ranges of the reference's vegetation table;
             3 % of the elements urban
  universal  the .lsm values of the bundled example (SBETA -2, FXEXP 2,
             CSOIL 2e6, SALP 2.6, FRZK 0.15, ZBOT -8 m, TBOT 282.15 K,
             CZIL 0.1, LVCOEF 0.5), forcing height 3 m, wind height 10 m,
             maximum snow albedo 0.75
  forcing    air temperature a 270..305 K diurnal sinusoid + N(0, 2 K),
             relative humidity U(30, 95) %, wind lognormal with mean 3 m/s,
             shortwave a clear-sky cosine times a U(0.3, 1) cloud factor,
             longwave from the air temperature, pressure from the elevation,
             hourly rain Bernoulli(0.1) x gamma(0.7, 3 mm/h), LAI U(0.5, 6)
"""
from __future__ import annotations

import ctypes

import numpy as np

L = 11  # PIHM_NOAH_MAXLYR
_F64P = ctypes.POINTER(ctypes.c_double)
_I32P = ctypes.POINTER(ctypes.c_int32)
BADVAL = -999.0

PARAM_DOUBLES = ("smcmax", "smcmin", "smcref", "smcwlt", "smcdry", "quartz", "csoil", "alpha", "beta", "ksatv",
                 "porosity", "depth", "area", "shdfac", "cmcfactr", "laimax", "laimin", "emissmax", "emissmin",
                 "albedomax", "albedomin", "z0max", "z0min", "snup", "cfactr", "rgl", "rsmin", "rsmax", "topt", "hs",
                 "sbeta", "salp", "frzx", "fxexp", "czil", "lvcoef", "zbot", "tbot", "zlvl", "zlvl_wind", "snoalb")
STATE_FIELDS = ("smc", "sh2o", "stc", "t1", "cmc", "sneqv", "snowh", "sndens", "ch", "cm", "snotime1",
                "albedo", "emissi", "q1", "ribb", "fcr")
FORCING_FIELDS = ("prcp", "sfctmp", "rh", "sfcspd", "soldn", "longwave", "sfcprs", "lai")

# readable fields (PIHM_NOAH_* of include/pihm_noah.h); per-layer ones first
LAYER_FIELDS = {"smc": 0, "sh2o": 1, "stc": 2, "et": 3, "runoff2_lyr": 4, "smflxv": 5}
SCALAR_FIELDS = {k: 16 + n for n, k in enumerate((
    "t1", "cmc", "sneqv", "snowh", "sndens", "ch", "cm", "albedo", "emissi", "q1", "fcr", "edir", "ec", "ett",
    "esnow", "etp", "drip", "pcpdrp", "snomlt", "ssoil", "sheat", "runoff2", "runoff3", "infil", "nwtbl",
    "snotime1", "sncovr", "beta", "eta", "soilm"))}


class NoahParams(ctypes.Structure):
    _fields_ = ([("nelem", ctypes.c_int32), ("nsoil", _I32P), ("sldpth", _F64P), ("nroot", _I32P),
                 ("rtdis", _F64P), ("isurban", _I32P)] + [(k, _F64P) for k in PARAM_DOUBLES])


class NoahState(ctypes.Structure):
    _fields_ = [(k, _F64P) for k in STATE_FIELDS]


class NoahForcing(ctypes.Structure):
    _fields_ = [(k, _F64P) for k in FORCING_FIELDS]


def _f64(a):
    return np.ascontiguousarray(a, np.float64)


def _i32(a):
    return np.ascontiguousarray(a, np.int32)


def params_struct(p: dict):
    """(struct, keep-alive list) for a parameter dict."""
    keep = []

    def ptr(a, kind):
        a = _f64(a) if kind == "d" else _i32(a)
        keep.append(a)
        return a.ctypes.data_as(_F64P if kind == "d" else _I32P)
    s = NoahParams()
    s.nelem = int(len(p["nsoil"]))
    s.nsoil = ptr(p["nsoil"], "i")
    s.sldpth = ptr(p["sldpth"], "d")
    s.nroot = ptr(p["nroot"], "i")
    s.rtdis = ptr(p["rtdis"], "d")
    s.isurban = ptr(p["isurban"], "i")
    for k in PARAM_DOUBLES:
        setattr(s, k, ptr(p[k], "d"))
    return s, keep


def state_struct(st: dict):
    keep = []
    s = NoahState()
    for k in STATE_FIELDS:
        if st.get(k) is not None:
            a = _f64(st[k])
            keep.append(a)
            setattr(s, k, a.ctypes.data_as(_F64P))
    return s, keep


def forcing_struct(f: dict):
    keep = []
    s = NoahForcing()
    for k in FORCING_FIELDS:
        a = _f64(f[k])
        keep.append(a)
        setattr(s, k, a.ctypes.data_as(_F64P))
    return s, keep


def find_layer(sldpth, nsoil, depth):
    """FindLayer, src/noah/lsm_func.c:57-84."""
    if depth <= 0.0:
        return 0
    dsum, j, ind = 0.0, 0, 0
    while dsum < depth:
        if sldpth[j] < 0.0:
            break
        dsum += sldpth[j]
        ind = j
        j += 1
    return min(ind + 1, nsoil)


def synthetic_noah(ws, seed: int = 0, nlayers: int = 4, urban_frac: float = 0.03):
    """Noah parameters and an initial state for watershed `ws` (see the
    module docstring); returns (params, state), dicts of numpy arrays in
    reference order."""
    assert nlayers == 4
    rng = np.random.default_rng(7000 + seed)
    a = ws.arrays
    ne = ws.nelem
    depth = np.asarray(a["depth"], np.float64)
    por = np.asarray(a["porosity"], np.float64)
    sldpth = np.zeros((ne, L))
    sldpth[:, 0], sldpth[:, 1], sldpth[:, 2] = 0.1, 0.3, 0.6
    sldpth[:, 3] = depth - 1.0
    nsoil = np.full(ne, nlayers, np.int32)
    rzd = np.asarray(a["rzd"], np.float64)
    nroot = np.array([find_layer(sldpth[i], nlayers, rzd[i]) for i in range(ne)], np.int32)
    nroot = np.maximum(nroot, 1)
    rtdis = np.zeros((ne, L))
    for i in range(ne):
        z = -np.cumsum(sldpth[i, :nlayers])
        rtdis[i, :nroot[i]] = -sldpth[i, :nroot[i]] / z[nroot[i] - 1]
    smcmin = rng.uniform(0.02, 0.08, ne)
    smcmax = smcmin + por
    smcwlt = smcmin + rng.uniform(0.05, 0.2, ne) * por
    smcref = smcmin + rng.uniform(0.5, 0.8, ne) * por
    laimin = rng.uniform(0.5, 1.5, ne)
    frzk = 0.15
    p = dict(
        nsoil=nsoil, sldpth=sldpth, nroot=nroot, rtdis=rtdis,
        isurban=(rng.random(ne) < urban_frac).astype(np.int32),
        smcmax=smcmax, smcmin=smcmin, smcref=smcref, smcwlt=smcwlt, smcdry=smcwlt.copy(),
        quartz=rng.uniform(0.1, 0.9, ne), csoil=np.full(ne, 2.0e6),
        alpha=np.asarray(a["alpha"], np.float64), beta=np.asarray(a["beta"], np.float64),
        ksatv=np.asarray(a["ksatv"], np.float64), porosity=por, depth=depth,
        area=np.asarray(a["area"], np.float64),
        shdfac=rng.uniform(0.3, 0.95, ne), cmcfactr=np.full(ne, 0.0002),
        laimax=laimin + rng.uniform(2.0, 4.5, ne), laimin=laimin,
        emissmax=rng.uniform(0.95, 0.98, ne), emissmin=rng.uniform(0.90, 0.95, ne),
        albedomax=rng.uniform(0.19, 0.25, ne), albedomin=rng.uniform(0.10, 0.18, ne),
        z0max=rng.uniform(0.1, 1.0, ne), z0min=rng.uniform(0.02, 0.09, ne),
        snup=rng.uniform(0.02, 0.08, ne), cfactr=np.full(ne, 0.5),
        rgl=rng.uniform(30.0, 100.0, ne), rsmin=rng.uniform(40.0, 300.0, ne), rsmax=np.full(ne, 5000.0),
        topt=np.full(ne, 298.0), hs=rng.uniform(36.0, 55.0, ne),
        sbeta=np.full(ne, -2.0), salp=np.full(ne, 2.6),
        frzx=frzk * (smcmax / smcref) * (0.412 / 0.468),  # InitLsm, src/noah/lsm_init.c:36-40
        fxexp=np.full(ne, 2.0), czil=np.full(ne, 0.1), lvcoef=np.full(ne, 0.5),
        zbot=np.full(ne, -8.0), tbot=np.full(ne, 282.15), zlvl=np.full(ne, 3.0),
        zlvl_wind=np.full(ne, 10.0), snoalb=np.full(ne, 0.75))
    # initial state: skin and soil temperatures from the air temperature as
    # the reference's relaxed start sets them (src/initialize.c:160-175)
    sfctmp = rng.uniform(262.0, 290.0, ne)
    stc = np.zeros((ne, L))
    grad = (sfctmp - p["tbot"]) / p["zbot"]
    stc[:, 0] = sfctmp + grad * sldpth[:, 0] * 0.5
    for j in range(1, nlayers):
        stc[:, j] = stc[:, j - 1] + grad * (sldpth[:, j - 1] + sldpth[:, j]) * 0.5
    smc = np.zeros((ne, L))
    sh2o = np.zeros((ne, L))
    lo = (smcmin + 0.02)[:, None]
    smc[:, :nlayers] = lo + (smcmax[:, None] - lo) * rng.uniform(0.05, 1.0, (ne, nlayers))
    frozen = stc[:, :nlayers] < 273.15
    sh2o[:, :nlayers] = np.where(frozen, smc[:, :nlayers] * rng.uniform(0.4, 1.0, (ne, nlayers)),
                                 smc[:, :nlayers])
    snow = rng.random(ne) < 0.3
    sneqv = np.where(snow, rng.uniform(0.005, 0.08, ne), 0.0)
    sndens = np.where(snow, rng.uniform(0.1, 0.35, ne), 0.0)
    st = dict(smc=smc, sh2o=sh2o, stc=stc, t1=sfctmp,
              cmc=rng.uniform(0.0, 0.5, ne) * p["shdfac"] * p["cmcfactr"] * laimin,
              sneqv=sneqv, snowh=np.where(snow, sneqv / np.where(snow, sndens, 1.0), 0.0), sndens=sndens,
              ch=np.full(ne, 1.0e-4), cm=np.full(ne, 1.0e-4),
              snotime1=np.where(snow, rng.uniform(0.0, 2.0e5, ne), 0.0),
              albedo=np.full(ne, 0.18), emissi=np.full(ne, 0.96), q1=np.full(ne, BADVAL),
              ribb=np.zeros(ne), fcr=np.ones(ne))
    return p, st


def forcing(ws, hour: int, seed: int = 0, diverse: bool = False) -> dict:
    """Per-element forcing of the land-surface step starting at `hour` (see
    the module docstring).  diverse=True draws every element's air
    temperature over 255..300 K and rain on a third of them regardless of
    the hour, so that one step takes snowfall, melt, freezing rain and frozen
    soil together (the parity fixtures)."""
    rng = np.random.default_rng((seed * 100003 + hour) & 0x7FFFFFFF)
    ne = ws.nelem
    zmax = np.asarray(ws.arrays["zmax"], np.float64)
    phase = 2.0 * np.pi * ((hour % 24) - 9.0) / 24.0
    if diverse:
        sfctmp = rng.uniform(255.0, 300.0, ne)
        wet = rng.random(ne) < 0.35
    else:
        sfctmp = 287.5 + 17.5 * np.sin(phase) + rng.normal(0.0, 2.0, ne)
        wet = rng.random(ne) < 0.1
    prcp = np.where(wet, rng.gamma(0.7, 3.0, ne), 0.0) / 3.6e6
    cosz = max(0.0, np.sin(2.0 * np.pi * ((hour % 24) - 6.0) / 24.0))
    if diverse:
        cosz = rng.uniform(0.0, 1.0, ne) * (rng.random(ne) < 0.6)
    soldn = 1000.0 * cosz * rng.uniform(0.3, 1.0, ne)
    sigma = 0.5
    sfcspd = rng.lognormal(np.log(3.0) - 0.5 * sigma * sigma, sigma, ne)
    longwave = rng.uniform(0.7, 0.9, ne) * 5.67e-8 * sfctmp ** 4
    sfcprs = 101325.0 * ((293.0 - 0.0065 * zmax) / 293.0) ** 5.26
    return dict(prcp=prcp, sfctmp=sfctmp, rh=rng.uniform(30.0, 95.0, ne), sfcspd=sfcspd, soldn=soldn,
                longwave=longwave, sfcprs=sfcprs, lai=rng.uniform(0.5, 6.0, ne))


def bind(lib):
    """Signatures of the Noah entry points on the library."""
    _VP = ctypes.c_void_p
    lib.pihm_gpu_noah_init.argtypes = [_VP, ctypes.POINTER(NoahParams), ctypes.POINTER(NoahState)]
    lib.pihm_gpu_noah_set_state.argtypes = [_VP, ctypes.POINTER(NoahState)]
    lib.pihm_gpu_noah_set_forcing.argtypes = [_VP, ctypes.POINTER(NoahForcing)]
    lib.pihm_gpu_noah_step.argtypes = [_VP, ctypes.c_double]
    lib.pihm_gpu_noah_begin.argtypes = [_VP, _VP]
    lib.pihm_gpu_noah_post_step.argtypes = [_VP, _VP, ctypes.c_double]
    lib.pihm_gpu_noah_get.argtypes = [_VP, ctypes.c_int, _F64P]
    for n in ("init", "set_state", "set_forcing", "step", "begin", "post_step", "get"):
        getattr(lib, "pihm_gpu_noah_" + n).restype = ctypes.c_int
    return lib


def field_shape(name: str, ne: int):
    return (ne, L) if name in LAYER_FIELDS else (ne,)


def field_id(name: str) -> int:
    return LAYER_FIELDS[name] if name in LAYER_FIELDS else SCALAR_FIELDS[name]
