"""Python bindings of the CPU checkers (test infrastructure only).

`Oracle`    -- the C restatement of the reference right-hand side
               (oracle/pihm_oracle.c), serial or OpenMP build.
`OracleLand`-- the C restatement of the land-surface step (ApplyForc +
               IntcpSnowEt, oracle/land_oracle.c).
`Reference` -- the reference's own serial/OpenMP code compiled from its
               sources (oracle/ref_harness.c + oracle/Makefile target `ref`);
               present only where the reference sources were available at
               build time.

Only tests/, the smoke check and the benchmark's CPU-baseline leg use this
module; the GPU library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "pihm-cuda_gb300"))

from pihm_gpu.meshdesc import MeshDesc, f64p  # noqa: E402

_F64P = ctypes.POINTER(ctypes.c_double)
_I32P = ctypes.POINTER(ctypes.c_int32)


def build(ref: bool = False) -> None:
    """Compile the restatement (and, when the reference sources exist, the
    reference harness) in place."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libpihm_ref.so"))


def reference_src() -> str | None:
    """The reference checkout: $PIHM_REFERENCE_SRC, else the one the
    reference harness was built from (_ref/REFERENCE_SRC, written by
    `make ref`); None when neither names an existing directory."""
    cand = os.environ.get("PIHM_REFERENCE_SRC")
    if not cand:
        try:
            with open(os.path.join(HERE, "_ref", "REFERENCE_SRC")) as f:
                cand = f.read().strip()
        except OSError:
            cand = None
    return cand if cand and os.path.isdir(cand) else None


def _lib(path: str) -> ctypes.CDLL:
    if not os.path.exists(path):
        build()
    return ctypes.CDLL(path)


class Oracle:
    """The restatement, one watershed per instance."""

    def __init__(self, ws, omp: bool = False, threads: int | None = None):
        name = "liboracle_omp.so" if omp else "liboracle.so"
        lib = _lib(os.path.join(HERE, "_build", name))
        lib.oracle_create.restype = ctypes.c_void_p
        lib.oracle_create.argtypes = [ctypes.POINTER(MeshDesc), ctypes.c_int,
                                      ctypes.c_int, ctypes.c_double]
        for fn in ("oracle_set_forcing",):
            getattr(lib, fn).argtypes = [ctypes.c_void_p, _F64P, _F64P, _F64P]
        lib.oracle_set_bc.argtypes = [ctypes.c_void_p, _F64P, _F64P]
        lib.oracle_set_ws0_surf.argtypes = [ctypes.c_void_p, _F64P]
        lib.oracle_set_river_edge_ovlflow.argtypes = [ctypes.c_void_p, _F64P]
        lib.oracle_rhs.argtypes = [ctypes.c_void_p, ctypes.c_double, _F64P, _F64P]
        lib.oracle_get_fluxes.argtypes = [ctypes.c_void_p] + [_F64P] * 6
        lib.oracle_post_step.argtypes = [ctypes.c_void_p, _F64P]
        lib.oracle_destroy.argtypes = [ctypes.c_void_p]
        lib.oracle_num_threads.restype = ctypes.c_int
        lib.oracle_set_num_threads.argtypes = [ctypes.c_int]
        lib.oracle_set_ulp_perturb.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self.lib = lib
        self.ws = ws
        self.desc = MeshDesc.from_arrays(ws.nelem, ws.nriver, ws.arrays)
        if threads:
            lib.oracle_set_num_threads(int(threads))
        self.h = lib.oracle_create(ctypes.byref(self.desc), ws.surf_mode,
                                   ws.riv_mode, ws.stepsize)

    def close(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    __del__ = close

    @property
    def threads(self) -> int:
        return self.lib.oracle_num_threads()

    def set_ulp_perturb(self, s: int):
        """+1 / -1: every pow() and log() result of this model's evaluations
        moves by one unit in the last place in that direction; 0: the
        reference's arithmetic exactly (the default)."""
        self.lib.oracle_set_ulp_perturb(self.h, int(s))

    def set_forcing(self, pcpdrp=None, edir=None, ett=None):
        self.lib.oracle_set_forcing(self.h, f64p(_c(pcpdrp)), f64p(_c(edir)),
                                    f64p(_c(ett)))

    def set_bc(self, elem_bc=None, river_bc=None):
        self.lib.oracle_set_bc(self.h, f64p(_c(elem_bc)), f64p(_c(river_bc)))

    def set_ws0_surf(self, ws0):
        self.lib.oracle_set_ws0_surf(self.h, f64p(_c(ws0)))

    def set_river_edge_ovlflow(self, ovl):
        self.lib.oracle_set_river_edge_ovlflow(self.h, f64p(_c(ovl)))

    def rhs(self, y, t: float = 0.0):
        y = _c(y)
        out = np.zeros_like(y)
        rc = self.lib.oracle_rhs(self.h, t, f64p(y), f64p(out))
        return out, rc

    def post_step(self, y):
        self.lib.oracle_post_step(self.h, f64p(_c(y)))

    def set_noah(self, noah: dict):
        """Flux-PIHM (_NOAH_) right-hand side with Noah's per-step inputs
        (et [nelem, nlayers], nwtbl, nroot, sh2o0, smcmin, smcmax, fcr)."""
        _set_noah(self.lib.oracle_set_noah, noah, self.h)

    def fluxes(self):
        ne, nr = self.ws.nelem, self.ws.nriver
        out = dict(ovlflow=np.zeros(3 * ne), subsurf=np.zeros(3 * ne),
                   infil=np.zeros(ne), rechg=np.zeros(ne),
                   et_split=np.zeros(5 * ne), rivflow=np.zeros(11 * nr))
        self.lib.oracle_get_fluxes(self.h, *(f64p(out[k]) for k in (
            "ovlflow", "subsurf", "infil", "rechg", "et_split", "rivflow")))
        return out


class Reference:
    """The reference's own code (compiled from its sources).  The reference
    keeps its model in globals, so one instance at a time."""

    def __init__(self, omp: bool = False, noah: bool = False):
        name = "libpihm_ref_noah.so" if noah else ("libpihm_ref_omp.so" if omp else "libpihm_ref.so")
        path = os.path.join(HERE, "_ref", name)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        lib.ref_build.argtypes = [ctypes.POINTER(MeshDesc), ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int]
        lib.ref_sizes.argtypes = [ctypes.POINTER(ctypes.c_int)] * 5
        lib.ref_export_double.argtypes = [ctypes.c_char_p, _F64P]
        lib.ref_export_int.argtypes = [ctypes.c_char_p, _I32P]
        lib.ref_set_forcing.argtypes = [_F64P, _F64P, _F64P]
        lib.ref_set_bc.argtypes = [_F64P, _F64P]
        lib.ref_set_ws0_surf.argtypes = [_F64P]
        lib.ref_set_river_edge_ovlflow.argtypes = [_F64P]
        lib.ref_ode.argtypes = [ctypes.c_double, _F64P, _F64P]
        lib.ref_get_fluxes.argtypes = [_F64P] * 6
        lib.ref_num_threads.restype = ctypes.c_int
        lib.ref_set_num_threads.argtypes = [ctypes.c_int]
        if noah:  # the Flux-PIHM build has the right-hand side only
            lib.ref_get_gwet.argtypes = [_F64P]
        else:
            lib.ref_load_example.argtypes = [ctypes.c_char_p, ctypes.c_char_p,
                                             _F64P, ctypes.c_int]
            lib.ref_apply_forcing.argtypes = [ctypes.c_int]
            lib.ref_model_times.argtypes = [ctypes.POINTER(ctypes.c_int)] * 4
            lib.ref_land_step.argtypes = [ctypes.c_int, ctypes.c_double]
            lib.ref_land_set_state.argtypes = [_F64P] * 4
            lib.ref_monthly.argtypes = [ctypes.c_int, ctypes.c_int, _F64P]
            lib.ref_monthly.restype = None
        self.lib = lib
        self.ne = self.nr = 0

    def build(self, ws):
        self.desc = MeshDesc.from_arrays(ws.nelem, ws.nriver, ws.arrays)
        self.lib.ref_build(ctypes.byref(self.desc), ws.surf_mode, ws.riv_mode,
                           int(ws.stepsize))
        self.ne, self.nr = ws.nelem, ws.nriver

    def load_deck(self, workdir: str, project: str):
        """Read an input deck with the reference's readers; returns y0."""
        y0 = np.zeros(8 * 1024 * 1024)
        rc = self.lib.ref_load_example(workdir.encode(), project.encode(),
                                       f64p(y0), y0.shape[0])
        assert rc == 0
        vals = [ctypes.c_int() for _ in range(5)]
        self.lib.ref_sizes(*[ctypes.byref(v) for v in vals])
        self.ne, self.nr = vals[0].value, vals[1].value
        self.stepsize, self.surf_mode, self.riv_mode = (vals[2].value,
                                                       vals[3].value,
                                                       vals[4].value)
        return y0[:3 * self.ne + 2 * self.nr].copy()

    def export(self, name: str, n: int, kind=np.float64):
        out = np.zeros(n, kind)
        if kind == np.float64:
            rc = self.lib.ref_export_double(name.encode(), f64p(out))
        else:
            rc = self.lib.ref_export_int(name.encode(),
                                         out.ctypes.data_as(_I32P))
        assert rc == 0, name
        return out

    def set_forcing(self, pcpdrp=None, edir=None, ett=None):
        self.lib.ref_set_forcing(f64p(_c(pcpdrp)), f64p(_c(edir)), f64p(_c(ett)))

    def set_bc(self, elem_bc=None, river_bc=None):
        self.lib.ref_set_bc(f64p(_c(elem_bc)), f64p(_c(river_bc)))

    def set_ws0_surf(self, ws0):
        self.lib.ref_set_ws0_surf(f64p(_c(ws0)))

    def set_river_edge_ovlflow(self, ovl):
        self.lib.ref_set_river_edge_ovlflow(f64p(_c(ovl)))

    def rhs(self, y, t: float = 0.0):
        y = _c(y)
        out = np.zeros_like(y)
        rc = self.lib.ref_ode(t, f64p(y), f64p(out))
        return out, rc

    def set_noah(self, noah: dict):
        _set_noah(self.lib.ref_set_noah, noah)

    # the Noah land-surface model (Flux-PIHM build): Noah(), Summary(),
    # NoahHydrol() of the reference on the model built by build()
    def noah_load(self, params: dict, state: dict, y0):
        from pihm_gpu import noah as N
        lib = self.lib
        lib.ref_noah_load.argtypes = [ctypes.POINTER(N.NoahParams), ctypes.POINTER(N.NoahState), _F64P]
        lib.ref_noah_forcing.argtypes = [ctypes.POINTER(N.NoahForcing)]
        lib.ref_noah_step.argtypes = [ctypes.c_double]
        lib.ref_noah_post.argtypes = [_F64P, ctypes.c_double]
        lib.ref_noah_get.argtypes = [ctypes.c_int, _F64P]
        ps, kp = N.params_struct(params)
        ss, ks = N.state_struct(state)
        assert lib.ref_noah_load(ctypes.byref(ps), ctypes.byref(ss), f64p(_c(y0))) == 0

    def noah_forcing(self, forcing: dict):
        from pihm_gpu import noah as N
        fs, kf = N.forcing_struct(forcing)
        assert self.lib.ref_noah_forcing(ctypes.byref(fs)) == 0

    def noah_step(self, dt: float):
        assert self.lib.ref_noah_step(float(dt)) == 0

    def noah_post(self, y, dt: float):
        assert self.lib.ref_noah_post(f64p(_c(y)), float(dt)) == 0

    def noah_get(self, name: str) -> np.ndarray:
        from pihm_gpu import noah as N
        out = np.zeros(N.field_shape(name, self.ne))
        assert self.lib.ref_noah_get(N.field_id(name), f64p(out.reshape(-1))) == 0
        return out

    # land-surface step of a loaded deck (ApplyForc + IntcpSnowEt)
    def land_set_state(self, unsat=None, gw=None, cmc=None, sneqv=None):
        keep = [_c(a) for a in (unsat, gw, cmc, sneqv)]
        assert self.lib.ref_land_set_state(*(f64p(a) for a in keep)) == 0

    def land_step(self, t: int, stepsize: float):
        assert self.lib.ref_land_step(int(t), float(stepsize)) == 0

    def land_fields(self) -> dict:
        return {k: self.export(k, self.ne) for k in ("prcp", "pcpdrp", "edir", "ett", "ec", "drip", "cmc", "sneqv")}

    def monthly(self, t: int, lc: int) -> np.ndarray:
        out = np.zeros(3)
        self.lib.ref_monthly(int(t), int(lc), f64p(out))
        return out

    def fluxes(self):
        ne, nr = self.ne, self.nr
        out = dict(ovlflow=np.zeros(3 * ne), subsurf=np.zeros(3 * ne),
                   infil=np.zeros(ne), rechg=np.zeros(ne),
                   et_split=np.zeros(5 * ne), rivflow=np.zeros(11 * nr))
        self.lib.ref_get_fluxes(*(f64p(out[k]) for k in (
            "ovlflow", "subsurf", "infil", "rechg", "et_split", "rivflow")))
        return out


class OracleLand:
    """The land-surface restatement (oracle/land_oracle.c) for a land.Land
    and the watershed's zmax, depth, porosity, rzd."""

    FIELDS = ("prcp", "pcpdrp", "edir", "ett", "ec", "drip", "cmc", "sneqv")

    def __init__(self, land, ws, omp: bool = False):
        from pihm_gpu import land as L
        name = "liboracle_omp.so" if omp else "liboracle.so"
        lib = _lib(os.path.join(HERE, "_build", name))
        lib.oracle_land_create.restype = ctypes.c_void_p
        lib.oracle_land_create.argtypes = [ctypes.POINTER(L.LandParamsC), ctypes.POINTER(L.ForcingSeriesC)] + \
            [_F64P] * 4
        lib.oracle_land_destroy.argtypes = [ctypes.c_void_p]
        lib.oracle_land_set_state.argtypes = [ctypes.c_void_p, _F64P, _F64P]
        lib.oracle_land_step.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_double, _F64P, _F64P]
        lib.oracle_land_step.restype = ctypes.c_int
        lib.oracle_land_get.argtypes = [ctypes.c_void_p, ctypes.c_int, _F64P]
        lib.oracle_land_monthly.argtypes = [ctypes.c_longlong, ctypes.c_int, _F64P]
        self.lib, self.ne = lib, land.nelem
        p, s = land.structs()
        mesh = [_c(ws.arrays[k]) for k in ("zmax", "depth", "porosity", "rzd")]
        self.h = lib.oracle_land_create(ctypes.byref(p), ctypes.byref(s), *(f64p(a) for a in mesh))

    def close(self):
        if getattr(self, "h", None):
            self.lib.oracle_land_destroy(self.h)
            self.h = None

    __del__ = close

    def set_state(self, cmc=None, sneqv=None):
        self.lib.oracle_land_set_state(self.h, f64p(_c(cmc)), f64p(_c(sneqv)))

    def step(self, t: int, stepsize: float, unsat, gw) -> int:
        return self.lib.oracle_land_step(self.h, int(t), float(stepsize), f64p(_c(unsat)), f64p(_c(gw)))

    def get(self, field: str) -> np.ndarray:
        out = np.zeros(self.ne)
        self.lib.oracle_land_get(self.h, self.FIELDS.index(field), f64p(out))
        return out

    def fields(self) -> dict:
        return {k: self.get(k) for k in self.FIELDS}

    def monthly(self, t: int, lc: int) -> np.ndarray:
        out = np.zeros(3)
        self.lib.oracle_land_monthly(int(t), int(lc), f64p(out))
        return out


def _set_noah(fn, noah, *head):
    """Call oracle_set_noah / ref_set_noah with a dict of Noah inputs."""
    et = np.ascontiguousarray(noah["et"], np.float64)
    nl = et.shape[1] if et.ndim == 2 else 0
    i32 = lambda a: np.ascontiguousarray(a, np.int32)
    keep = [et, i32(noah["nwtbl"]), i32(noah["nroot"])] + [_c(noah[k]) for k in ("sh2o0", "smcmin", "smcmax", "fcr")]
    fn.argtypes = ([ctypes.c_void_p] if head else []) + [_F64P, ctypes.c_int, _I32P, _I32P] + [_F64P] * 4
    fn.restype = ctypes.c_int
    rc = fn(*head, f64p(keep[0]), nl, keep[1].ctypes.data_as(_I32P), keep[2].ctypes.data_as(_I32P),
            *(f64p(a) for a in keep[3:]))
    assert rc == 0


def _c(a):
    if a is None:
        return None
    return np.ascontiguousarray(a, np.float64)
