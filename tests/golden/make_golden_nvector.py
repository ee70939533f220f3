"""Golden vectors of the serial N_Vector operations, produced by the
reference's own SUNDIALS 2.7 nvector_serial.c (compiled into
oracle/_ref/libpihm_ref.so by oracle/Makefile target `ref`).

    python tests/golden/make_golden_nvector.py

writes tests/golden/nvector_calls.npz: the operands and, for every
coefficient case of N_VLinearSum (with z aliasing nothing, x or y) and every
other operation, the reference's result.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

COEFS = [(1.0, 1.0), (1.0, -1.0), (-1.0, 1.0), (1.0, 0.37), (0.37, 1.0), (-1.0, 2.5),
         (2.5, -1.0), (0.7, 0.7), (0.7, -0.7), (0.3, -2.9)]


class SerialNV:
    """The reference's serial N_Vector functions over numpy buffers."""

    def __init__(self, lib):
        self.lib = lib
        P = ctypes.c_void_p
        D = ctypes.c_double
        lib.N_VMake_Serial.restype = P
        lib.N_VMake_Serial.argtypes = [ctypes.c_long, P]
        lib.N_VDestroy_Serial.argtypes = [P]
        for name, args, res in [
            ("N_VLinearSum_Serial", [D, P, D, P, P], None), ("N_VConst_Serial", [D, P], None),
            ("N_VProd_Serial", [P, P, P], None), ("N_VDiv_Serial", [P, P, P], None),
            ("N_VScale_Serial", [D, P, P], None), ("N_VAbs_Serial", [P, P], None),
            ("N_VInv_Serial", [P, P], None), ("N_VAddConst_Serial", [P, D, P], None),
            ("N_VDotProd_Serial", [P, P], D), ("N_VMaxNorm_Serial", [P], D),
            ("N_VWrmsNorm_Serial", [P, P], D), ("N_VWrmsNormMask_Serial", [P, P, P], D),
            ("N_VMin_Serial", [P], D), ("N_VWL2Norm_Serial", [P, P], D), ("N_VL1Norm_Serial", [P], D),
            ("N_VCompare_Serial", [D, P, P], None), ("N_VInvTest_Serial", [P, P], ctypes.c_int),
            ("N_VConstrMask_Serial", [P, P, P], ctypes.c_int), ("N_VMinQuotient_Serial", [P, P], D)]:
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res

    def wrap(self, a):
        return self.lib.N_VMake_Serial(a.size, a.ctypes.data)


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libpihm_ref.so"))
    S = SerialNV(lib)
    rng = np.random.default_rng(42)
    n = 1000
    x = rng.normal(size=n)
    x[::7] = 0.0
    y = rng.uniform(0.5, 2.0, n)
    w = rng.uniform(1e3, 1e5, n)
    idm = rng.choice([0.0, 1.0], size=n)
    c = rng.choice([0.0, 1.0, -1.0, 2.0, -2.0], size=n)
    den = rng.normal(size=n)
    den[::3] = 0.0
    out = dict(x=x, y=y, w=w, idm=idm, c=c, den=den, coefs=np.array(COEFS))
    for k, (a, b) in enumerate(COEFS):
        for alias in ("none", "x", "y"):
            xx, yy = x.copy(), y.copy()
            zz = xx if alias == "x" else (yy if alias == "y" else np.zeros(n))
            vx, vy = S.wrap(xx), S.wrap(yy)
            vz = vx if alias == "x" else (vy if alias == "y" else S.wrap(zz))
            lib.N_VLinearSum_Serial(a, vx, b, vy, vz)
            out[f"lin{k}_{alias}"] = zz.copy()
    z = np.zeros(n)
    vx, vy, vz, vw, vi, vc, vd = (S.wrap(a) for a in (x, y, z, w, idm, c, den))
    def run(name, fn):
        z[:] = 0.0
        fn()
        out[name] = z.copy()
    run("const", lambda: lib.N_VConst_Serial(3.25, vz))
    run("prod", lambda: lib.N_VProd_Serial(vx, vy, vz))
    run("div", lambda: lib.N_VDiv_Serial(vx, vy, vz))
    run("scale", lambda: lib.N_VScale_Serial(0.3, vx, vz))
    run("neg", lambda: lib.N_VScale_Serial(-1.0, vx, vz))
    run("abs", lambda: lib.N_VAbs_Serial(vx, vz))
    run("inv", lambda: lib.N_VInv_Serial(vy, vz))
    run("addconst", lambda: lib.N_VAddConst_Serial(vx, -0.5, vz))
    run("compare", lambda: lib.N_VCompare_Serial(0.8, vx, vz))
    z[:] = 9.0
    out["invtest_ok"] = np.array(lib.N_VInvTest_Serial(vx, vz))
    out["invtest"] = z.copy()
    z[:] = 0.0
    out["constr_ok"] = np.array(lib.N_VConstrMask_Serial(vc, vx, vz))
    out["constr"] = z.copy()
    out["dot"] = np.array(lib.N_VDotProd_Serial(vx, vw))
    out["maxnorm"] = np.array(lib.N_VMaxNorm_Serial(vx))
    out["wrms"] = np.array(lib.N_VWrmsNorm_Serial(vx, vw))
    out["wrmsmask"] = np.array(lib.N_VWrmsNormMask_Serial(vx, vw, vi))
    out["min"] = np.array(lib.N_VMin_Serial(vx))
    out["wl2"] = np.array(lib.N_VWL2Norm_Serial(vx, vw))
    out["l1"] = np.array(lib.N_VL1Norm_Serial(vx))
    out["minq"] = np.array(lib.N_VMinQuotient_Serial(vx, vd))
    np.savez_compressed(os.path.join(HERE, "nvector_calls.npz"), **out)
    print("wrote", os.path.join(HERE, "nvector_calls.npz"))


if __name__ == "__main__":
    main()
