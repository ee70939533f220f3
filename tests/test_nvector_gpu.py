"""Device N_Vector operations against the serial N_Vector's arithmetic
(oracle/nvector_oracle.py): element-wise results bit for bit, reductions
within rounding of a different summation order."""
import ctypes

import numpy as np
import pytest

import nvector_oracle as NO
import pihm_gpu.nvector as NV

pytestmark = pytest.mark.gpu

SIZES = [1, 7, 1000, 65_537, 3_060_000]


@pytest.fixture(scope="module")
def nv():
    import torch
    from pihm_gpu import nvector
    return nvector.load(), torch


def _vec(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _mk(lib, t):
    return lib.N_VMake_PihmGpu(t.numel(), ctypes.c_void_p(t.data_ptr()), None)


COEFS = [(1.0, 1.0), (1.0, -1.0), (-1.0, 1.0), (1.0, 0.37), (0.37, 1.0), (-1.0, 2.5),
         (2.5, -1.0), (0.7, 0.7), (0.7, -0.7), (0.3, -2.9)]


@pytest.mark.parametrize("n", SIZES)
def test_linear_sum_cases(nv, n):
    lib, torch = nv
    rng = np.random.default_rng(n)
    x = rng.normal(size=n)
    y = rng.normal(size=n)
    for a, b in COEFS:
        for alias in (None, "x", "y"):
            tx, ty = _vec(torch, x), _vec(torch, y)
            tz = tx if alias == "x" else (ty if alias == "y" else torch.empty_like(tx))
            vx, vy, vz = _mk(lib, tx), _mk(lib, ty), _mk(lib, tz)
            lib.N_VLinearSum_PihmGpu(a, vx, b, vy, vz)
            torch.cuda.synchronize()
            want = NO.linear_sum(a, x, b, y, alias)
            assert np.array_equal(tz.cpu().numpy(), want), (a, b, alias)
            for v in (vx, vy, vz):
                if v != vz or alias is None:
                    lib.N_VDestroy_PihmGpu(v)


@pytest.mark.parametrize("n", SIZES)
def test_elementwise_ops(nv, n):
    lib, torch = nv
    rng = np.random.default_rng(100 + n)
    x = rng.normal(size=n)
    x[::5] = 0.0
    y = rng.uniform(0.5, 2.0, n)
    tx, ty, tz = _vec(torch, x), _vec(torch, y), _vec(torch, np.zeros(n))
    vx, vy, vz = _mk(lib, tx), _mk(lib, ty), _mk(lib, tz)
    checks = [
        (lambda: lib.N_VConst_PihmGpu(3.25, vz), np.full(n, 3.25)),
        (lambda: lib.N_VProd_PihmGpu(vx, vy, vz), x * y),
        (lambda: lib.N_VDiv_PihmGpu(vx, vy, vz), x / y),
        (lambda: lib.N_VScale_PihmGpu(0.3, vx, vz), NO.scale(0.3, x)),
        (lambda: lib.N_VScale_PihmGpu(-1.0, vx, vz), NO.scale(-1.0, x)),
        (lambda: lib.N_VAbs_PihmGpu(vx, vz), np.abs(x)),
        (lambda: lib.N_VInv_PihmGpu(vy, vz), 1.0 / y),
        (lambda: lib.N_VAddConst_PihmGpu(vx, -0.5, vz), x + -0.5),
        (lambda: lib.N_VCompare_PihmGpu(0.8, vx, vz), NO.compare(0.8, x)),
    ]
    for fn, want in checks:
        fn()
        torch.cuda.synchronize()
        assert np.array_equal(tz.cpu().numpy(), want)
    # InvTest (z untouched where x == 0)
    tz.copy_(_vec(torch, np.full(n, 9.0)))
    ok = lib.N_VInvTest_PihmGpu(vx, vz)
    want_ok, want_z = NO.inv_test(x, np.full(n, 9.0))
    assert bool(ok) == want_ok and np.array_equal(tz.cpu().numpy(), want_z)
    # ConstrMask
    c = rng.choice([0.0, 1.0, -1.0, 2.0, -2.0], size=n)
    tc = _vec(torch, c)
    vc = _mk(lib, tc)
    ok = lib.N_VConstrMask_PihmGpu(vc, vx, vz)
    want_ok, want_m = NO.constr_mask(c, x)
    assert bool(ok) == want_ok and np.array_equal(tz.cpu().numpy(), want_m)
    for v in (vx, vy, vz, vc):
        lib.N_VDestroy_PihmGpu(v)


@pytest.mark.parametrize("n", SIZES)
def test_reductions(nv, n):
    lib, torch = nv
    rng = np.random.default_rng(200 + n)
    x = rng.normal(size=n)
    w = rng.uniform(1e3, 1e5, n)
    idm = rng.choice([0.0, 1.0], size=n)
    den = rng.normal(size=n)
    den[::3] = 0.0
    tx, tw, ti, td = (_vec(torch, a) for a in (x, w, idm, den))
    vx, vw, vi, vd = (_mk(lib, t) for t in (tx, tw, ti, td))
    rtol = 1e-13 + 2.2e-16 * np.log2(max(n, 2)) * 4
    pairs = [
        (lib.N_VDotProd_PihmGpu(vx, vw), NO.dot(x, w)),
        (lib.N_VWrmsNorm_PihmGpu(vx, vw), NO.wrms(x, w)),
        (lib.N_VWrmsNormMask_PihmGpu(vx, vw, vi), NO.wrms_mask(x, w, idm)),
        (lib.N_VWL2Norm_PihmGpu(vx, vw), NO.wl2(x, w)),
        (lib.N_VL1Norm_PihmGpu(vx), NO.l1(x)),
    ]
    scale_dot = float(np.abs(x * w).sum())
    for k, (got, want) in enumerate(pairs):
        ref = scale_dot if k == 0 else abs(want)
        assert abs(got - want) <= rtol * ref, (k, got, want)
    # order-free reductions are exact
    assert lib.N_VMaxNorm_PihmGpu(vx) == NO.max_norm(x)
    assert lib.N_VMin_PihmGpu(vx) == NO.vmin(x)
    assert lib.N_VMinQuotient_PihmGpu(vx, vd) == NO.min_quotient(x, den)
    # determinism: the same call twice gives the same bits
    assert lib.N_VDotProd_PihmGpu(vx, vw) == lib.N_VDotProd_PihmGpu(vx, vw)
    for v in (vx, vw, vi, vd):
        lib.N_VDestroy_PihmGpu(v)


def test_clone_and_family(nv):
    lib, torch = nv
    v = lib.N_VNew_PihmGpu(1000, None)
    w = lib.N_VClone_PihmGpu(v)
    a = np.arange(1000.0)
    assert lib.N_VCopyFromHost_PihmGpu(v, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    lib.N_VScale_PihmGpu(2.0, v, w)
    out = np.zeros(1000)
    assert lib.N_VCopyToHost_PihmGpu(w, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    assert np.array_equal(out, 2.0 * a)
    assert lib.N_VGetVectorID_PihmGpu(v) == 6  # SUNDIALS_NVEC_CUSTOM
    lib.N_VDestroy_PihmGpu(v)
    assert lib.N_VWL2Norm_PihmGpu(w, w) > 0  # family scratch outlives the first member
    lib.N_VDestroy_PihmGpu(w)


def test_raw_entry_points(nv):
    lib, torch = nv
    from pihm_gpu import nvector
    rng = np.random.default_rng(5)
    n = 100_003
    x, w = rng.normal(size=n), rng.uniform(1, 2, n)
    tx, tw = _vec(torch, x), _vec(torch, w)
    r = nvector.wrms_norm(tx.data_ptr(), tw.data_ptr(), n)
    assert abs(r - NO.wrms(x, w)) <= 1e-13 * NO.wrms(x, w)
    d = nvector.dot_prod(tx.data_ptr(), tw.data_ptr(), n)
    assert abs(d - NO.dot(x, w)) <= 1e-13 * float(np.abs(x * w).sum())


def _coef_value(kind, s, value=0.0):
    # the host forms of pihm_nv_coef (IEEE double, as the integrator forms them)
    if kind == NV.COEF_NEG:
        return -s
    if kind == NV.COEF_INV:
        return 1.0 / s
    if kind == NV.COEF_INV_INV:
        return 1.0 / (1.0 / s)
    if kind == NV.COEF_NEG_INV_INV:
        return -(1.0 / (1.0 / s))
    return value


SLOT_VALUES = [1.0, -1.0, 0.37, 2.5, -0.7, 0.7, 3.0, 1e-300]


@pytest.mark.parametrize("n", [7, 65_537, 3_060_000])
def test_device_scalars(nv, n):
    """Slot reductions equal the reductions that return to the host, bit for
    bit; linear sums with slot-derived coefficients equal N_VLinearSum with
    the host-formed coefficients (the case analysis made from the values on
    the device), for every coefficient kind and z aliasing."""
    lib, torch = nv
    rng = np.random.default_rng(300 + n)
    base = lib.N_VNew_PihmGpu(n, None)
    vecs = [lib.N_VClone_PihmGpu(base) for _ in range(5)]
    vx, vy, vz, ve, vo = vecs

    def put(v, a):
        a = np.ascontiguousarray(a, np.float64)
        assert lib.N_VCopyFromHost_PihmGpu(v, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0

    def get(v):
        out = np.empty(n)
        assert lib.N_VCopyToHost_PihmGpu(v, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
        return out

    def set_slot(slot, value):
        e = np.zeros(n)
        e[0] = value
        put(ve, e)
        put(vo, np.ones(n))
        assert lib.N_VDotProdSlot_PihmGpu(ve, vo, slot) == 0

    def fetch(count, word=None):
        out = (ctypes.c_double * count)()
        w = ctypes.c_uint(0)
        assert lib.N_VFetchSlots_PihmGpu(base, count, out, ctypes.c_void_p(word) if word else None,
                                         ctypes.byref(w)) == 0
        return list(out), w.value

    x = rng.normal(size=n)
    w = rng.uniform(1e3, 1e5, n)
    put(vx, x)
    put(vy, w)
    assert lib.N_VDotProdSlot_PihmGpu(vx, vy, 2) == 0
    assert lib.N_VWrmsNormSlot_PihmGpu(vx, vy, 3) == 0
    s2, s3 = fetch(4)[0][2:]
    assert s2 == lib.N_VDotProd_PihmGpu(vx, vy)
    assert s3 == lib.N_VWrmsNorm_PihmGpu(vx, vy)
    # the error word travels with the slots
    word = torch.tensor([7], dtype=torch.int32, device="cuda")
    vals, wv = fetch(4, word.data_ptr())
    assert wv == 7 and vals[2] == s2

    y = rng.normal(size=n)
    kinds = [NV.COEF_HOST, NV.COEF_NEG, NV.COEF_INV, NV.COEF_INV_INV, NV.COEF_NEG_INV_INV]
    large = n > 100_000
    checked = 0
    for sa in (SLOT_VALUES[:3] if large else SLOT_VALUES):
        for sb in ((-1.0,) if large else (1.0, -1.0, 0.37, -0.37)):
            set_slot(0, sa)
            set_slot(1, sb)
            for ka in kinds:
                for kb in ((NV.COEF_NEG, NV.COEF_NEG_INV_INV) if large else kinds):
                    a = _coef_value(ka, sa, sa)
                    b = _coef_value(kb, sb, sb)
                    for alias in (None, "x", "y"):
                        put(vx, x)
                        put(vy, y)
                        vzz = vx if alias == "x" else (vy if alias == "y" else vz)
                        ca = NV.Coef(ka, 0, sa if ka == NV.COEF_HOST else 0.0)
                        cb = NV.Coef(kb, 1, sb if kb == NV.COEF_HOST else 0.0)
                        assert lib.N_VLinearSumCoef_PihmGpu(ctypes.byref(ca), vx, ctypes.byref(cb), vy, vzz) == 0
                        want = NO.linear_sum(a, x, b, y, alias)
                        assert np.array_equal(get(vzz), want), (sa, sb, ka, kb, alias)
                        checked += 1
    assert checked > 0
    for v in vecs + [base]:
        lib.N_VDestroy_PihmGpu(v)
