"""Error of the table-driven FP64 pow used by the right-hand-side kernels,
against 60-digit decimal references, on the argument ranges the model
produces (Manning h^0.6666667, van Genuchten powers of saturation, their
complements), with CUDA's pow measured alongside."""
import ctypes
import decimal
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

decimal.getcontext().prec = 60


def _ulp_err(got, x, y):
    exact = decimal.Decimal(float(x)).ln() * decimal.Decimal(float(y))
    exact = exact.exp()
    ulp = math.ulp(float(exact))
    return float(abs(decimal.Decimal(float(got)) - exact) / decimal.Decimal(ulp))


def _cases(rng, n):
    cases = []
    h = np.exp(rng.uniform(np.log(1e-9), np.log(20.0), n))
    cases.append((h, np.full(n, 0.6666667)))
    beta = rng.uniform(1.2, 2.5, n)
    m = beta / (beta - 1.0)
    satn = rng.uniform(0.1, 1.0, n)
    cases.append((satn, m))
    cases.append((1.0 / satn, m))
    a = np.exp(rng.uniform(np.log(1e-12), np.log(1.0), n))
    cases.append((a, (beta - 1.0) / beta))
    cases.append((np.exp(rng.uniform(np.log(1e-12), np.log(1e4), n)), 1.0 / beta))
    cases.append((np.exp(rng.uniform(-50, 50, n)), rng.uniform(-6, 6, n)))
    return cases


def test_pow_fast_error_bound():
    import torch
    from pihm_gpu import capi
    lib = capi.load()
    f = lib.pihm_gpu_selftest_pow
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int64, ctypes.c_void_p]
    f.restype = ctypes.c_int
    rng = np.random.default_rng(7)
    worst_fast = worst_cuda = 0.0
    for x, y in _cases(rng, 3000):
        tx = torch.from_numpy(x).cuda()
        ty = torch.from_numpy(y).cuda()
        fast = torch.empty_like(tx)
        ref = torch.empty_like(tx)
        assert f(tx.data_ptr(), ty.data_ptr(), fast.data_ptr(), ref.data_ptr(), x.size, None) == 0
        torch.cuda.synchronize()
        fa, cu = fast.cpu().numpy(), ref.cpu().numpy()
        for k in range(x.size):
            worst_fast = max(worst_fast, _ulp_err(fa[k], x[k], y[k]))
            worst_cuda = max(worst_cuda, _ulp_err(cu[k], x[k], y[k]))
    print(f"max ulp error: table-driven pow {worst_fast:.3f}, CUDA pow {worst_cuda:.3f}")
    assert worst_fast <= 1.0, worst_fast


def test_pow_fast_special_values():
    import torch
    from pihm_gpu import capi
    lib = capi.load()
    f = lib.pihm_gpu_selftest_pow
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int64, ctypes.c_void_p]
    x = np.array([0.0, 1.0, 2.0, 4.0, 1e-310, np.inf, 0.5, 1e-300, 1e300, 1.0,
                  0.0, 0.0, 0.0, 0.0, -0.0, -0.0, 0.0])
    y = np.array([0.6666667, 3.7, 0.5, 0.5, 0.5, 0.5, 2000.0, 2.0, 0.5, 0.0,
                  3.0, 0.0, -1.0, np.nan, 3.0, 0.5, 5e-324])
    tx, ty = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    fast, ref = torch.empty_like(tx), torch.empty_like(tx)
    assert f(tx.data_ptr(), ty.data_ptr(), fast.data_ptr(), ref.data_ptr(), x.size, None) == 0
    torch.cuda.synchronize()
    fa, cu = fast.cpu().numpy(), ref.cpu().numpy()
    assert fa[0] == 0.0 and fa[1] == 1.0
    for k in range(x.size):
        if np.isfinite(cu[k]) and cu[k] != 0:
            assert abs(fa[k] - cu[k]) <= 2 * math.ulp(cu[k]), (k, fa[k], cu[k])
        else:  # zeros (with their sign), infinities and NaNs exactly as CUDA's pow
            assert (fa[k:k + 1].view(np.int64) == cu[k:k + 1].view(np.int64)).all() or (
                np.isnan(fa[k]) and np.isnan(cu[k])), (k, fa[k], cu[k])


def _manning(x, river):
    import torch
    from pihm_gpu import capi
    lib = capi.load()
    f = lib.pihm_gpu_selftest_pow_manning
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    f.restype = ctypes.c_int
    tx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    out = torch.empty_like(tx)
    assert f(tx.data_ptr(), int(river), out.data_ptr(), x.size, None) == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("river,p", [(0, 0.6666667), (1, 2.0 / 3.0)])
def test_pow_manning_error_bound(river, p):
    """x^0.6666667 (overland flow) and x^(2/3) (channel flow) through the
    integer-pipe power: within 0.6 ulp of the exact power of the double
    exponent over ponding depths and hydraulic radii, and over the whole range
    the path covers, [2^-126, 2^127)."""
    rng = np.random.default_rng(11 + river)
    typical = np.exp(rng.uniform(np.log(1e-9), np.log(1e3), 6000))
    wide = np.exp2(rng.uniform(-126.0, 126.99, 3000))
    edges = np.array([2.0 ** -126, np.nextafter(2.0 ** -126, 1.0), 2.0 ** 127 * (1 - 2 ** -52), 1.0,
                      np.nextafter(1.0, 0.0), np.nextafter(1.0, 2.0), 8.0, 0.125, 1e-4, 2e-4])
    x = np.concatenate([typical, wide, edges])
    got = _manning(x, river)
    errs = np.array([_ulp_err(got[k], x[k], p) for k in range(x.size)])
    print(f"pow_manning({p!r}): max ulp error {errs.max():.3f} (typical range "
          f"{errs[:typical.size].max():.3f})")
    assert errs.max() <= 0.6, (errs.max(), x[int(errs.argmax())])


@pytest.mark.parametrize("river", [0, 1])
def test_pow_manning_outside_range_is_pow_fast(river):
    """Zero, subnormals, values beyond 2^127, infinities and NaN take
    pow_fast, bit for bit."""
    import torch
    from pihm_gpu import capi
    p = 2.0 / 3.0 if river else 0.6666667
    x = np.array([0.0, 5e-324, 1e-310, 2.0 ** -127, 2.0 ** 127, 1e300, np.inf, np.nan, -1.0, -0.0])
    got = _manning(x, river)
    lib = capi.load()
    f = lib.pihm_gpu_selftest_pow
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int64, ctypes.c_void_p]
    tx = torch.from_numpy(x).cuda()
    ty = torch.full_like(tx, p)
    fast = torch.empty_like(tx)
    assert f(tx.data_ptr(), ty.data_ptr(), fast.data_ptr(), None, x.size, None) == 0
    torch.cuda.synchronize()
    want = fast.cpu().numpy()
    assert np.array_equal(got.view(np.int64), want.view(np.int64)), (got, want)
