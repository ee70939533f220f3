"""The integer-pipe logarithm, exponential and power of the right-hand-side
kernels (pihm-cuda_gb300/csrc/int_math.cuh).

The arithmetic is integer, so the header compiled for the host
(tests/int_math_host.cpp) gives the bits the GPU computes: the CPU tests
measure the power's error against 200-bit references on the argument ranges
the model produces (van Genuchten powers of saturation and their complements,
Manning's h^0.6666667) and on wide ranges, and hold the division and square
root to the IEEE results bit for bit; the GPU tests check that the device
returns the same bits as the host build."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "pihm-cuda_gb300", "csrc")
P = ctypes.c_void_p


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    so = str(tmp_path_factory.mktemp("im") / "libim.so")
    subprocess.run([gxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-I", CSRC,
                    os.path.join(HERE, "int_math_host.cpp"), "-o", so], check=True)
    return ctypes.CDLL(so)


def host_pow(lib, x, y):
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    out = np.empty_like(x)
    ok = np.empty(x.size, np.int32)
    lib.im_pow(P(x.ctypes.data), P(y.ctypes.data), P(out.ctypes.data), P(ok.ctypes.data),
               ctypes.c_int64(x.size))
    return out, ok.astype(bool)


def model_cases(rng, n):
    beta = rng.uniform(1.2, 2.5, n)
    m = beta / (beta - 1.0)
    satn = rng.uniform(0.1, 1.0, n)
    a = np.exp(rng.uniform(np.log(1e-15), 0.0, n))
    return {
        "satn^m": (satn, m),
        "(1/satn)^m": (1.0 / satn, m),
        "(1-satn^m)^e": (a, (beta - 1.0) / beta),
        "v^(1/beta)": (np.exp(rng.uniform(np.log(1e-12), np.log(1e4), n)), 1.0 / beta),
        "h^0.6666667": (np.exp(rng.uniform(np.log(1e-9), np.log(20.0), n)), np.full(n, 0.6666667)),
        "h^(2/3)": (np.exp(rng.uniform(np.log(1e-6), np.log(50.0), n)), np.full(n, 2.0 / 3.0)),
        "wide": (np.exp(rng.uniform(-40.0, 40.0, n)), rng.uniform(-3.0, 3.0, n)),
    }


def test_error_against_high_precision_references(host_lib):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    rng = np.random.default_rng(2024)
    for name, (x, y) in model_cases(rng, 4000).items():
        got, ok = host_pow(host_lib, x, y)
        if name != "wide":
            assert ok.all(), name  # every power of the model takes the integer path
        worst, misrounded = 0.0, 0
        for k in np.nonzero(ok)[0]:
            exact = mpmath.power(mpmath.mpf(float(x[k])), mpmath.mpf(float(y[k])))
            ulp = np.spacing(abs(float(exact)))
            err = float(abs(mpmath.mpf(float(got[k])) - exact) / ulp)
            worst = max(worst, err)
            misrounded += err > 0.5
        print(f"{name}: worst {worst:.4f} ulp, {misrounded} of {int(ok.sum())} not correctly rounded")
        assert worst < 0.502, (name, worst)
        assert misrounded <= 0.005 * ok.sum(), (name, misrounded)


def test_reciprocal_power_through_the_shared_logarithm(host_lib):
    """fl(1/x)^y from the logarithm of x and the exact residual of the
    division (log2k_recip, Psi's (1/satn)^m in the element kernel): within
    0.502 ulp of the exact power of the rounded reciprocal, like pow_i, on
    the model's saturations and exponents and on wide ranges."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    rng = np.random.default_rng(31)
    n = 4000
    beta = rng.uniform(1.2, 2.5, n)
    cases = {
        "(1/satn)^m": (rng.uniform(0.1, 1.0, n), beta / (beta - 1.0)),
        "satn near 1": (1.0 - rng.integers(0, 2000, n) * 2.0 ** -53, beta / (beta - 1.0)),
        "wide": (np.exp(rng.uniform(-20.0, 20.0, n)), rng.uniform(-3.0, 3.0, n)),
    }
    for name, (x, y) in cases.items():
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        out = np.empty_like(x)
        ok = np.empty(x.size, np.int32)
        host_lib.im_pow_recip(P(x.ctypes.data), P(y.ctypes.data), P(out.ctypes.data), P(ok.ctypes.data),
                              ctypes.c_int64(x.size))
        ok = ok.astype(bool)
        assert ok.mean() > 0.99, name
        q = 1.0 / x
        worst, misrounded = 0.0, 0
        for k in np.nonzero(ok)[0]:
            exact = mpmath.power(mpmath.mpf(float(q[k])), mpmath.mpf(float(y[k])))
            err = float(abs(mpmath.mpf(float(out[k])) - exact) / np.spacing(abs(float(exact))))
            worst = max(worst, err)
            misrounded += err > 0.5
        print(f"{name}: worst {worst:.4f} ulp, {misrounded} of {int(ok.sum())} not correctly rounded")
        assert worst < 0.502, (name, worst)
        assert misrounded <= 0.005 * ok.sum(), (name, misrounded)


def test_exact_cases_and_declined_arguments(host_lib):
    x = np.array([1.0, 0.5, 2.0, 4.0, 0.25, 8.0, 0.0, 0.0,
                  1.0, 0.0, 0.0, -0.0, -1.0, np.nan, np.inf, 1e-310, 2.0 ** 130, 2.0, 2.0])
    y = np.array([3.7, 2.0, 10.0, 0.5, -1.5, 1.0 / 3.0, 0.5, 7.0,
                  0.0, 0.0, -0.5, 0.5, 0.5, 0.5, 0.5, 0.5, 0.5, 1e-9, 1e12])
    got, ok = host_pow(host_lib, x, y)
    assert ok[:8].all()
    assert list(got[:8]) == [1.0, 0.25, 1024.0, 2.0, 8.0, 2.0, 0.0, 0.0]
    assert not np.signbit(got[6:8]).any()
    # y = 0, +0 to a non-positive power, -0, negative, NaN, infinite,
    # subnormal or huge x, tiny or huge exponents: declined (the kernels use
    # the FP64 path there)
    assert not ok[8:].any()


@pytest.mark.gpu
def test_device_bits_equal_host_bits(host_lib):
    import torch
    from pihm_gpu import capi
    lib = capi.load()
    f = lib.pihm_gpu_selftest_pow_int
    f.argtypes = [P] * 4 + [ctypes.c_int64, P]
    f.restype = ctypes.c_int
    rng = np.random.default_rng(77)
    for name, (x, y) in model_cases(rng, 200_000).items():
        want, ok_h = host_pow(host_lib, x, y)
        tx, ty = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
        out = torch.empty_like(tx)
        ok = torch.empty(x.size, dtype=torch.int32, device="cuda")
        assert f(tx.data_ptr(), ty.data_ptr(), out.data_ptr(), ok.data_ptr(), x.size, None) == 0
        torch.cuda.synchronize()
        assert np.array_equal(ok.cpu().numpy().astype(bool), ok_h), name
        got = out.cpu().numpy()
        assert np.array_equal(got[ok_h].view(np.int64), want[ok_h].view(np.int64)), name


def host_div_sqrt(lib, a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    q, r = np.empty_like(a), np.empty_like(a)
    okq, okr = np.empty(a.size, np.int32), np.empty(a.size, np.int32)
    lib.im_div(P(a.ctypes.data), P(b.ctypes.data), P(q.ctypes.data), P(okq.ctypes.data), ctypes.c_int64(a.size))
    lib.im_sqrt(P(a.ctypes.data), P(r.ctypes.data), P(okr.ctypes.data), ctypes.c_int64(a.size))
    return q, okq.astype(bool), r, okr.astype(bool)


def div_sqrt_cases(rng, n):
    bits = lambda: np.frombuffer(rng.integers(0, 2 ** 63, n, dtype=np.int64).tobytes(), np.float64)  # noqa: E731
    sign = lambda: rng.choice([-1.0, 1.0], n)  # noqa: E731
    near1 = lambda: 1.0 + rng.integers(-4000, 4000, n) * 2.0 ** -52  # noqa: E731
    return {
        "model": (rng.uniform(0.0, 10.0, n), rng.uniform(0.1, 10.0, n)),
        "wide": (np.exp(rng.uniform(-340, 340, n)) * sign(), np.exp(rng.uniform(-340, 340, n)) * sign()),
        "near one": (near1() * rng.choice([1.0, 2.0, 4.0], n), near1()),
        "integers": (rng.integers(1, 1 << 53, n).astype(np.float64), rng.integers(1, 1 << 26, n).astype(np.float64)),
        "squares": ((rng.integers(1, 1 << 26, n).astype(np.float64)) ** 2, np.full(n, 3.0)),
        "bit patterns": (np.abs(bits()), bits()),
        "zero dividends": (np.zeros(n) * sign(), np.exp(rng.uniform(-340, 340, n)) * sign()),
    }


def test_division_and_sqrt_are_ieee_bit_for_bit(host_lib):
    rng = np.random.default_rng(99)
    for name, (a, b) in div_sqrt_cases(rng, 400_000).items():
        q, okq, r, okr = host_div_sqrt(host_lib, a, b)
        with np.errstate(all="ignore"):
            wq, wr = a / b, np.sqrt(a)
        assert okq.mean() > 0.7 and okr[a >= 0].mean() > 0.99, name
        assert np.array_equal(q[okq].view(np.int64), wq[okq].view(np.int64)), name
        assert np.array_equal(r[okr].view(np.int64), wr[okr].view(np.int64)), name
    # a zero dividend gives the signed zero and the root of a zero is that
    # zero; subnormals, infinities, NaN, zero divisors and out-of-range
    # quotients are declined; the square root declines negative arguments too
    a = np.array([0.0, -0.0, 5e-324, np.inf, np.nan, 1.0, 1e300, 1e-300, -4.0])
    b = np.array([-1.0, 1.0, 1.0, 1.0, 1.0, 0.0, 1e-300, 1e300, 1.0])
    q, okq, r, okr = host_div_sqrt(host_lib, a, b)
    assert list(okq) == [True, True] + [False] * 6 + [True] and q[8] == -4.0
    assert q[0] == 0.0 and np.signbit(q[0]) and q[1] == 0.0 and np.signbit(q[1])
    assert list(okr) == [True, True, False, False, False, True, True, True, False]
    assert r[0] == 0.0 and not np.signbit(r[0]) and np.signbit(r[1])


@pytest.mark.gpu
def test_device_division_and_sqrt_bits_equal_host_bits(host_lib):
    import torch
    from pihm_gpu import capi
    lib = capi.load()
    f = lib.pihm_gpu_selftest_div_sqrt_int
    f.argtypes = [P] * 5 + [ctypes.c_int64, P]
    f.restype = ctypes.c_int
    rng = np.random.default_rng(5)
    for name, (a, b) in div_sqrt_cases(rng, 500_000).items():
        q, okq, r, okr = host_div_sqrt(host_lib, a, b)
        ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        gq, gr = torch.empty_like(ta), torch.empty_like(ta)
        ok = torch.empty(a.size, dtype=torch.int32, device="cuda")
        assert f(ta.data_ptr(), tb.data_ptr(), gq.data_ptr(), gr.data_ptr(), ok.data_ptr(), a.size, None) == 0
        torch.cuda.synchronize()
        o = ok.cpu().numpy()
        assert np.array_equal((o & 1).astype(bool), okq) and np.array_equal((o & 2).astype(bool), okr), name
        assert np.array_equal(gq.cpu().numpy()[okq].view(np.int64), q[okq].view(np.int64)), name
        assert np.array_equal(gr.cpu().numpy()[okr].view(np.int64), r[okr].view(np.int64)), name
