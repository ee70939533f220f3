"""The numpy N_Vector restatement against golden vectors produced by the
reference's serial N_Vector (tests/golden/make_golden_nvector.py): every
result bit for bit."""
import os

import numpy as np

import nvector_oracle as NO

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nvector_calls.npz")


def test_nvector_oracle_bit_exact():
    z = np.load(GOLD)
    x, y, w, idm, c, den = (z[k] for k in ("x", "y", "w", "idm", "c", "den"))
    for k, (a, b) in enumerate(z["coefs"]):
        for alias in ("none", "x", "y"):
            got = NO.linear_sum(a, x, b, y, None if alias == "none" else alias)
            assert np.array_equal(got, z[f"lin{k}_{alias}"]), (a, b, alias)
    assert np.array_equal(np.full_like(x, 3.25), z["const"])
    assert np.array_equal(x * y, z["prod"])
    assert np.array_equal(x / y, z["div"])
    assert np.array_equal(NO.scale(0.3, x), z["scale"])
    assert np.array_equal(NO.scale(-1.0, x), z["neg"])
    assert np.array_equal(np.abs(x), z["abs"])
    assert np.array_equal(1.0 / y, z["inv"])
    assert np.array_equal(x + -0.5, z["addconst"])
    assert np.array_equal(NO.compare(0.8, x), z["compare"])
    ok, zz = NO.inv_test(x, np.full_like(x, 9.0))
    assert ok == bool(z["invtest_ok"]) and np.array_equal(zz, z["invtest"])
    ok, m = NO.constr_mask(c, x)
    assert ok == bool(z["constr_ok"]) and np.array_equal(m, z["constr"])
    assert NO.dot(x, w) == float(z["dot"])
    assert NO.max_norm(x) == float(z["maxnorm"])
    assert NO.wrms(x, w) == float(z["wrms"])
    assert NO.wrms_mask(x, w, idm) == float(z["wrmsmask"])
    assert NO.vmin(x) == float(z["min"])
    assert NO.wl2(x, w) == float(z["wl2"])
    assert NO.l1(x) == float(z["l1"])
    assert NO.min_quotient(x, den) == float(z["minq"])
