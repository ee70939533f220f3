"""numpy restatement of the SUNDIALS 2.7 serial N_Vector operations
(cvode/src/nvec_ser/nvector_serial.c:421-1060 of the reference) -- test
infrastructure only.

Element-wise operations follow the serial code's case analysis, because the
special cases change the rounding (e.g. a == b computes a*(x+y), not
a*x + b*y); numpy evaluates each element with one IEEE operation per C
operator, so these agree bit for bit with the C code.  Reductions are
restated as left-to-right sums (math.fsum is NOT used: the serial code
accumulates in order).
"""
from __future__ import annotations

import math

import numpy as np


def linear_sum(a, x, b, y, z_is=None):
    """z = a*x + b*y.  `z_is` names the operand z aliases ('x', 'y' or None),
    which selects the serial code's in-place (axpy) branches."""
    if b == 1.0 and z_is == "y":
        if a == 1.0:
            return y + x
        if a == -1.0:
            return y - x
        return y + a * x
    if a == 1.0 and z_is == "x":
        if b == 1.0:
            return x + y
        if b == -1.0:
            return x - y
        return x + b * y
    if a == 1.0 and b == 1.0:
        return x + y
    if a == 1.0 and b == -1.0:
        return x - y
    if a == -1.0 and b == 1.0:
        return y - x
    if a == 1.0:
        return (b * y) + x
    if b == 1.0:
        return (a * x) + y
    if a == -1.0:
        return (b * y) - x
    if b == -1.0:
        return (a * x) - y
    if a == b:
        return a * (x + y)
    if a == -b:
        return a * (x - y)
    return (a * x) + (b * y)


def scale(c, x):
    if c == 1.0:
        return x.copy()
    if c == -1.0:
        return -x
    return c * x


def _seqsum(v):
    s = 0.0
    for t in v.tolist():
        s += t
    return s


def dot(x, y):
    return _seqsum(x * y)


def wrms(x, w):
    p = x * w
    return math.sqrt(_seqsum(p * p) / x.size)


def wrms_mask(x, w, idm):
    p = np.where(idm > 0.0, x * w, 0.0)
    return math.sqrt(_seqsum(p * p) / x.size)


def wl2(x, w):
    p = x * w
    return math.sqrt(_seqsum(p * p))


def l1(x):
    return _seqsum(np.abs(x))


def max_norm(x):
    return float(np.max(np.abs(x))) if x.size else 0.0


def vmin(x):
    return float(np.min(x))


def compare(c, x):
    return np.where(np.abs(x) >= c, 1.0, 0.0)


def inv_test(x, z):
    z = z.copy()
    nz = x != 0.0
    z[nz] = 1.0 / x[nz]
    return bool(np.all(nz)), z


def constr_mask(c, x):
    m = np.zeros_like(x)
    p = x * c
    strong = (c > 1.5) | (c < -1.5)
    weak = ~strong & ((c > 0.5) | (c < -0.5))
    bad = (c != 0.0) & ((strong & (p <= 0.0)) | (weak & (p < 0.0)))
    m[bad] = 1.0
    return bool(not bad.any()), m


def min_quotient(num, den):
    nz = den != 0.0
    if not nz.any():
        return np.finfo(np.float64).max
    return float(np.min(num[nz] / den[nz]))
