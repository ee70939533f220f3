"""Generate fp64_tables.h: the lookup tables of the table-driven FP64 pow in
fp64_math.cuh, computed to 60 significant digits with Python's decimal module.

    python gen_fp64_tables.py > fp64_tables.h

Method (P. T. P. Tang, "Table-driven implementation of the exponential
function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989, and
"Table-driven implementation of the logarithm function in IEEE
floating-point arithmetic", ACM TOMS 16(4), 1990):

  log:  x = 2^k m, m in [1, 2); i = the top 10 fraction bits of m;
        F_i = double nearest 1 / (1 + (i + 1/2) / 1024);
        ln x = k ln2 + G_i + log1p(m F_i - 1), G_i = -ln F_i
        G_i is split as G_hi (a multiple of 2^-42, so k*L2_hi + G_hi is
        exact) + G_lo.
  exp:  z = (1024 q + j) ln2 / 1024 + r, |r| <= ln2 / 2048;
        exp z = 2^q * T_j * exp(r), T_j = 2^(j/1024) split as T_hi + T_lo.

1024 entries per table (40 KB in all) keep the polynomials short: log1p(r)
to r^5 for |r| <= 2^-11 and expm1(r) to r^4 for |r| <= ln2/2048.
"""
import decimal
from decimal import Decimal as D

decimal.getcontext().prec = 60

N = 1024  # entries per table

LN2 = D(2).ln()


def dbl(v: D) -> float:
    """Round a decimal to the nearest double (via its exact repr)."""
    return float(v)


def exact(f: float) -> D:
    return D(f)  # a double's exact decimal value


def split42(v: D):
    hi = D(round(v * (D(2) ** 42))) / (D(2) ** 42)
    return float(hi), dbl(v - hi)


def main():
    out = []
    out.append("// Generated by gen_fp64_tables.py -- tables of the table-driven FP64 pow")
    out.append("// (Tang 1989/1990), 60-digit decimal arithmetic.  Do not edit.")
    out.append("#pragma once")
    out.append("")
    F, GH, GL = [], [], []
    for i in range(N):
        c = 1 + (D(i) + D("0.5")) / N
        f = dbl(1 / c)
        g = -(exact(f).ln())
        gh, gl = split42(g)
        assert exact(gh) + exact(gl) - g < D(2) ** -95
        F.append(f)
        GH.append(gh)
        GL.append(gl)
    TH, TL = [], []
    for j in range(N):
        t = (D(2) ** (D(j) / N))
        th = dbl(t)
        tl = dbl(t - exact(th))
        TH.append(th)
        TL.append(tl)
    l2h, l2l = split42(LN2)
    c = LN2 / N
    ch = dbl(c)
    cl = dbl(c - exact(ch))
    inv = dbl(N / LN2)

    def arr(name, vals):
        out.append(f"static __device__ const double {name}[{N}] = {{")
        for k in range(0, N, 4):
            out.append("    " + ", ".join(v.hex() if False else repr_hex(v) for v in vals[k:k + 4]) + ",")
        out.append("};")

    arr("kLogF", F)
    arr("kLogGhi", GH)
    arr("kLogGlo", GL)
    arr("kExpThi", TH)
    arr("kExpTlo", TL)
    out.append(f"static constexpr double kLn2Hi = {repr_hex(l2h)};  // ln 2, multiple of 2^-42")
    out.append(f"static constexpr double kLn2Lo = {repr_hex(l2l)};")
    out.append(f"static constexpr int kTableBits = {N.bit_length() - 1};")
    out.append(f"static constexpr double kLn2ByNHi = {repr_hex(ch)};  // ln 2 / {N}")
    out.append(f"static constexpr double kLn2ByNLo = {repr_hex(cl)};")
    out.append(f"static constexpr double kNByLn2 = {repr_hex(inv)};")
    print("\n".join(out))


def repr_hex(v: float) -> str:
    """A C hexadecimal floating literal that is exactly v."""
    return float.hex(v)


if __name__ == "__main__":
    main()
