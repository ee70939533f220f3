"""Generate int_tables.h: the lookup tables and constants of the integer-pipe
logarithm and exponential in int_math.cuh, computed to 60 significant digits
with Python's decimal module.

    python gen_int_tables.py > int_tables.h

Method (the table-driven reductions of P. T. P. Tang, ACM TOMS 15(2) 1989 and
16(4) 1990, carried out in fixed-point integer arithmetic):

  log:  x = 2^k m, m in [1, 2); i = the top 10 fraction bits of m;
        c_i = 1 + (i + 1/2)/1024, F_i = round(4096 / c_i) / 4096 (12 bits,
        so M F_i - 2^64 is exact in 64-bit integer arithmetic for the 53-bit
        integer mantissa M); r = m F_i - 1, |r| < 2^-10.4;
        1024 log2 x = 1024 k + H_i + (1024/ln 2) log1p(r), H_i = -1024 log2 F_i.
  exp:  2^(t/1024), t = 1024 q + j + f, |f| <= 1/2:
        2^(t/1024) = 2^q T_j exp(f ln2/1024), T_j = 2^(j/1024).
"""
import decimal
from decimal import Decimal as D

decimal.getcontext().prec = 60

N = 1024
LN2 = D(2).ln()


def rnd(v: D) -> int:
    return int(v.to_integral_value(rounding=decimal.ROUND_HALF_EVEN))


def main():
    out = ["// Generated by gen_int_tables.py -- tables of the integer-pipe log/exp",
           "// (int_math.cuh), 60-digit decimal arithmetic.  Do not edit.",
           "#pragma once", "", "#include <cstdint>", ""]
    F, H = [], []
    for i in range(N):
        c = 1 + (D(i) + D("0.5")) / N
        fi = rnd(D(4096) / c)
        F.append(fi)
        h = -D(1024) * (D(fi) / 4096).ln() / LN2  # -1024 log2 F_i
        H.append(rnd(h * (D(2) ** 53)))
        assert 0 <= H[-1] < 2 ** 63
    T = []
    for j in range(N):
        t = D(2) ** (D(j) / N)
        T.append(rnd(t * (D(2) ** 63)))
        assert 2 ** 63 <= T[-1] < 2 ** 64
    # check the reduction bound |r| < 2^-10.4 over every interval's ends
    worst = D(0)
    for i in range(N):
        for m in (1 + D(i) / N, 1 + D(i + 1) / N):
            worst = max(worst, abs(m * D(F[i]) / 4096 - 1))
    assert worst < D(2) ** D("-10.4"), worst

    def arr(ctype, name, vals, per=4):
        out.append(f"PIHM_IM_TABLE {ctype} {name}[{N}] = {{")
        for k in range(0, N, per):
            out.append("    " + ", ".join(f"{v}" + ("ull" if ctype == "uint64_t" else "ll" if ctype == "int64_t"
                                                    else "u") for v in vals[k:k + per]) + ",")
        out.append("};")

    arr("uint16_t", "kImLogF", F, 16)
    arr("int64_t", "kImLogH", H)
    arr("uint64_t", "kImExpT", T)
    consts = {
        # log1p(r) - r = r^2 (-1/2 + r/3 - r^2/4 + r^3/5), at scale 2^62
        "kImL5": rnd(D(2) ** 62 / 5), "kImL4": -(2 ** 60), "kImL3": rnd(D(2) ** 62 / 3), "kImL2": -(2 ** 61),
        # 1024 / ln 2 at scale 2^52
        "kImK": rnd(D(N) / LN2 * D(2) ** 52),
        # ln 2 at scale 2^63
        "kImLn2": rnd(LN2 * D(2) ** 63),
        # expm1(r) - r = r^2 (1/2 + r/6 + r^2/24 + r^3/120), at scale 2^62
        "kImE120": rnd(D(2) ** 62 / 120), "kImE24": rnd(D(2) ** 62 / 24), "kImE6": rnd(D(2) ** 62 / 6),
        "kImE2": 2 ** 61,
    }
    for k, v in consts.items():
        assert -(2 ** 63) <= v < 2 ** 63
        out.append(f"static constexpr int64_t {k} = {v}ll;")
    print("\n".join(out))


if __name__ == "__main__":
    main()
