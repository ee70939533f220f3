// Table-driven FP64 pow for the right-hand-side kernels (sm_103a).
//
// GB300 issues about two FP64 instructions per clock per SM, so the dozens of
// FP64 operations inside a general-purpose pow dominate the PIHM right-hand
// side.  pow_fast(x, y) = exp(y ln x) follows P. T. P. Tang's table-driven
// algorithms ("Table-driven implementation of the exponential function in
// IEEE floating-point arithmetic", ACM TOMS 15(2) 1989; "... of the logarithm
// function ...", ACM TOMS 16(4) 1990) with 1024-entry tables generated by
// gen_fp64_tables.py:
//
//   ln x:  x = 2^k m, m in [1,2); i = top 10 fraction bits; r = m F_i - 1 is
//          formed exactly (two-product, Sterbenz); ln x = k ln2 + G_i +
//          log1p(r), log1p by its Taylor series to r^5 (|r| <= 2^-11, the
//          next term below 2^-68), carried as a double-double;
//   y ln x: double-double product;
//   exp:   z = (1024 q + j) ln2/1024 + r, |r| <= ln2/2048;
//          exp z = 2^q T_j (1 + expm1 r), expm1 by its Taylor series to r^4
//          (the next term below 2^-64 relative).
//
// Error: about 0.51 ulp for the arguments the model produces (checked against
// 60-digit references and CUDA's pow in tests/test_fp64_math_gpu.py).  The
// fast path needs x positive and normal and |y ln x| < 700; +0 to a positive
// power is +0, and everything else (x < 0, -0, subnormal, inf, nan, other
// powers of +0, overflow, underflow) goes to pow().
#pragma once

#include <cmath>

#include "fp64_cmp.h"
#include "fp64_tables.h"

namespace pihm {

__device__ __forceinline__ double exp_dd_fast(double zh, double zl) {
  const double shifter = 0x1.8p52;  // 1.5 * 2^52: rounds to an integer in the low bits
  const double u = fma(zh, kNByLn2, shifter);
  const int kk = __double2loint(u);
  const double nd = u - shifter;
  double r = fma(-nd, kLn2ByNHi, zh);
  r = fma(-nd, kLn2ByNLo, r) + zl;
  double p = fma(r, 1.0 / 24.0, 1.0 / 6.0);
  p = fma(p, r, 0.5);
  p = fma(p, r * r, r);  // expm1(r)
  const int j = kk & ((1 << kTableBits) - 1);
  const int q = kk >> kTableBits;
  const double th = __ldg(&kExpThi[j]);
  const double tl = __ldg(&kExpTlo[j]);
  const double res = th + fma(th, p, tl);
  return __longlong_as_double(__double_as_longlong(res) + ((long long)q << 52));
}

// ln x as a double-double (sh + lo) for x positive and normal (the logarithm
// half of pow_fast); false for anything else.
__device__ __forceinline__ bool log_dd_fast(double x, double &sh, double &lo) {
  const long long xb = __double_as_longlong(x);
  const unsigned top = (unsigned)((unsigned long long)xb >> 52);  // sign and exponent
  if (top - 1u >= 2046u) return false;  // x <= 0, zero, subnormal, inf or nan
  const int k = (int)top - 1023;
  const double m = __longlong_as_double((xb & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
  const int i = (int)((xb >> (52 - kTableBits)) & ((1 << kTableBits) - 1));
  const double F = __ldg(&kLogF[i]);
  const double gh = __ldg(&kLogGhi[i]);
  const double gl = __ldg(&kLogGlo[i]);
  const double p = m * F;
  const double pe = fma(m, F, -p);
  const double rh = p - 1.0;
  double q = fma(rh, 0.2, -0.25);
  q = fma(q, rh, 1.0 / 3.0);
  q = fma(q, rh, -0.5);
  const double t = (rh * rh) * q;
  const double kd = (double)k;
  const double s1 = fma(kd, kLn2Hi, gh);
  sh = s1 + rh;
  const double bb = sh - s1;
  const double se = (s1 - (sh - bb)) + (rh - bb);
  lo = se + (fma(-pe, rh, pe) + (t + fma(kd, kLn2Lo, gl)));
  return true;
}

// y (sh + lo) as a double-double zh + zl (Dekker's product with an FMA)
__device__ __forceinline__ void mul_dd(double y, double sh, double lo, double &zh, double &zl) {
  zh = y * sh;
  zl = fma(y, lo, fma(y, sh, -zh));
}

// (ah + al) - (bh + bl) as an unnormalised double-double: Knuth's two-sum of
// the high parts, its error plus the difference of the low parts
__device__ __forceinline__ void sub_dd(double ah, double al, double bh, double bl, double &sh,
                                       double &sl) {
  sh = ah - bh;
  const double bb = sh - ah;
  sl = ((ah - (sh - bb)) - (bh + bb)) + (al - bl);
}

// exp(zh + zl) through the table path when |zh| < 700 (the range
// exp_dd_fast covers); false otherwise
__device__ __forceinline__ bool exp_dd_checked(double zh, double zl, double &r) {
  if (!cmp::abs_lt_c(zh, 700.0)) return false;
  r = exp_dd_fast(zh, zl);
  return true;
}

// x^y from ln x = sh + lo (log_dd_fast), y finite; pow(x, y) is the fallback
// when y ln x leaves the fast range.  pow_fast(x, y) == pow_from_log(x, sh,
// lo, y) bit for bit.
__device__ __forceinline__ double pow_from_log(double x, double sh, double lo, double y) {
  double zh, zl, r;
  mul_dd(y, sh, lo, zh, zl);
  return exp_dd_checked(zh, zl, r) ? r : pow(x, y);
}

__device__ __forceinline__ double pow_fast(double x, double y) {
  const long long xb = __double_as_longlong(x);
  const unsigned top = (unsigned)((unsigned long long)xb >> 52);  // sign and exponent
  if (top - 1u >= 2046u) {  // x <= 0, zero, subnormal, inf or nan
    // +0 to a positive power is +0 (C99 F.9.4.4): a full soil column makes
    // 1 - satn^m exactly 0, so this case is common enough to skip the call
    if (xb == 0 && cmp::gt0(y)) return 0.0;
    return pow(x, y);
  }
  const int k = (int)top - 1023;
  const double m = __longlong_as_double((xb & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
  const int i = (int)((xb >> (52 - kTableBits)) & ((1 << kTableBits) - 1));
  const double F = __ldg(&kLogF[i]);
  const double gh = __ldg(&kLogGhi[i]);
  const double gl = __ldg(&kLogGlo[i]);
  // r = m F - 1 = rh + pe exactly
  const double p = m * F;
  const double pe = fma(m, F, -p);
  const double rh = p - 1.0;
  // log1p(rh) - rh = rh^2 (-1/2 + rh (1/3 + rh (-1/4 + rh/5)))
  double q = fma(rh, 0.2, -0.25);
  q = fma(q, rh, 1.0 / 3.0);
  q = fma(q, rh, -0.5);
  const double t = (rh * rh) * q;
  // k ln2 + G_hi is exact; add rh with an exact two-sum
  const double kd = (double)k;
  const double s1 = fma(kd, kLn2Hi, gh);
  const double sh = s1 + rh;
  const double bb = sh - s1;
  const double se = (s1 - (sh - bb)) + (rh - bb);
  // low part: two-sum error, the low half of r (times 1 - rh), the series
  // tail, k ln2_lo + G_lo
  const double lo = se + (fma(-pe, rh, pe) + (t + fma(kd, kLn2Lo, gl)));
  // z = y (sh + lo) as a double-double
  double zh, zl, res;
  mul_dd(y, sh, lo, zh, zl);
  return exp_dd_checked(zh, zl, res) ? res : pow(x, y);
}

// Manning exponents: OverlandFlow's 0.6666667 (src/lat_flow.c:279-283) and
// the river's 2.0 / 3.0 (src/river_flow.c), as offsets from 2/3:
// fl(0.6666667) - 2/3 and fl(2/3) - 2/3, exact to 2^-100.
constexpr double kManningSurf = 0.6666667;
constexpr double kManningSurfDelta = 0x1.1e54c66aaaaabp-25;
constexpr double kManningRiv = 2.0 / 3.0;
constexpr double kManningRivDelta = -0x1.5555555555555p-55;

__device__ __forceinline__ float lg2_approx(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// x^p for p = 2/3 + delta with |delta| <= 2^-24 (the Manning exponents), in
// about 24 FP64 operations instead of pow_fast's 37:
//
//   x^p = x * x^(-1/3) * exp(delta ln x)
//
//   x^(-1/3): with x = 2^k m, k = 3q + s (s in {0, 1, 2}), a single-precision
//     estimate r0 = 2^-q 2^(-(s + lg2 m)/3) from lg2/ex2.approx on [1, 2)
//     and (-1, 0] (relative error about 2^-22; 2^-q goes into the exponent
//     field exactly), corrected by the binomial series
//     (1 - e)^(-1/3) = 1 + e/3 + 2e^2/9 + 14e^3/81 + ... with e = 1 - x r0^3;
//     r0^2 is exact (r0 has 24 significant bits) and r0^3 is carried as an
//     exact two-product, so e is exact to 2^-100 and the dropped 14e^3/81 is
//     below 2^-60;
//   exp(delta ln x) = 1 + v, v = u + u^2/2 + u^3/6, u = delta ln x,
//     |u| < 2^-17 over the range below (the next term is below 2^-72); ln x
//     from the 1024-entry log table (|r| <= 2^-11) and log1p(r) to r^3,
//     absolute error below 2e-14, which moves u by less than 2^-69;
//   x r0 = ph + pl exactly, and everything else goes into one correction
//     term: x^p = ph + (pl + ph w), w = (1 + c)(1 + v) - 1.
//
// Error: the final rounding (0.5 ulp) plus about 2^-60 relative
// (tests/test_fp64_math_gpu.py measures it against 60-digit references).
// x outside [2^-126, 2^127) (zero, subnormal, huge, negative, inf, NaN)
// goes to pow_fast(x, p).
__device__ __forceinline__ double pow_manning(double x, double p, double delta) {
  const long long xb = __double_as_longlong(x);
  const unsigned hi = (unsigned)((unsigned long long)xb >> 32);
  const unsigned lo = (unsigned)xb;
  const unsigned top = hi >> 20;  // sign and exponent
  if (top - (1023u - 126u) >= 253u) return pow_fast(x, p);
  const int k = (int)top - 1023;
  const int q = (k + 384) / 3 - 128;  // floor(k / 3): k + 384 > 0
  const int s3 = k - 3 * q;
  // m in [1, 2) truncated to single precision, and r0 = 2^-q 2^y widened
  // exactly, y = -(s + lg2 m)/3 in (-1, 0]
  const float mf = __uint_as_float(0x3F800000u | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
  const float y = -((float)s3 + lg2_approx(mf)) * (1.0f / 3.0f);
  const unsigned rb = __float_as_uint(ex2_approx(y));
  const int rhi = (int)((rb >> 3) + ((1023u - 127u) << 20)) - q * (1 << 20);
  const double r0 = __hiloint2double(rhi, (int)(rb << 29));
  // e = 1 - x r0^3, with r0^3 = r3h + r3l
  const double r2 = r0 * r0;
  const double r3h = r2 * r0;
  const double r3l = fma(r2, r0, -r3h);
  const double e = fma(-x, r3l, fma(-x, r3h, 1.0));
  const double c = e * fma(e, 2.0 / 9.0, 1.0 / 3.0);
  // ln x = k ln 2 + G_i + log1p(r), r = m F_i - 1
  const double m = __longlong_as_double((xb & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
  const int i = (int)((xb >> (52 - kTableBits)) & ((1 << kTableBits) - 1));
  const double r = fma(m, __ldg(&kLogF[i]), -1.0);
  const double lp = fma(fma(r, 1.0 / 3.0, -0.5), r * r, r);
  const double lnx = fma((double)k, kLn2Hi, __ldg(&kLogGhi[i])) + lp;
  const double u = delta * lnx;
  const double v = fma(u, u * fma(u, 1.0 / 6.0, 0.5), u);
  const double w = fma(c, v, c + v);
  const double ph = x * r0;
  const double pl = fma(x, r0, -ph);
  return ph + fma(ph, w, pl);
}

}  // namespace pihm
