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
#include "int_math.cuh"

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
// the river's 2.0 / 3.0 (src/river_flow.c).
constexpr double kManningSurf = 0.6666667;
constexpr double kManningRiv = 2.0 / 3.0;

// pow_fast as an out-of-line call: the fallback of pow_any, taken by few
// lanes, so its code and registers stay out of the callers
static __device__ __noinline__ double pow_slow(double x, double y) { return pow_fast(x, y); }

// x^y: the integer-pipe power (int_math.cuh) where x and y are inside its
// ranges -- every power of the right-hand side's states -- and pow_fast
// otherwise (x <= 0, subnormal, huge or tiny x, y zero or extreme, results
// outside about (1e-29, 8e28)).  Both are within 0.502 ulp of the exact
// power.
__device__ __forceinline__ double pow_any(double x, double y) {
  double r;
  return im::pow_i(x, y, r) ? r : pow_slow(x, y);
}

// a / b and sqrt(x), correctly rounded: the integer-pipe paths where the
// operands and the result are normal, the FP64 instructions otherwise (the
// same bits either way)
// The FP64 instructions sit out of line, as pow_any's fallback does: a
// division or root inlined behind the test would be predicated rather than
// branched around, and issued to the FP64 pipe by every warp.
static __device__ __noinline__ double div_slow(double a, double b) { return a / b; }
static __device__ __noinline__ double sqrt_slow(double x) { return sqrt(x); }
__device__ __forceinline__ double div_any(double a, double b) {
  double q;
  return im::div_i(a, b, q) ? q : div_slow(a, b);
}
__device__ __forceinline__ double sqrt_any(double x) {
  double r;
  return im::sqrt_i(x, r) ? r : sqrt_slow(x);
}

// the Manning powers h^0.6666667 and h^(2/3)
__device__ __forceinline__ double pow_manning(double x, double p) { return pow_any(x, p); }

}  // namespace pihm
