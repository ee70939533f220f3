// FP64 logarithm, exponential and power evaluated on the integer pipe.
//
// GB300 retires 2 FP64 lanes per clock per SM but 64 integer lanes: a
// warp-wide FP64 instruction holds the SM's FP64 pipe for 16 cycles, an
// integer instruction for half a cycle.  The right-hand side's powers
// (van Genuchten's KrFunc and Psi, Manning's h^0.6666667) therefore run
// here in 64-bit fixed point with 128-bit products, and only their inputs
// and outputs are doubles.
//
// Representation: a base-2 logarithm is carried in units of 1/1024 ("t
// units"): x^y = 2^(t/1024) with t = y * 1024 log2 x.
//
//   log2k(x):  x = 2^k m, m in [1, 2), M = 2^52 m (the 53-bit mantissa);
//              i = the top 10 fraction bits of m; F_i = round(4096/c_i)/4096,
//              c_i = 1 + (i + 1/2)/1024 (kImLogF); r = m F_i - 1 is
//              M F_i - 2^64 in units of 2^-64, exact in wrapping 64-bit
//              arithmetic (|r| < 2^-10.4); then
//                1024 log2 x = 1024 k + H_i + (1024/ln 2) log1p(r),
//              H_i = -1024 log2 F_i (kImLogH), log1p(r) = r + r^2 T(r),
//              T = -1/2 + r/3 - r^2/4 + r^3/5 (the next term is below
//              2^-62).  Returned as k and w = (H_i + (1024/ln 2) log1p r)
//              in units of 2^-53 (|w| < 2^63).
//   mul_t:     t = y (1024 k + w 2^-53), the 53 x 64-bit product exact in
//              128 bits, kept as N = round(t) and f = t - N in units of
//              2^-64 (|t| < 1.5 * 2^16).
//   exp2k(t):  j = N mod 1024, q = floor(N / 1024), r = f ln2 / 1024
//              (|r| <= ln2/2048); 2^(t/1024) = 2^q T_j (1 + expm1 r),
//              T_j = 2^(j/1024) (kImExpT, units of 2^-63), expm1(r) = r +
//              r^2 E(r), E = 1/2 + r/6 + r^2/24 + r^3/120 (the next term
//              is below 2^-78); the 64-bit mantissa is rounded to 53 bits.
//
// These are the table-driven reductions of P. T. P. Tang ("Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2) 1989; "... of the logarithm function ...",
// ACM TOMS 16(4) 1990) carried out in fixed point.  Error budget, relative
// to the result of a power: w's roundings times |y| (|y| 2^-63.5), the
// truncation of t (2^-64 t units, 2^-74.5), the exponential's fixed-point
// error (about 2^-62), then the final rounding to 53 bits: 0.5 ulp plus a
// few thousandths of an ulp, so the result is the correctly rounded power
// except within that distance of a rounding boundary.  tests/test_int_math.py checks the bound against 60-digit
// references on the CPU build of this file (the arithmetic is integer, so
// the host and the GPU give the same bits; the GPU test checks that).
//
// Ranges: log2k wants x positive and normal with |k| <= 126; mul_t wants y
// normal with exponent in [-20, 29] and |t| < 1.5 * 2^16 (a power in about
// (1e-29, 8e28)); each returns false otherwise and the caller takes another
// path.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define PIHM_IM_FN __device__ __forceinline__
#define PIHM_IM_TABLE static __device__ const
#define PIHM_IM_LD(v) __ldg(&(v))
#else
#define PIHM_IM_FN static inline
#define PIHM_IM_TABLE static const
#define PIHM_IM_LD(v) (v)
#endif

#include "int_tables.h"

namespace pihm {
namespace im {

typedef __int128 i128;

PIHM_IM_FN int64_t mulhi(int64_t a, int64_t b) {
#if defined(__CUDA_ARCH__)
  return __mul64hi(a, b);
#else
  return (int64_t)(((i128)a * b) >> 64);
#endif
}

// the high half of a 32 x 32-bit signed product (one instruction on the GPU)
PIHM_IM_FN int32_t mulhi32(int32_t a, int32_t b) {
#if defined(__CUDA_ARCH__)
  return __mulhi(a, b);
#else
  return (int32_t)(((int64_t)a * b) >> 32);
#endif
}

// the polynomial constants (2^62 units) in 2^31 units, rounded, for the
// 32-bit Horner steps
#define PIHM_IM_Q31(c62) ((int32_t)(((c62) + (1ll << 30)) >> 31))
constexpr int32_t kImL5q = PIHM_IM_Q31(kImL5), kImL4q = PIHM_IM_Q31(kImL4);
constexpr int32_t kImE120q = PIHM_IM_Q31(kImE120), kImE24q = PIHM_IM_Q31(kImE24), kImE6q = PIHM_IM_Q31(kImE6);
#undef PIHM_IM_Q31

PIHM_IM_FN uint64_t dbits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

PIHM_IM_FN double bitsd(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

constexpr uint64_t kFrac = 0xFFFFFFFFFFFFFull;
constexpr int64_t kNMax = 3 * (1ll << 15);  // |t| < 1.5 * 2^16: a normal result

// A value t in t units (1024 log2 of a power) as round(t) and the rest in
// units of 2^-64: t = n + f 2^-64, f in [-2^63, 2^63).
struct TVal {
  int64_t n;
  int64_t f;
};

// 1024 log2 x = 1024 k + w 2^-53, for x positive and normal with |k| <= 126.
PIHM_IM_FN bool log2k(double x, int &k, int64_t &w) {
  const uint64_t xb = dbits(x);
  const unsigned top = (unsigned)(xb >> 52);  // sign and biased exponent
  if (top - 897u >= 253u) return false;       // not positive, or |k| > 126
  k = (int)top - 1023;
  const uint64_t M = (xb & kFrac) | (1ull << 52);
  const unsigned i = (unsigned)(xb >> 42) & 1023u;
  // r 2^64 = M F_i - 2^64: the low 64 bits of the product, read as signed
  const int64_t R = (int64_t)(M * (uint64_t)PIHM_IM_LD(kImLogF[i]));
  const int64_t r = R * 256;  // r 2^72, |r 2^72| < 2^61.6
  // T(r) 2^62 by Horner's rule; its first step, L4 + r L5, needs about 23
  // bits (the later products scale its error by |r| < 2^-10.4 twice more and
  // by r^2), so it runs in 32-bit fixed point (2^31 units)
  const int32_t r32 = (int32_t)((r + (1ll << 39)) >> 40);  // r 2^32
  int64_t h = (int64_t)(kImL4q + mulhi32(kImL5q, r32)) << 31;
  h = kImL3 + (mulhi(h, r) >> 8);
  h = kImL2 + (mulhi(h, r) >> 8);
  const int64_t r2 = mulhi(r, r);               // r^2 2^80
  const int64_t lp = r + (mulhi(r2, h) >> 6);   // log1p(r) 2^72
  w = PIHM_IM_LD(kImLogH[i]) + ((mulhi(lp, kImK) + 64) >> 7);
  return true;
}

// t = y (1024 k + w 2^-53) for y normal with exponent in [-20, 29] and
// |t| < 1.5 * 2^16; false otherwise
PIHM_IM_FN bool mul_t(double y, int k, int64_t w, TVal &t) {
  const uint64_t yb = dbits(y);
  const int ey = (int)((yb >> 52) & 2047u) - 1023;
  if ((unsigned)(ey + 20) >= 50u) return false;
  const int64_t my = (int64_t)((yb & kFrac) | (1ull << 52));
  // Q = My (k 2^63 + w) exactly (|My k| < 2^60, |My w| < 2^116); y =
  // My 2^(ey - 52) and 1024 k + w 2^-53 = (k 2^63 + w) 2^-53, so
  // t 2^64 = Q 2^(ey - 41), a right shift by 12..61
  i128 Q = (i128)my * w + ((i128)(my * k) << 63);
  Q >>= 41 - ey;
  if (yb >> 63) Q = -Q;
  const int64_t hi = (int64_t)(Q >> 64);
  const uint64_t lo = (uint64_t)Q;
  t.n = hi + (int64_t)(lo >> 63);  // round(t)
  t.f = (int64_t)lo;               // t - round(t), units of 2^-64
  return t.n < kNMax && t.n > -kNMax;
}

// 2^(t/1024) for |t| < 1.5 * 2^16: a normal double
PIHM_IM_FN double exp2k(TVal t) {
  const unsigned j = (unsigned)t.n & 1023u;
  int q = (int)(t.n >> 10);
  const int64_t r = mulhi(t.f, kImLn2) >> 1;   // f ln2 / 1024 in units of 2^-72
  // E(r) 2^62 by Horner's rule; E6 + r (E24 + r E120) needs about 30 bits
  // (expm1 = r + r^2 E with |r| <= 2^-11.5), so its two steps run in 32-bit
  // fixed point (2^31 units, error below 2^-30.9)
  const int32_t r32 = (int32_t)((r + (1ll << 39)) >> 40);  // r 2^32
  int32_t h31 = kImE24q + mulhi32(kImE120q, r32);
  h31 = kImE6q + mulhi32(h31, r32);
  const int64_t h = kImE2 + (mulhi((int64_t)h31 << 31, r) >> 8);
  const int64_t r2 = mulhi(r, r);              // r^2 2^80
  const int64_t e = r + (mulhi(r2, h) >> 6);   // expm1(r) 2^72
  const uint64_t T = PIHM_IM_LD(kImExpT[j]);   // 2^(j/1024) 2^63
  uint64_t res = T + (uint64_t)(mulhi((int64_t)(T >> 1), e) >> 7);  // 2^63 T (1 + e)
  if (!(res >> 63)) {  // below 1 (j = 0, e < 0)
    res <<= 1;
    q -= 1;
  }
  uint64_t mant = (res >> 11) + ((res >> 10) & 1u);
  if (mant >> 53) {
    mant >>= 1;
    q += 1;
  }
  return bitsd(((uint64_t)(q + 1023) << 52) + (mant & kFrac));
}

// 1024 log2 q for q = fl(1/x), the correctly rounded reciprocal of x, from
// x's own (k, w): q x = 1 + d exactly, with d = D 2^(ex + eq - 104) and D
// the low 64 bits of the product of the two 53-bit mantissas (the product
// is 2^(104 - ex - eq) + D, |D| <= 2^52), so 1024 log2 q = -(1024 k + w
// 2^-53) + (1024/ln 2) d, the d^2 term being below 2^-100.  Saves the
// logarithm of q where x^y and (1/x)^y are both wanted.  False unless q is
// positive and normal with q x within 2^-51 of 1.
PIHM_IM_FN bool log2k_recip(double x, double q, int k, int64_t w, int &kq, int64_t &wq) {
  const uint64_t xb = dbits(x), qb = dbits(q);
  const int ex = (int)((xb >> 52) & 2047u), eq = (int)((qb >> 52) & 2047u);
  if (eq - 1u >= 2046u || (qb >> 63)) return false;
  const int s = 104 - (ex - 1023) - (eq - 1023);  // q x = (Mx Mq) 2^-s
  if (s != 104 && s != 105) return false;
  const uint64_t Mx = (xb & kFrac) | (1ull << 52), Mq = (qb & kFrac) | (1ull << 52);
  const int64_t D = (int64_t)(Mx * Mq);  // Mx Mq - 2^s (2^s vanishes mod 2^64)
  if (D > (1ll << 53) || D < -(1ll << 53)) return false;  // |D| <= 2^52 for a correctly rounded q
  // (1024/ln 2) D 2^-s in units of 2^-53: mulhi(D 2^8, kImK) is
  // (1024/ln 2) D 2^-4 (kImK = (1024/ln 2) 2^52), rounded by 2^(57 - s)
  const int sh = s - 57;  // 47 or 48
  const int64_t c = (mulhi(D * 256, kImK) + (1ll << (sh - 1))) >> sh;
  kq = -k;
  wq = -w + c;
  return true;
}

// x^y on the integer path; false when x or y is outside its ranges.  +0 to
// a positive power is +0 (C99 F.9.4.4), which a full soil column produces
// (1 - satn^m == 0).
PIHM_IM_FN bool pow_i(double x, double y, double &out) {
  int k;
  int64_t w;
  TVal t;
  if (dbits(x) == 0 && dbits(y) - 1u < 0x7FF0000000000000ull) {
    out = 0.0;
    return true;
  }
  if (!log2k(x, k, w) || !mul_t(y, k, w, t)) return false;
  out = exp2k(t);
  return true;
}


// ---------------------------------------------------------------------------
// Division and square root, correctly rounded (round to nearest even), on
// the integer pipe.  A single-precision reciprocal (or reciprocal square
// root) of the leading 24 bits seeds two Newton steps in 64-bit fixed point
// (relative error about 2^-60), which give the 53-bit result to within a
// small fraction of a unit; an exact 128-bit comparison against the
// rounding midpoint then decides the last bit.  The results are therefore
// the IEEE quotient and root bit for bit, whatever the seed's own rounding
// (the host build seeds with a correctly rounded float, the GPU with
// rcp.approx / rsqrt.approx).  A zero dividend over a normal divisor and the
// root of a zero give the signed zero; other operands or results outside the
// normal range are declined (false) and the caller uses the FP64
// instruction.
// ---------------------------------------------------------------------------

PIHM_IM_FN float rcp_seed(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / x;
#endif
}

PIHM_IM_FN float rsqrt_seed(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / std::sqrt(x);
#endif
}

PIHM_IM_FN uint32_t umulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

PIHM_IM_FN uint64_t umulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

PIHM_IM_FN uint32_t fbits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

PIHM_IM_FN float bitsf(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// a seed r (a float in (0.25, 1]) as r 2^63, at most 2^63 - 1
PIHM_IM_FN uint64_t seed_fixed(float r) {
  const uint32_t rb = fbits(r);
  const int ex = (int)(rb >> 23) - 127;  // -2 or -1 ... 0
  const uint64_t m = (uint64_t)((rb & 0x7FFFFFu) | 0x800000u);  // 2^23 (1 + f)
  const uint64_t v = m << (40 + ex);
  return v >> 63 ? 0x7FFFFFFFFFFFFFFFull : v;
}

// q = a / b for normal (or zero) a and normal b with a normal quotient
PIHM_IM_FN bool div_i(double a, double b, double &q) {
  const uint64_t ab = dbits(a), bb = dbits(b);
  const unsigned ea = (unsigned)(ab >> 52) & 2047u, eb = (unsigned)(bb >> 52) & 2047u;
  if (eb - 1u >= 2046u) return false;  // zero, subnormal, inf or nan divisor
  if (ea - 1u >= 2046u) {
    if (ab << 1) return false;  // subnormal, inf or nan dividend
    q = bitsd((ab ^ bb) & (1ull << 63));
    return true;
  }
  const uint64_t Ma = (ab & kFrac) | (1ull << 52), Mb = (bb & kFrac) | (1ull << 52);
  // 1/mb, mb = Mb 2^-52 in [1, 2): R = r 2^63.  Newton's step r <- r (1 + e),
  // e = 1 - mb r, never overshoots 1/mb in exact arithmetic; the first step
  // (from the seed's 2^-23 to about 2^-30) runs in 32-bit fixed point, the
  // second (to about 2^-60) in 64-bit
  const uint64_t R0 = seed_fixed(rcp_seed(bitsf(0x3F800000u | (uint32_t)((Mb & kFrac) >> 29))));
  const int32_t R32 = (int32_t)(R0 >> 32);                  // r 2^31 (< 2^31)
  const int32_t e32 = (int32_t)((1u << 30) - umulhi32((uint32_t)(Mb >> 21), (uint32_t)R32));  // e 2^30
  uint64_t R = (uint64_t)(R32 + mulhi32(R32, e32) * 4) << 32;
  {
    const uint64_t B = Mb << 11;  // mb 2^63
    // e = 1 - mb r in units of 2^-62
    const int64_t e = (int64_t)((1ull << 62) - umulhi(B, R));
    R = (uint64_t)((int64_t)R + mulhi((int64_t)R, e) * 4);
  }
  // ma r 2^62 in (2^61, 2^63)
  const uint64_t Q = umulhi(Ma << 11, R);
  int ex = (int)ea - (int)eb;
  uint64_t q0;
  int s;  // quotient bits: a / b = Ma 2^s / Mb in units of the result's ulp
  if (Q >> 62) {
    q0 = Q >> 10;
    s = 52;
  } else {
    q0 = Q >> 9;
    s = 53;
    ex -= 1;
  }
  // the exact quotient against the midpoint q0 + 1/2:
  //   2 Ma 2^s  vs  (2 q0 + 1) Mb
  const i128 lhs = (i128)Ma << (s + 1);
  const i128 rhs = (i128)(2 * q0 + 1) * (i128)Mb;
  uint64_t mant = q0 + ((lhs > rhs) || (lhs == rhs && (q0 & 1u)));
  if (mant >> 53) {
    mant >>= 1;
    ex += 1;
  }
  const int eq = ex + 1023;
  if (eq < 1 || eq > 2046) return false;
  q = bitsd((((ab ^ bb) >> 63) << 63) | ((uint64_t)eq << 52) | (mant & kFrac));
  return true;
}

// sqrt(x) for positive normal x, or a zero
PIHM_IM_FN bool sqrt_i(double x, double &r) {
  const uint64_t xb = dbits(x);
  if ((xb << 1) == 0) {  // sqrt(+-0) = +-0
    r = x;
    return true;
  }
  const unsigned top = (unsigned)(xb >> 52);  // sign and biased exponent
  if (top - 1u >= 2046u) return false;       // not positive and normal
  const int ex = (int)top - 1023;
  const int odd = ex & 1;
  // x = m 2^(ex - odd), m = M 2^-52 in [1, 4)
  const uint64_t M = ((xb & kFrac) | (1ull << 52)) << odd;
  const float mf = bitsf((uint32_t)(0x3F800000u + ((uint32_t)odd << 23)) | (uint32_t)((xb & kFrac) >> 29));
  // 1/sqrt(m) by Newton's step y <- y (1 + e / 2), e = 1 - m y^2, which
  // never overshoots in exact arithmetic: the first step (from the seed's
  // 2^-23 to about 2^-29) in 32-bit fixed point, the second in 64-bit
  const int32_t Y32 = (int32_t)(seed_fixed(rsqrt_seed(mf)) >> 32);  // y 2^31 (y < 1)
  const uint32_t y2_32 = (uint32_t)(((uint64_t)Y32 * (uint64_t)Y32) >> 30);  // y^2 2^32
  const int32_t e32 = (int32_t)((1u << 30) - umulhi32((uint32_t)(M >> 22), y2_32));  // e 2^30
  uint64_t Y = (uint64_t)(Y32 + mulhi32(Y32, e32) * 2) << 32;  // y 2^63
  const uint64_t Mm = M << 10;  // m 2^62
  {
    // e = 1 - m y^2 in units of 2^-60
    const uint64_t y2 = umulhi(Y, Y);  // y^2 2^62
    const int64_t e = (int64_t)((1ull << 60) - umulhi(Mm, y2));
    Y = (uint64_t)((int64_t)Y + mulhi((int64_t)Y, e) * 8);
  }
  // sqrt(m) 2^61 = m y 2^61, then 53 bits
  const uint64_t S = umulhi(Mm, Y);
  const uint64_t s0 = S >> 9;
  // round(sqrt(M 2^52)): (2 s0 + 1)^2 against 4 M 2^52 (never equal)
  const unsigned __int128 lhs = (unsigned __int128)M << 54;
  const unsigned __int128 rhs = (unsigned __int128)(2 * s0 + 1) * (2 * s0 + 1);
  uint64_t mant = s0 + (lhs > rhs);
  int er = (ex - odd) / 2;
  if (mant >> 53) {
    mant >>= 1;
    er += 1;
  }
  r = bitsd(((uint64_t)(er + 1023) << 52) | (mant & kFrac));
  return true;
}

}  // namespace im
}  // namespace pihm
