// IEEE comparisons of doubles evaluated on the integer pipe.
//
// sm_103a retires about two FP64 lanes per clock per SM, and a DSETP holds
// the FP64 pipe as long as a DFMA does, while the integer pipe beside it is
// idle in the right-hand-side kernels.  Each helper returns exactly what the
// C comparison returns, including NaN operands (every ordered comparison is
// false) and signed zeros (-0 == +0), from the bit patterns:
//
//   * a non-negative double (sign bit clear) orders like its bit pattern read
//     as an unsigned integer; +inf is 0x7FF0000000000000 and every larger
//     pattern with the sign clear is a NaN;
//   * a negative double orders in reverse of its pattern; -0 is
//     0x8000000000000000 and every pattern above 0xFFF0000000000000 is a NaN.
//
// The constants c of the *_c helpers must be finite and positive, that of
// gt_nc finite and negative (the callers pass model constants such as the
// depression storage); the *_v helpers take two arbitrary doubles.  Host
// builds use the same code on memcpy'd bits (tests/test_fp64_cmp.py checks
// every helper against the C comparisons on signed zeros, subnormals,
// infinities, NaNs and random values).
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PIHM_CMP_FN __host__ __device__ __forceinline__
#else
#define PIHM_CMP_FN inline
#endif

namespace pihm {
namespace cmp {

constexpr uint64_t kInf = 0x7FF0000000000000ull;
constexpr uint64_t kNegZero = 0x8000000000000000ull;
constexpr uint64_t kNegInf = 0xFFF0000000000000ull;
constexpr uint64_t kMag = 0x7FFFFFFFFFFFFFFFull;

PIHM_CMP_FN uint64_t bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

// x > 0: the patterns 1 .. +inf
PIHM_CMP_FN bool gt0(double x) { return bits(x) - 1u < kInf; }
// x >= 0: +0 .. +inf, or -0
PIHM_CMP_FN bool ge0(double x) {
  const uint64_t b = bits(x);
  return b <= kInf || b == kNegZero;
}
// x < 0: the patterns above -0 up to -inf
PIHM_CMP_FN bool lt0(double x) { return bits(x) - (kNegZero + 1u) < kInf; }
// x <= 0: -0 .. -inf, or +0
PIHM_CMP_FN bool le0(double x) {
  const uint64_t b = bits(x);
  return b - kNegZero <= kInf || b == 0u;
}
// x == 0 (either zero)
PIHM_CMP_FN bool eq0(double x) { return (bits(x) << 1) == 0u; }
// x is a NaN
PIHM_CMP_FN bool isnan_(double x) { return (bits(x) & kMag) > kInf; }

// x > c and x >= c for a finite c > 0: x lies in (c, +inf] or [c, +inf]
PIHM_CMP_FN bool gt_c(double x, double c) {
  const uint64_t cb = bits(c);
  return bits(x) - cb - 1u < kInf - cb;
}
PIHM_CMP_FN bool ge_c(double x, double c) {
  const uint64_t cb = bits(c);
  return bits(x) - cb <= kInf - cb;
}
// x < c and x <= c for a finite c > 0: x in [+0, c) (or [+0, c]), or x
// negative (-0 .. -inf)
PIHM_CMP_FN bool lt_c(double x, double c) {
  const uint64_t b = bits(x);
  return b < bits(c) || b - kNegZero <= kInf;
}
PIHM_CMP_FN bool le_c(double x, double c) {
  const uint64_t b = bits(x);
  return b <= bits(c) || b - kNegZero <= kInf;
}

// x > c for a finite c < 0: x non-negative (+0 .. +inf, or -0), or negative
// with a smaller magnitude than c
PIHM_CMP_FN bool gt_nc(double x, double c) {
  const uint64_t b = bits(x);
  return b <= kInf || b - kNegZero < bits(c) - kNegZero;
}

// Two arbitrary doubles.  key() maps a non-NaN double to a signed integer in
// the double's order, with both zeros on 0: non-negative patterns stay, a
// negative one becomes minus its magnitude.
PIHM_CMP_FN int64_t key(uint64_t b) {
  const int64_t mag = (int64_t)(b & kMag);
  return (b >> 63) ? -mag : mag;
}
PIHM_CMP_FN bool ordered(uint64_t a, uint64_t b) { return (a & kMag) <= kInf && (b & kMag) <= kInf; }
PIHM_CMP_FN bool lt_v(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  return ordered(a, b) && key(a) < key(b);
}
PIHM_CMP_FN bool le_v(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  return ordered(a, b) && key(a) <= key(b);
}
PIHM_CMP_FN bool gt_v(double x, double y) { return lt_v(y, x); }
PIHM_CMP_FN bool ge_v(double x, double y) { return le_v(y, x); }

// |x| < c for a finite c > 0
PIHM_CMP_FN bool abs_lt_c(double x, double c) { return (bits(x) & kMag) < bits(c); }

PIHM_CMP_FN double from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// -x when neg is true, else x: the C unary minus flips the sign bit and
// nothing else, so it too stays off the FP64 pipe
PIHM_CMP_FN double neg_if(double x, bool neg) { return from_bits(bits(x) ^ ((uint64_t)neg << 63)); }

}  // namespace cmp
}  // namespace pihm
