// Derived from SUNDIALS 2.7.0 (CVODE 2.9.0). Copyright (c) 2002-2016,
// Lawrence Livermore National Security; produced at the Lawrence Livermore
// National Laboratory (UCRL-CODE-155951). Redistributed under the SUNDIALS
// BSD-3 licence: its full text, conditions and disclaimer are in
// pihm-cuda_gb300/NOTICE.SUNDIALS.
//
// Arithmetic of the N_Vector operations, shared by the single-vector kernels
// (nvector.cu) and the batch engine's program kernel (batch_kernels.cu) so
// that both produce bit-identical vectors and norms.
//
// Element-wise operations use __dmul_rn/__dadd_rn so the compiler cannot fuse
// a multiply and an add: every element equals what the serial N_Vector
// computes (cvode/src/nvec_ser/nvector_serial.c:421-1060), including its
// special cases (a == 1, b == -1, a == b, ...) which change the rounding.
//
// Divisions and reciprocals run on the integer pipe (int_math.cuh: a float
// seed, two fixed-point Newton steps and an exact midpoint test, the IEEE
// quotient bit for bit) with the FP64 instruction for zeros, subnormals,
// infinities and NaN: GB300 retires 2 FP64 lanes per clock per SM, and an
// FP64 division costs about as much pipe time as fifteen additions.
#pragma once

#include <cmath>

#include "int_math.cuh"
#include "nv_reduce.cuh"
#include "nv_select.h"

namespace pihm_nv {

// The FP64 division for operands outside the integer path's ranges, out of
// line: inlined behind the test it would be predicated, and every warp
// would issue it.
static __device__ __noinline__ double div_rn_slow(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ double div_rn(double a, double b) {
  double q;
  return pihm::im::div_i(a, b, q) ? q : div_rn_slow(a, b);
}

// z_i = OP(a, b, x_i, y_i, z_i)
template <int OP>
__device__ __forceinline__ double ew_eval(double a, double b, double x, double y, double z) {
  if (OP == EW_LIN) return __dadd_rn(__dmul_rn(a, x), __dmul_rn(b, y));
  if (OP == EW_LIN1) return __dadd_rn(__dmul_rn(a, x), y);
  if (OP == EW_LIN2) return __dsub_rn(__dmul_rn(a, x), y);
  if (OP == EW_SUM) return __dadd_rn(x, y);
  if (OP == EW_DIFF) return __dsub_rn(x, y);
  if (OP == EW_SCALESUM) return __dmul_rn(a, __dadd_rn(x, y));
  if (OP == EW_SCALEDIFF) return __dmul_rn(a, __dsub_rn(x, y));
  if (OP == EW_AXPY) return __dadd_rn(z, __dmul_rn(a, x));
  if (OP == EW_AXPY1) return __dadd_rn(z, x);
  if (OP == EW_AXPYM1) return __dsub_rn(z, x);
  if (OP == EW_CONST) return a;
  if (OP == EW_PROD) return __dmul_rn(x, y);
  if (OP == EW_DIV) return div_rn(x, y);
  if (OP == EW_SCALE) return __dmul_rn(a, x);
  if (OP == EW_COPY) return x;
  if (OP == EW_NEG) return -x;
  if (OP == EW_ABS) return fabs(x);
  if (OP == EW_INV) return div_rn(1.0, x);
  if (OP == EW_ADDCONST) return __dadd_rn(x, b);
  return (fabs(x) >= a) ? 1.0 : 0.0;
}

// Per-entry term of a reduction
template <int OP>
__device__ __forceinline__ Pair red_term(double x, double y) {
  Pair t = red_identity<OP>();
  if (OP == R_DOT) t.v = __dmul_rn(x, y);
  else if (OP == R_MAXABS) t.v = fabs(x);
  else if (OP == R_WSQ) {
    const double p = __dmul_rn(x, y);
    t.v = __dmul_rn(p, p);
  } else if (OP == R_MIN) t.v = x;
  else if (OP == R_L1) t.v = fabs(x);
  return t;
}

}  // namespace pihm_nv
