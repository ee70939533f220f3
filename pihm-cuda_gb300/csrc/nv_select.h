// Derived from SUNDIALS 2.7.0 (CVODE 2.9.0). Copyright (c) 2002-2016,
// Lawrence Livermore National Security; produced at the Lawrence Livermore
// National Laboratory (UCRL-CODE-155951). Redistributed under the SUNDIALS
// BSD-3 licence: its full text, conditions and disclaimer are in
// pihm-cuda_gb300/NOTICE.SUNDIALS.
//
// Host- and device-side description of the N_Vector operations shared by the
// single-vector kernels (nvector.cu) and the batch engine (batch.cpp,
// batch_kernels.cu): operation codes, reduction sizes and the serial
// N_Vector's case analysis that picks an operation variant.  The arithmetic
// itself is in nv_ops.cuh.
#pragma once

#ifdef __CUDACC__
#define PIHM_HD __host__ __device__
#else
#define PIHM_HD
#endif

namespace pihm_nv {

constexpr int kThreads = 256;

enum RedOp { R_DOT = 0, R_MAXABS, R_WSQ, R_WSQ_MASK, R_MIN, R_L1, R_INVTEST, R_CONSTR, R_MINQ };

constexpr int kMaxBlocks = 608;  // 4 x 152 SMs: most blocks a reduction uses

// Blocks of kThreads threads a reduction over n entries uses.  The reduction
// order depends only on n, so a norm is identical from run to run and between
// the single-vector and the batched engines.
PIHM_HD inline unsigned red_grid_for(long long n) {
  long long b = (n + 4LL * kThreads - 1) / (4LL * kThreads);
  if (b > kMaxBlocks) b = kMaxBlocks;
  return (unsigned)(b > 0 ? b : 1);
}

enum EwOp {
  EW_LIN = 0,      // a*x + b*y
  EW_LIN1,         // a*x + y
  EW_LIN2,         // a*x - y
  EW_SUM,          // x + y
  EW_DIFF,         // x - y
  EW_SCALESUM,     // a*(x + y)
  EW_SCALEDIFF,    // a*(x - y)
  EW_AXPY,         // y += a*x   (z == y)
  EW_AXPY1,        // y += x
  EW_AXPYM1,       // y -= x
  EW_CONST,        // c
  EW_PROD,         // x*y
  EW_DIV,          // x/y
  EW_SCALE,        // c*x
  EW_COPY,         // x
  EW_NEG,          // -x
  EW_ABS,          // |x|
  EW_INV,          // 1/x
  EW_ADDCONST,     // x + b
  EW_COMPARE,      // |x| >= c ? 1 : 0
  EW_COUNT
};

// Which operands an operation reads (x, y, the old z).
PIHM_HD inline bool ew_reads_x(int op) { return op != EW_CONST; }
PIHM_HD inline bool ew_reads_y(int op) {
  return op == EW_LIN || op == EW_LIN1 || op == EW_LIN2 || op == EW_SUM || op == EW_DIFF ||
         op == EW_SCALESUM || op == EW_SCALEDIFF || op == EW_PROD || op == EW_DIV;
}
PIHM_HD inline bool ew_reads_z(int op) {
  return op == EW_AXPY || op == EW_AXPY1 || op == EW_AXPYM1;
}

// An element-wise call after the serial N_Vector's case analysis: the
// operation, its constants and which handle is its x and its y.
template <class H>
struct EwCall {
  int op;
  double a, b;
  H x, y, z;
};

// N_VLinearSum: z = a*x + b*y, nvector_serial.c:421-506
template <class H>
PIHM_HD EwCall<H> select_linear_sum(double a, H x, double b, H y, H z) {
  if (b == 1.0 && z == y) {
    if (a == 1.0) return {EW_AXPY1, a, b, x, y, z};
    if (a == -1.0) return {EW_AXPYM1, a, b, x, y, z};
    return {EW_AXPY, a, b, x, y, z};
  }
  if (a == 1.0 && z == x) {
    if (b == 1.0) return {EW_AXPY1, b, a, y, x, z};
    if (b == -1.0) return {EW_AXPYM1, b, a, y, x, z};
    return {EW_AXPY, b, a, y, x, z};
  }
  if (a == 1.0 && b == 1.0) return {EW_SUM, a, b, x, y, z};
  bool test;
  if ((test = (a == 1.0 && b == -1.0)) || (a == -1.0 && b == 1.0)) {
    H v1 = test ? y : x, v2 = test ? x : y;
    return {EW_DIFF, 0, 0, v2, v1, z};
  }
  if ((test = (a == 1.0)) || (b == 1.0)) {
    double c = test ? b : a;
    H v1 = test ? y : x, v2 = test ? x : y;
    return {EW_LIN1, c, 0, v1, v2, z};
  }
  if ((test = (a == -1.0)) || (b == -1.0)) {
    double c = test ? b : a;
    H v1 = test ? y : x, v2 = test ? x : y;
    return {EW_LIN2, c, 0, v1, v2, z};
  }
  if (a == b) return {EW_SCALESUM, a, 0, x, y, z};
  if (a == -b) return {EW_SCALEDIFF, a, 0, x, y, z};
  return {EW_LIN, a, b, x, y, z};
}

// N_VScale: z = c*x, nvector_serial.c:559-584
template <class H>
EwCall<H> select_scale(double c, H x, H z) {
  if (z == x) return {EW_SCALE, c, 0, x, x, z};
  if (c == 1.0) return {EW_COPY, 0, 0, x, x, z};
  if (c == -1.0) return {EW_NEG, 0, 0, x, x, z};
  return {EW_SCALE, c, 0, x, x, z};
}

// Coefficients of a linear sum taken from device-resident reduction results
// (slots): the values a GMRES iteration forms on the host from a norm or a
// dot product -- sig = 1/||v|| and 1/sig in the difference-quotient product,
// -h in Gram-Schmidt -- formed here with the same IEEE operations.
enum CoefKind { COEF_HOST = 0, COEF_NEG, COEF_INV, COEF_INV_INV, COEF_NEG_INV_INV };

PIHM_HD inline double coef_div(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

PIHM_HD inline double coef_value(int kind, double value, double s) {
  switch (kind) {
    case COEF_NEG: return -s;
    case COEF_INV: return coef_div(1.0, s);
    case COEF_INV_INV: return coef_div(1.0, coef_div(1.0, s));
    case COEF_NEG_INV_INV: return -coef_div(1.0, coef_div(1.0, s));
    default: return value;
  }
}

}  // namespace pihm_nv
