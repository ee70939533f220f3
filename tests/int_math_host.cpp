// Host build of the integer-pipe logarithm / exponential / power
// (pihm-cuda_gb300/csrc/int_math.cuh) for the CPU tests: the arithmetic is
// integer, so these functions return the bits the GPU kernels compute.
#include <cstdint>

#include "int_math.cuh"

extern "C" {

// out[i] = x[i]^y[i] on the integer path; ok[i] = 0 where it declines
void im_pow(const double *x, const double *y, double *out, int32_t *ok, int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    double r = 0.0;
    ok[i] = pihm::im::pow_i(x[i], y[i], r) ? 1 : 0;
    out[i] = r;
  }
}

// 1024 log2 x as (k, w 2^-53)
void im_log2k(const double *x, int32_t *k, int64_t *w, int32_t *ok, int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    int kk = 0;
    int64_t ww = 0;
    ok[i] = pihm::im::log2k(x[i], kk, ww) ? 1 : 0;
    k[i] = kk;
    w[i] = ww;
  }
}

// 2^(t / 1024) for t = tn + tf 2^-64
void im_exp2k(const int64_t *tn, const int64_t *tf, double *out, int64_t n) {
  for (int64_t i = 0; i < n; i++) out[i] = pihm::im::exp2k(pihm::im::TVal{tn[i], tf[i]});
}
}

extern "C" {
// q[i] = a[i] / b[i] on the integer path; ok[i] = 0 where it declines
void im_div(const double *a, const double *b, double *q, int32_t *ok, int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    double r = 0.0;
    ok[i] = pihm::im::div_i(a[i], b[i], r) ? 1 : 0;
    q[i] = r;
  }
}

// r[i] = sqrt(x[i]) on the integer path; ok[i] = 0 where it declines
void im_sqrt(const double *x, double *r, int32_t *ok, int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    double v = 0.0;
    ok[i] = pihm::im::sqrt_i(x[i], v) ? 1 : 0;
    r[i] = v;
  }
}
}

extern "C" {
// out[i] = fl(1/x[i])^y[i] through the logarithm of x[i] (log2k_recip);
// ok[i] = 0 where a step declines
void im_pow_recip(const double *x, const double *y, double *out, int32_t *ok, int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    double q = 0.0, r = 0.0;
    int k = 0, kq = 0;
    int64_t w = 0, wq = 0;
    pihm::im::TVal t{0, 0};
    const bool good = pihm::im::div_i(1.0, x[i], q) && pihm::im::log2k(x[i], k, w) &&
                      pihm::im::log2k_recip(x[i], q, k, w, kq, wq) && pihm::im::mul_t(y[i], kq, wq, t);
    if (good) r = pihm::im::exp2k(t);
    ok[i] = good ? 1 : 0;
    out[i] = r;
  }
}
}
