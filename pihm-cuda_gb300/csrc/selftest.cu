// Diagnostic entry points: the power of the right-hand-side kernels (pow_any)
// next to CUDA's pow, and the Manning-exponent power, element by element, so
// tests can measure their error.
#include <cstdint>

#include "fp64_math.cuh"

namespace {
__global__ void k_pow_pair(const double *x, const double *y, double *fast, double *ref, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fast[i] = pihm::pow_any(x[i], y[i]);
  if (ref) ref[i] = pow(x[i], y[i]);
}

__global__ void k_pow_manning(const double *x, int river, double *out, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = river ? pihm::pow_manning(x[i], pihm::kManningRiv) : pihm::pow_manning(x[i], pihm::kManningSurf);
}
}  // namespace

extern "C" int pihm_gpu_selftest_pow(const double *x, const double *y, double *fast, double *cuda_pow,
                                     int64_t n, void *stream) {
  if (n <= 0 || !x || !y || !fast) return -1;
  k_pow_pair<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, y, fast, cuda_pow, n);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

extern "C" int pihm_gpu_selftest_pow_manning(const double *x, int river, double *out, int64_t n,
                                             void *stream) {
  if (n <= 0 || !x || !out) return -1;
  k_pow_manning<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, river, out, n);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

namespace {
__global__ void k_pow_int(const double *x, const double *y, double *out, int32_t *ok, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double r = 0.0;
  ok[i] = pihm::im::pow_i(x[i], y[i], r) ? 1 : 0;
  out[i] = r;
}
}  // namespace

// The integer-pipe power (int_math.cuh) alone, element by element: out[i] =
// x[i]^y[i] where ok[i] = 1, ok[i] = 0 where x or y is outside its ranges.
extern "C" int pihm_gpu_selftest_pow_int(const double *x, const double *y, double *out, int32_t *ok,
                                         int64_t n, void *stream) {
  if (n <= 0 || !x || !y || !out || !ok) return -1;
  k_pow_int<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, y, out, ok, n);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

namespace {
__global__ void k_div_sqrt_int(const double *a, const double *b, double *q, double *r, int32_t *ok,
                               long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double qq = 0.0, rr = 0.0;
  const bool okq = pihm::im::div_i(a[i], b[i], qq);
  const bool okr = pihm::im::sqrt_i(a[i], rr);
  q[i] = qq;
  r[i] = rr;
  ok[i] = (okq ? 1 : 0) | (okr ? 2 : 0);
}
}  // namespace

// The integer-pipe division and square root alone: q[i] = a[i] / b[i] and
// r[i] = sqrt(a[i]); bit 0 of ok[i] set where the division took the integer
// path, bit 1 where the square root did.
extern "C" int pihm_gpu_selftest_div_sqrt_int(const double *a, const double *b, double *q, double *r,
                                              int32_t *ok, int64_t n, void *stream) {
  if (n <= 0 || !a || !b || !q || !r || !ok) return -1;
  k_div_sqrt_int<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a, b, q, r, ok, n);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
