// pihm_gpu_nv_wrms_norm_noalloc: the WRMS norm of the N_Vector operations
// for callers that cannot allocate device memory.
//
// Who cannot allocate: code that runs while a CUDA graph is being captured
// (cudaMalloc is not a stream operation and cannot be recorded), code inside a
// host framework that owns all device memory through its own allocator and
// forbids others from calling cudaMalloc, and integrator callbacks that run
// thousands of times per step, where an allocation per call is a device-wide
// synchronisation (the reference's RHS allocated and freed scratch on every
// call, src/ode_cuda.cu:78-79).  The regular entry point,
// pihm_gpu_nv_wrms_norm, creates a workspace with cudaMalloc/cudaMallocHost
// the first time a stream uses it; this variant allocates nothing.
//
// Its workspace is a file-scope __device__ array (about 64 KiB), which every
// GPU that loads the library holds until the process exits.  All calls share
// it: two calls that overlap on the GPU (different streams, no ordering
// between them) race on it and give wrong results.  The first call on a device
// looks up the array's device address (cudaGetSymbolAddress) with that device
// current; make that first call before any stream capture begins.
#include <cmath>
#include <mutex>

#include "pihm_nvector.h"
#include "nv_reduce.cuh"

namespace pihm_nv {

// ---------------------------------------------------------------------------
// WRMS norm with a library-static workspace (pihm_gpu_nv_wrms_norm_noalloc)
//
// The workspace is a file-scope __device__ array: every GPU that loads this
// library holds it until the process exits.  It keeps one partial sum per
// block (one block per kNoAllocChunk consecutive elements), a ticket and the
// result, so the longest vector it can reduce is
// kNoAllocMaxBlocks * kNoAllocChunk = 33,554,432 elements.
// ---------------------------------------------------------------------------
constexpr int kNoAllocChunk = 4096;        // elements per block
constexpr int kNoAllocMaxBlocks = 8192;    // partial-sum slots
constexpr long long kNoAllocMaxLen = (long long)kNoAllocMaxBlocks * kNoAllocChunk;
// [0, kNoAllocMaxBlocks) partials, then the ticket (as bits of one double)
constexpr int kNoAllocDoubles = kNoAllocMaxBlocks + 32;
static __device__ __align__(256) double g_noalloc_ws[kNoAllocDoubles];

// Same per-element arithmetic and block tree as k_red<R_WSQ>; block b reduces
// the contiguous chunk [b * kNoAllocChunk, (b + 1) * kNoAllocChunk).  The last
// block to finish writes sqrt(sum / n) to `out` (device memory of the caller).
__global__ void __launch_bounds__(kThreads) k_wrms_static(long long n, const double *__restrict__ x,
                                                          const double *__restrict__ w, double *ws,
                                                          double *out) {
  __shared__ Pair sh[kThreads / 32];
  __shared__ bool last;
  unsigned int *ticket = (unsigned int *)(ws + kNoAllocMaxBlocks);
  Pair acc = red_identity<R_WSQ>();
  const long long lo = (long long)blockIdx.x * kNoAllocChunk;
  long long hi = lo + kNoAllocChunk;
  if (hi > n) hi = n;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double p = __dmul_rn(x[i], w[i]);
    acc = red_combine<R_WSQ>(acc, Pair{__dmul_rn(p, p), 0.0});
  }
  acc = red_block<R_WSQ>(acc, sh);
  if (threadIdx.x == 0) {
    ws[blockIdx.x] = acc.v;
    __threadfence();
    last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  Pair v = red_identity<R_WSQ>();
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
    v = red_combine<R_WSQ>(v, Pair{((volatile double *)ws)[b], 0.0});
  v = red_block<R_WSQ>(v, sh);
  if (threadIdx.x == 0) {
    out[0] = sqrt(v.v / (double)n);
    *ticket = 0u;
  }
}

}  // namespace pihm_nv

using namespace pihm_nv;

namespace {
constexpr int kMaxDevices = 64;
double *g_ws_addr[kMaxDevices];
std::mutex g_ws_mu;

// Device address of g_noalloc_ws for the current device (looked up once per
// device, with that device current).
double *workspace_address(int *rc) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    *rc = -2;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_ws_mu);
  if (!g_ws_addr[dev]) {
    double *p = nullptr;
    if (cudaGetSymbolAddress((void **)&p, g_noalloc_ws) != cudaSuccess || !p) {
      *rc = -2;
      return nullptr;
    }
    g_ws_addr[dev] = p;
  }
  *rc = 0;
  return g_ws_addr[dev];
}
}  // namespace

extern "C" int pihm_gpu_nv_wrms_norm_noalloc(const double *x, const double *w, int64_t n, void *stream,
                                             double *result_dev) {
  if (n <= 0 || !x || !w || !result_dev) return -1;
  if (n > kNoAllocMaxLen) return PIHM_GPU_NOALLOC_ERR_TOO_LONG;
  int rc = 0;
  double *ws = workspace_address(&rc);
  if (!ws) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // the ticket must start at zero (a call that failed midway may have left it set)
  if (cudaMemsetAsync(ws + kNoAllocMaxBlocks, 0, sizeof(unsigned int), st) != cudaSuccess) return -2;
  const unsigned grid = (unsigned)((n + kNoAllocChunk - 1) / kNoAllocChunk);
  // cudaLaunchKernel returns this launch's own status, so an error left on
  // the thread by some earlier, unrelated call is neither blamed on this one
  // nor taken from its owner; only an error of this launch is cleared.
  long long n_arg = n;
  void *args[] = {&n_arg, (void *)&x, (void *)&w, &ws, &result_dev};
  const cudaError_t e = cudaLaunchKernel((const void *)k_wrms_static, dim3(grid), dim3(kThreads), args, 0, st);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return -2;
  }
  return 0;
}
