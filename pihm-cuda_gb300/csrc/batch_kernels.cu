// The batch engine's program kernel (batch_device.h).
#include "batch_device.h"
#include "nv_ops.cuh"

namespace pihm {
namespace batch {

using namespace pihm_nv;

namespace {

// Position of entry j of a watershed's state vector in the arena-wide
// right-hand-side staging vector, which has the single-watershed layout
// [surf | unsat | gw] over ne_cap elements and [stage | rivgw] over nr_cap
// segments.
__device__ __forceinline__ long long stage_pos(const SysInfo &s, long long j, long long ne_cap,
                                               long long nr_cap) {
  const long long ne = s.ne;
  if (j < 3 * ne) {
    const long long p = (j >= ne) + (j >= 2 * ne);
    return p * ne_cap + s.eoff + (j - p * ne);
  }
  const long long jr = j - 3 * ne;
  const long long q = (jr >= s.nr);
  return 3 * ne_cap + q * nr_cap + s.roff + (jr - q * s.nr);
}

// A thread works on kU grid-stride iterations together, so that the loads of
// kU entries are in flight at once; the reduction still accumulates them in
// grid-stride order, so every kU gives the same bits.  The batch engine's
// tuner picks kU (1, 2 or 4) by timing.

// z = OP(a, b, x, y, z) for a run-time operation code
__device__ __forceinline__ double ew_eval_rt(int op, double a, double b, double x, double y, double z) {
  switch (op) {
    case EW_LIN: return ew_eval<EW_LIN>(a, b, x, y, z);
    case EW_LIN1: return ew_eval<EW_LIN1>(a, b, x, y, z);
    case EW_LIN2: return ew_eval<EW_LIN2>(a, b, x, y, z);
    case EW_SUM: return ew_eval<EW_SUM>(a, b, x, y, z);
    case EW_DIFF: return ew_eval<EW_DIFF>(a, b, x, y, z);
    case EW_SCALESUM: return ew_eval<EW_SCALESUM>(a, b, x, y, z);
    case EW_SCALEDIFF: return ew_eval<EW_SCALEDIFF>(a, b, x, y, z);
    case EW_AXPY: return ew_eval<EW_AXPY>(a, b, x, y, z);
    case EW_AXPY1: return ew_eval<EW_AXPY1>(a, b, x, y, z);
    case EW_AXPYM1: return ew_eval<EW_AXPYM1>(a, b, x, y, z);
    case EW_CONST: return ew_eval<EW_CONST>(a, b, x, y, z);
    case EW_PROD: return ew_eval<EW_PROD>(a, b, x, y, z);
    case EW_DIV: return ew_eval<EW_DIV>(a, b, x, y, z);
    case EW_SCALE: return ew_eval<EW_SCALE>(a, b, x, y, z);
    case EW_COPY: return ew_eval<EW_COPY>(a, b, x, y, z);
    case EW_NEG: return ew_eval<EW_NEG>(a, b, x, y, z);
    case EW_ABS: return ew_eval<EW_ABS>(a, b, x, y, z);
    case EW_INV: return ew_eval<EW_INV>(a, b, x, y, z);
    case EW_ADDCONST: return ew_eval<EW_ADDCONST>(a, b, x, y, z);
    default: return ew_eval<EW_COMPARE>(a, b, x, y, z);
  }
}

// Apply one operation to the entries j[0..nu).  base points at the
// watershed's entry 0 in vector slot 0; slots are vs entries apart.
template <int kU>
__device__ __forceinline__ void exec_op(const Op &o, const DeviceArena &A, const SysInfo &S, double *base,
                                        long long vs, const long long (&j)[kU], int nu) {
  if (o.code < EW_COUNT) {
    const bool rx = ew_reads_x(o.code), ry = ew_reads_y(o.code), rz = ew_reads_z(o.code);
    const double *x = base + o.x * vs, *y = base + o.y * vs;
    double *z = base + o.z * vs;
    double xv[kU], yv[kU], zv[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      xv[u] = (u < nu && rx) ? x[j[u]] : 0.0;
      yv[u] = (u < nu && ry) ? y[j[u]] : 0.0;
      zv[u] = (u < nu && rz) ? z[j[u]] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kU; u++)
      if (u < nu) z[j[u]] = ew_eval_rt(o.code, o.a, o.b, xv[u], yv[u], zv[u]);
    return;
  }
  switch (o.code) {
    case OP_STAGE_IN: {
      double v[kU];
#pragma unroll
      for (int u = 0; u < kU; u++)
        if (u < nu) v[u] = base[o.x * vs + j[u]];
#pragma unroll
      for (int u = 0; u < kU; u++)
        if (u < nu) A.rhs_in[stage_pos(S, j[u], A.m.ne, A.m.nr)] = v[u];
      break;
    }
    case OP_STAGE_OUT: {
      double v[kU];
#pragma unroll
      for (int u = 0; u < kU; u++)
        if (u < nu) v[u] = A.rhs_out[stage_pos(S, j[u], A.m.ne, A.m.nr)];
#pragma unroll
      for (int u = 0; u < kU; u++)
        if (u < nu) base[o.z * vs + j[u]] = v[u];
      break;
    }
    case OP_FORCING:
#pragma unroll
      for (int u = 0; u < kU; u++)
        if (u < nu && j[u] < S.ne) {
          const long long g = S.eoff + j[u];
          ((double *)A.m.pcpdrp)[g] = o.a;
          ((double *)A.m.edir)[g] = o.b;
          ((double *)A.m.ett)[g] = o.c;
        }
      break;
    case OP_WS0:
#pragma unroll
      for (int u = 0; u < kU; u++)
        if (u < nu && j[u] < S.ne) ((double *)A.m.ws0_surf)[S.eoff + j[u]] = base[o.x * vs + j[u]];
      break;
    case OP_RECORD:
      if (j[0] == 0) A.rec[S.rec_off + o.i0] = A.m.rivflow[(long long)DOWN_CHANL2CHANL * A.m.nr + S.roff + o.i1];
      break;
    default: break;
  }
}

// One block of one watershed's program: the element-wise operations over the
// block's grid-strided entries, then (RED >= 0) the reduction, combined
// exactly as the single-vector reduction kernel combines it.
template <int kU, int RED>
__device__ void run_block(const DeviceArena &A, const RoundSys &R, const SysInfo &S, const Op *prog, int b) {
  __shared__ Pair sh[kThreads / 32];
  __shared__ bool last;
  const long long vs = A.neq_cap;
  double *base = A.vec + S.off;
  const int nops = R.prog_len;
  const long long n = S.neq;
  const long long stride = (long long)S.nblk * kThreads;
  Pair acc = red_identity<(RED >= 0 ? RED : 0)>();
  for (long long j0 = (long long)b * kThreads + threadIdx.x; j0 < n; j0 += kU * stride) {
    long long j[kU];
    int nu = 0;
#pragma unroll
    for (int u = 0; u < kU; u++) {
      j[u] = j0 + u * stride;
      nu += (j[u] < n);
    }
    for (int p = 0; p < nops; p++) exec_op<kU>(prog[p], A, S, base, vs, j, nu);
    if (RED >= 0) {
      double xv[kU], yv[kU];
#pragma unroll
      for (int u = 0; u < kU; u++)
        if (u < nu) {
          xv[u] = base[R.rx * vs + j[u]];
          yv[u] = (RED == R_DOT || RED == R_WSQ) ? base[R.ry * vs + j[u]] : 0.0;
        }
#pragma unroll
      for (int u = 0; u < kU; u++)
        if (u < nu) acc = red_combine<RED>(acc, red_term<RED>(xv[u], yv[u]));
    }
  }
  if (RED < 0) return;
  acc = red_block<RED>(acc, sh);
  double *partials = A.partials + (long long)R.sys * 2 * kMaxBlocks;
  unsigned int *ticket = A.tickets + R.sys;
  if (threadIdx.x == 0) {
    partials[b] = acc.v;
    partials[kMaxBlocks + b] = acc.f;
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    last = (t == (unsigned)S.nblk - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  Pair v = red_identity<RED>();
  for (int q = threadIdx.x; q < S.nblk; q += blockDim.x) {
    Pair p = {((volatile double *)partials)[q], ((volatile double *)partials)[kMaxBlocks + q]};
    v = red_combine<RED>(v, p);
  }
  v = red_block<RED>(v, sh);
  if (threadIdx.x == 0) {
    A.results[2 * R.sys] = v.v;
    A.results[2 * R.sys + 1] = v.f;
    *ticket = 0u;
  }
}

template <int kU>
__global__ void __launch_bounds__(kThreads, (kU == 1 ? 6 : (kU == 2 ? 5 : 3))) k_program(DeviceArena A, int nrs) {
  // Stage the round's block ranges and then this block's program in shared
  // memory: one coalesced pass each instead of a chain of dependent global
  // loads before any entry is touched.
  extern __shared__ __align__(16) unsigned char smem[];
  Op *s_ops = reinterpret_cast<Op *>(smem);
  int32_t *s_bstart = reinterpret_cast<int32_t *>(smem + sizeof(Op) * kMaxProgOps);
  for (int i = threadIdx.x; i < nrs; i += blockDim.x) s_bstart[i] = A.round[i].bstart;
  __syncthreads();
  int lo = 0, hi = nrs - 1;
  const int blk = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (s_bstart[mid] <= blk) lo = mid;
    else hi = mid - 1;
  }
  const RoundSys R = A.round[lo];
  const SysInfo S = A.sysinfo[R.sys];
  const int b = blk - R.bstart;
  if (b >= S.nblk) return;
  {
    const double *src = reinterpret_cast<const double *>(A.ops + R.prog_off);
    double *dst = reinterpret_cast<double *>(s_ops);
    const int nw = R.prog_len * (int)(sizeof(Op) / sizeof(double));
    for (int i = threadIdx.x; i < nw; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  switch (R.red) {
    case R_DOT: run_block<kU, R_DOT>(A, R, S, s_ops, b); break;
    case R_MAXABS: run_block<kU, R_MAXABS>(A, R, S, s_ops, b); break;
    case R_WSQ: run_block<kU, R_WSQ>(A, R, S, s_ops, b); break;
    case R_MIN: run_block<kU, R_MIN>(A, R, S, s_ops, b); break;
    default: run_block<kU, -1>(A, R, S, s_ops, b); break;
  }
}

}  // namespace

static_assert(sizeof(Op) == 40 && sizeof(Op) % sizeof(double) == 0, "Op is staged as doubles");

// blockIdx.y picks the descriptor, blockIdx.x a kGatherChunk-byte chunk of
// it; 8-byte words where source, destination and size allow, else 4-byte
// words, else bytes
constexpr uint64_t kGatherChunk = 64 * 1024;

__global__ void __launch_bounds__(256) k_gather_host(const CopyDesc *desc, int n) {
  const CopyDesc d = desc[blockIdx.y];
  const uint64_t lo = (uint64_t)blockIdx.x * kGatherChunk;
  if (lo >= d.bytes) return;
  const uint64_t hi = min(d.bytes, lo + kGatherChunk);
  const uintptr_t align = (uintptr_t)d.src | (uintptr_t)d.dst | (uintptr_t)d.bytes;
  const char *src = (const char *)d.src;
  char *dst = (char *)d.dst;
  if ((align & 7) == 0) {
    for (uint64_t b = lo + 8 * (uint64_t)threadIdx.x; b < hi; b += 8 * (uint64_t)blockDim.x)
      *(uint64_t *)(dst + b) = *(const uint64_t *)(src + b);
  } else if ((align & 3) == 0) {
    for (uint64_t b = lo + 4 * (uint64_t)threadIdx.x; b < hi; b += 4 * (uint64_t)blockDim.x)
      *(uint32_t *)(dst + b) = *(const uint32_t *)(src + b);
  } else {
    for (uint64_t b = lo + threadIdx.x; b < hi; b += blockDim.x) dst[b] = src[b];
  }
}

cudaError_t launch_gather_host(const CopyDesc *desc, int n, uint64_t max_bytes, cudaStream_t st) {
  if (n <= 0 || max_bytes == 0) return cudaSuccess;
  if (n > 65535) return cudaErrorInvalidValue;
  const dim3 grid((unsigned)((max_bytes + kGatherChunk - 1) / kGatherChunk), (unsigned)n);
  k_gather_host<<<grid, 256, 0, st>>>(desc, n);
  return cudaGetLastError();
}

cudaError_t launch_program(const DeviceArena &a, int nrs, int nblocks, int variant, cudaStream_t st) {
  if (nrs <= 0 || nblocks <= 0) return cudaSuccess;
  const size_t smem = sizeof(Op) * kMaxProgOps + sizeof(int32_t) * (size_t)nrs;
  if (variant == 0) k_program<1><<<nblocks, kThreads, smem, st>>>(a, nrs);
  else if (variant == 1) k_program<2><<<nblocks, kThreads, smem, st>>>(a, nrs);
  else k_program<4><<<nblocks, kThreads, smem, st>>>(a, nrs);
  return cudaGetLastError();
}

}  // namespace batch
}  // namespace pihm
