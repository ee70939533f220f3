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

template <int OP>
__device__ __forceinline__ void ew_at(const Op &o, double *base, long long vs, long long j) {
  const double xv = ew_reads_x(OP) ? base[o.x * vs + j] : 0.0;
  const double yv = ew_reads_y(OP) ? base[o.y * vs + j] : 0.0;
  double *z = base + o.z * vs + j;
  const double zv = ew_reads_z(OP) ? *z : 0.0;
  *z = ew_eval<OP>(o.a, o.b, xv, yv, zv);
}

// Apply one operation to entry j.  base points at the watershed's entry 0 in
// vector slot 0; slots are vs entries apart.
__device__ __forceinline__ void exec_op(const Op &o, const DeviceArena &A, const SysInfo &S, double *base,
                                        long long vs, long long j) {
  switch (o.code) {
    case EW_LIN: ew_at<EW_LIN>(o, base, vs, j); break;
    case EW_LIN1: ew_at<EW_LIN1>(o, base, vs, j); break;
    case EW_LIN2: ew_at<EW_LIN2>(o, base, vs, j); break;
    case EW_SUM: ew_at<EW_SUM>(o, base, vs, j); break;
    case EW_DIFF: ew_at<EW_DIFF>(o, base, vs, j); break;
    case EW_SCALESUM: ew_at<EW_SCALESUM>(o, base, vs, j); break;
    case EW_SCALEDIFF: ew_at<EW_SCALEDIFF>(o, base, vs, j); break;
    case EW_AXPY: ew_at<EW_AXPY>(o, base, vs, j); break;
    case EW_AXPY1: ew_at<EW_AXPY1>(o, base, vs, j); break;
    case EW_AXPYM1: ew_at<EW_AXPYM1>(o, base, vs, j); break;
    case EW_CONST: ew_at<EW_CONST>(o, base, vs, j); break;
    case EW_PROD: ew_at<EW_PROD>(o, base, vs, j); break;
    case EW_DIV: ew_at<EW_DIV>(o, base, vs, j); break;
    case EW_SCALE: ew_at<EW_SCALE>(o, base, vs, j); break;
    case EW_COPY: ew_at<EW_COPY>(o, base, vs, j); break;
    case EW_NEG: ew_at<EW_NEG>(o, base, vs, j); break;
    case EW_ABS: ew_at<EW_ABS>(o, base, vs, j); break;
    case EW_INV: ew_at<EW_INV>(o, base, vs, j); break;
    case EW_ADDCONST: ew_at<EW_ADDCONST>(o, base, vs, j); break;
    case EW_COMPARE: ew_at<EW_COMPARE>(o, base, vs, j); break;
    case OP_STAGE_IN:
      A.rhs_in[stage_pos(S, j, A.m.ne, A.m.nr)] = base[o.x * vs + j];
      break;
    case OP_STAGE_OUT:
      base[o.z * vs + j] = A.rhs_out[stage_pos(S, j, A.m.ne, A.m.nr)];
      break;
    case OP_FORCING:
      if (j < S.ne) {
        const long long g = S.eoff + j;
        ((double *)A.m.pcpdrp)[g] = o.a;
        ((double *)A.m.edir)[g] = o.b;
        ((double *)A.m.ett)[g] = o.c;
      }
      break;
    case OP_WS0:
      if (j < S.ne) ((double *)A.m.ws0_surf)[S.eoff + j] = base[o.x * vs + j];
      break;
    case OP_RECORD:
      if (j == 0) A.rec[S.rec_off + o.i0] = A.m.rivflow[(long long)DOWN_CHANL2CHANL * A.m.nr + S.roff + o.i1];
      break;
    default: break;
  }
}

// One block of one watershed's program: the element-wise operations over the
// block's grid-strided entries, then (RED >= 0) the reduction, combined
// exactly as the single-vector reduction kernel combines it.
template <int RED>
__device__ void run_block(const DeviceArena &A, const RoundSys &R, const SysInfo &S, int b) {
  __shared__ Pair sh[kThreads / 32];
  __shared__ bool last;
  const long long vs = A.neq_cap;
  double *base = A.vec + S.off;
  const Op *prog = A.ops + R.prog_off;
  const int nops = R.prog_len;
  const long long n = S.neq;
  const long long stride = (long long)S.nblk * kThreads;
  Pair acc = red_identity<(RED >= 0 ? RED : 0)>();
  for (long long j = (long long)b * kThreads + threadIdx.x; j < n; j += stride) {
    for (int p = 0; p < nops; p++) exec_op(prog[p], A, S, base, vs, j);
    if (RED >= 0) {
      const double xv = base[R.rx * vs + j];
      const double yv = (RED == R_DOT || RED == R_WSQ) ? base[R.ry * vs + j] : 0.0;
      acc = red_combine<RED>(acc, red_term<RED>(xv, yv));
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

__global__ void __launch_bounds__(kThreads) k_program(DeviceArena A, int nrs) {
  // the round entry whose block range holds this block
  int lo = 0, hi = nrs - 1;
  const int blk = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (A.round[mid].bstart <= blk) lo = mid;
    else hi = mid - 1;
  }
  const RoundSys R = A.round[lo];
  const SysInfo S = A.sysinfo[R.sys];
  const int b = blk - R.bstart;
  if (b >= S.nblk) return;
  switch (R.red) {
    case R_DOT: run_block<R_DOT>(A, R, S, b); break;
    case R_MAXABS: run_block<R_MAXABS>(A, R, S, b); break;
    case R_WSQ: run_block<R_WSQ>(A, R, S, b); break;
    case R_MIN: run_block<R_MIN>(A, R, S, b); break;
    default: run_block<-1>(A, R, S, b); break;
  }
}

}  // namespace

cudaError_t launch_program(const DeviceArena &a, int nrs, int nblocks, cudaStream_t st) {
  if (nrs <= 0 || nblocks <= 0) return cudaSuccess;
  k_program<<<nblocks, kThreads, 0, st>>>(a, nrs);
  return cudaGetLastError();
}

}  // namespace batch
}  // namespace pihm
