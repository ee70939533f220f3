// Warp-shuffle / block reduction helpers shared by the N_Vector kernels.
#pragma once

#include <cmath>

#include "nv_select.h"

namespace pihm_nv {

struct Pair {
  double v;
  double f;  // flag channel (found / failed)
};

template <int OP>
__device__ __forceinline__ Pair red_identity() {
  if (OP == R_MAXABS) return {0.0, 0.0};
  if (OP == R_MIN || OP == R_MINQ) return {INFINITY, 0.0};
  return {0.0, 0.0};
}

template <int OP>
__device__ __forceinline__ Pair red_combine(Pair p, Pair q) {
  if (OP == R_MAXABS) return {fmax(p.v, q.v), 0.0};
  if (OP == R_MIN || OP == R_MINQ) return {fmin(p.v, q.v), fmax(p.f, q.f)};
  if (OP == R_INVTEST || OP == R_CONSTR) return {0.0, fmax(p.f, q.f)};
  return {__dadd_rn(p.v, q.v), 0.0};
}

template <int OP>
__device__ __forceinline__ Pair red_block(Pair v, Pair *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Pair q;
    q.v = __shfl_down_sync(0xffffffffu, v.v, o);
    q.f = __shfl_down_sync(0xffffffffu, v.f, o);
    v = red_combine<OP>(v, q);
  }
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : red_identity<OP>();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      Pair q;
      q.v = __shfl_down_sync(0xffffffffu, v.v, o);
      q.f = __shfl_down_sync(0xffffffffu, v.f, o);
      v = red_combine<OP>(v, q);
    }
  }
  return v;
}

}  // namespace pihm_nv
