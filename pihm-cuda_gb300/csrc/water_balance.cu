// Watershed water balance of one model step on the device: the three sums of
// PrintWaterBal (src/print.c:337-542) over the current state and fluxes --
//   sources  sum over elements of prcp area dt,
//   sinks    sum over elements of (edir + ett + ec) area dt plus the outlet
//            segments' DOWN_CHANL2CHANL flux times dt,
//   storage  sum over elements of (cmc + sneqv + surf + (unsat + gw) porosity)
//            area plus the segments' (stage + gw porosity) area.
// With the land-surface model attached (include/pihm_land.h) prcp, ec, cmc
// and sneqv are its planes; without it the forcing is given directly, so
// prcp = pcpdrp and ec = cmc = sneqv = 0 (no canopy or snow).
// The caller accumulates src - snk - (storage - previous storage) as the
// reference's cumulative error.  Sums are deterministic (fixed block tree and
// a fixed-order final pass).
#include "nv_reduce.cuh"
#include "pihm_internal.h"

namespace pihm {

namespace {

constexpr int kWbThreads = 256;
constexpr int kWbMaxBlocks = 1024;

__global__ void __launch_bounds__(kWbThreads) k_water_balance(DevMesh m, const double *__restrict__ y, double dt,
                                                              double *partials) {
  const int ne = m.ne, nr = m.nr;
  double src = 0.0, snk = 0.0, strg = 0.0;
  const long long n = (long long)ne + nr;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    if (t < ne) {
      const int i = (int)t;
      const double area = m.area[i];
      if (m.land_prcp) {
        src += m.land_prcp[i] * area * dt;
        snk += (m.edir[i] + m.ett[i] + m.land_ec[i]) * area * dt;
        strg += (m.land_cmc[i] + m.land_sneqv[i] + y[i] + (y[ne + i] + y[2 * ne + i]) * m.porosity[i]) * area;
      } else {
        src += m.pcpdrp[i] * area * dt;
        snk += (m.edir[i] + m.ett[i]) * area * dt;
        strg += (y[i] + (y[ne + i] + y[2 * ne + i]) * m.porosity[i]) * area;
      }
    } else {
      const int s = (int)(t - ne);
      strg += (y[3 * ne + s] + y[3 * ne + nr + s] * m.r_porosity[s]) * m.r_area[s];
      if (m.down[s] < 0) snk += m.rivflow[DOWN_CHANL2CHANL * nr + s] * dt;
    }
  }
  __shared__ pihm_nv::Pair sh[kWbThreads / 32];
  double v[3] = {src, snk, strg};
#pragma unroll
  for (int q = 0; q < 3; q++) {
    pihm_nv::Pair p = {v[q], 0.0};
    p = pihm_nv::red_block<pihm_nv::R_DOT>(p, sh);
    if (threadIdx.x == 0) partials[q * kWbMaxBlocks + blockIdx.x] = p.v;
    __syncthreads();
  }
}

__global__ void k_water_balance_final(const double *partials, int nblocks, double *out) {
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int b = 0; b < nblocks; b++) s += partials[threadIdx.x * kWbMaxBlocks + b];
    out[threadIdx.x] = s;
  }
}

}  // namespace

}  // namespace pihm

using namespace pihm;

extern "C" int pihm_gpu_water_balance(pihm_gpu_ctx *c, const double *y_dev, double dt, double *out) {
  if (!c || !y_dev || !out || !(dt > 0.0)) return PIHM_GPU_ERR_ARG;
  const long long n = (long long)c->ne + c->nr;
  long long g = (n + kWbThreads - 1) / kWbThreads;
  if (g > kWbMaxBlocks) g = kWbMaxBlocks;
  if (g < 1) g = 1;
  double *buf = nullptr;  // partials [3][kWbMaxBlocks], then the three sums
  if (cudaMallocAsync((void **)&buf, sizeof(double) * (3 * kWbMaxBlocks + 3), c->stream) != cudaSuccess)
    return PIHM_GPU_ERR_NOMEM;
  k_water_balance<<<(unsigned)g, kWbThreads, 0, c->stream>>>(c->m, y_dev, dt, buf);
  k_water_balance_final<<<1, 32, 0, c->stream>>>(buf, (int)g, buf + 3 * kWbMaxBlocks);
  c->launches += 2;
  int rc = PIHM_GPU_OK;
  if (cudaMemcpyAsync(out, buf + 3 * kWbMaxBlocks, sizeof(double) * 3, cudaMemcpyDeviceToHost, c->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    rc = PIHM_GPU_ERR_CUDA;
  cudaFreeAsync(buf, c->stream);
  return rc;
}
