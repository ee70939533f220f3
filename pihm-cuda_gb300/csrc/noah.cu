// The Noah land-surface model of Flux-PIHM on the device (include/pihm_noah.h).
//
// One thread per element and kernel:
//   k_noah_step   Noah() over a land-surface step (noah_phys.cuh: CalHum,
//                 FrozRain, net radiation, SFlx with its snowpack,
//                 frozen-soil, soil-heat and canopy physics)
//   k_noah_post   after a model step: Summary's _NOAH_ part (MassBalance's
//                 infiltration and subsurface runoff, src/update.c:100-165;
//                 runoff2, FindWaterTable, CalcLatFlx, src/update.c:34-41)
//                 and NoahHydrol (FindWaterTable, the moisture clamps, SmFlx,
//                 src/noah/noah.c:57-97)
//   k_noah_inputs what the Flux-PIHM right-hand side reads: GwTransp's layer
//                 sum (noah/lsm_func.c:163-185) and whether the water table
//                 lies within the root zone, Infil's top-layer saturation
//                 (src/vert_flow.c:94-98), the frozen-soil factor, and the
//                 right-hand side's edir, ett and pcpdrp planes
// Every plane is in the context's internal element order; per-layer planes
// are [layer][ne].  The state never leaves the device between steps.
#include <cmath>
#include <cstring>
#include <vector>

#include "noah_phys.cuh"
#include "pihm_internal.h"
#include "pihm_noah.h"

namespace pihm {

// scalar per-element planes
enum NoahScalar {
  // parameters
  NS_SMCMAX = 0, NS_SMCMIN, NS_SMCREF, NS_SMCWLT, NS_SMCDRY, NS_QUARTZ, NS_CSOIL, NS_ALPHA, NS_BETA, NS_KSATV,
  NS_POROSITY, NS_DEPTH, NS_AREA, NS_SHDFAC, NS_CMCFACTR, NS_LAIMAX, NS_LAIMIN, NS_EMISSMAX, NS_EMISSMIN,
  NS_ALBEDOMAX, NS_ALBEDOMIN, NS_Z0MAX, NS_Z0MIN, NS_SNUP, NS_CFACTR, NS_RGL, NS_RSMIN, NS_RSMAX, NS_TOPT, NS_HS,
  NS_SBETA, NS_SALP, NS_FRZX, NS_FXEXP, NS_CZIL, NS_LVCOEF, NS_ZBOT, NS_TBOT, NS_ZLVL, NS_ZLVL_WIND, NS_SNOALB,
  // forcing
  NS_PRCP, NS_SFCTMP, NS_RH, NS_SFCSPD, NS_SOLDN, NS_LONGWAVE, NS_SFCPRS, NS_LAI,
  // carried state
  NS_T1, NS_CMC, NS_SNEQV, NS_SNOWH, NS_SNDENS, NS_CH, NS_CM, NS_SNOTIME1, NS_ALBEDO, NS_EMISSI, NS_Q1, NS_RIBB,
  NS_FCR,
  // outputs
  NS_EDIR, NS_EC, NS_ETT, NS_ESNOW, NS_ETP, NS_DRIP, NS_PCPDRP, NS_SNOMLT, NS_SSOIL, NS_SHEAT, NS_RUNOFF2,
  NS_RUNOFF3, NS_INFIL, NS_SNCOVR, NS_BETA_S, NS_ETA, NS_SOILM,
  // kept from step to step like the reference's wf.etns, which SnoPac's dew
  // branch leaves unchanged and SFlx then reads
  NS_ETNS,
  // the previous model step's groundwater and unsaturated storage (ws0)
  NS_GW0, NS_UNSAT0,
  NS_COUNT
};
enum NoahLayer { NL_SLDPTH = 0, NL_ZSOIL, NL_RTDIS, NL_SMC, NL_SH2O, NL_STC, NL_ET, NL_RUNOFF2_LYR, NL_SMFLXV, NL_COUNT };
enum NoahInt { NI_NSOIL = 0, NI_NROOT, NI_ISURBAN, NI_NWTBL, NI_COUNT };

struct NoahPlanes {
  double *s[NS_COUNT];
  double *l[NL_COUNT];
  int32_t *i[NI_COUNT];
  int32_t *order;   // [ne] elements grouped by the branches Noah() will take (k_noah_classify)
  int32_t *cls;     // [2 * kNoahClasses] class sizes, then cursors
  int ne;
};

namespace {

using noah::Col;
using noah::L;

__device__ void load_col(const NoahPlanes &P, int i, Col &c) {
  const int ne = P.ne;
  c.nsoil = P.i[NI_NSOIL][i];
  c.nroot = P.i[NI_NROOT][i];
  c.isurban = P.i[NI_ISURBAN][i];
  c.nwtbl = P.i[NI_NWTBL][i];
  for (int k = 0; k < L; k++) {
    const bool in = k < c.nsoil;
    c.sldpth[k] = in ? P.l[NL_SLDPTH][k * ne + i] : 0.0;
    c.zsoil[k] = in ? P.l[NL_ZSOIL][k * ne + i] : 0.0;
    c.rtdis[k] = in ? P.l[NL_RTDIS][k * ne + i] : 0.0;
    c.smc[k] = in ? P.l[NL_SMC][k * ne + i] : 0.0;
    c.sh2o[k] = in ? P.l[NL_SH2O][k * ne + i] : 0.0;
    c.stc[k] = in ? P.l[NL_STC][k * ne + i] : 0.0;
    c.et[k] = in ? P.l[NL_ET][k * ne + i] : 0.0;
    c.runoff2_lyr[k] = in ? P.l[NL_RUNOFF2_LYR][k * ne + i] : 0.0;
    c.smflxv[k] = in ? P.l[NL_SMFLXV][k * ne + i] : 0.0;
    c.satdpth[k] = 0.0;
  }
  const double *const *s = P.s;
  c.smcmax = s[NS_SMCMAX][i]; c.smcmin = s[NS_SMCMIN][i]; c.smcref = s[NS_SMCREF][i];
  c.smcwlt = s[NS_SMCWLT][i]; c.smcdry = s[NS_SMCDRY][i]; c.quartz = s[NS_QUARTZ][i];
  c.csoil = s[NS_CSOIL][i]; c.alpha = s[NS_ALPHA][i]; c.beta = s[NS_BETA][i]; c.ksatv = s[NS_KSATV][i];
  c.porosity = s[NS_POROSITY][i]; c.depth = s[NS_DEPTH][i]; c.area = s[NS_AREA][i];
  c.shdfac = s[NS_SHDFAC][i]; c.cmcfactr = s[NS_CMCFACTR][i]; c.laimax = s[NS_LAIMAX][i];
  c.laimin = s[NS_LAIMIN][i]; c.emissmax = s[NS_EMISSMAX][i]; c.emissmin = s[NS_EMISSMIN][i];
  c.albedomax = s[NS_ALBEDOMAX][i]; c.albedomin = s[NS_ALBEDOMIN][i]; c.z0max = s[NS_Z0MAX][i];
  c.z0min = s[NS_Z0MIN][i]; c.snup = s[NS_SNUP][i]; c.cfactr = s[NS_CFACTR][i]; c.rgl = s[NS_RGL][i];
  c.rsmin = s[NS_RSMIN][i]; c.rsmax = s[NS_RSMAX][i]; c.topt = s[NS_TOPT][i]; c.hs = s[NS_HS][i];
  c.sbeta = s[NS_SBETA][i]; c.salp = s[NS_SALP][i]; c.frzx = s[NS_FRZX][i]; c.fxexp = s[NS_FXEXP][i];
  c.czil = s[NS_CZIL][i]; c.lvcoef = s[NS_LVCOEF][i]; c.zbot = s[NS_ZBOT][i]; c.tbot = s[NS_TBOT][i];
  c.zlvl = s[NS_ZLVL][i]; c.zlvl_wind = s[NS_ZLVL_WIND][i]; c.snoalb = s[NS_SNOALB][i];
  c.prcp = s[NS_PRCP][i]; c.sfctmp = s[NS_SFCTMP][i]; c.rh = s[NS_RH][i]; c.sfcspd = s[NS_SFCSPD][i];
  c.soldn = s[NS_SOLDN][i]; c.longwave = s[NS_LONGWAVE][i]; c.sfcprs = s[NS_SFCPRS][i];
  c.proj_lai = s[NS_LAI][i];
  c.t1 = s[NS_T1][i]; c.cmc = s[NS_CMC][i]; c.sneqv = s[NS_SNEQV][i]; c.snowh = s[NS_SNOWH][i];
  c.sndens = s[NS_SNDENS][i]; c.ch = s[NS_CH][i]; c.cm = s[NS_CM][i]; c.snotime1 = s[NS_SNOTIME1][i];
  c.albedo = s[NS_ALBEDO][i]; c.emissi = s[NS_EMISSI][i]; c.q1 = s[NS_Q1][i]; c.ribb = s[NS_RIBB][i];
  c.fcr = s[NS_FCR][i];
  c.edir = s[NS_EDIR][i]; c.ec = s[NS_EC][i]; c.ett = s[NS_ETT][i]; c.esnow = s[NS_ESNOW][i];
  c.etp = s[NS_ETP][i]; c.drip = s[NS_DRIP][i]; c.pcpdrp = s[NS_PCPDRP][i]; c.snomlt = s[NS_SNOMLT][i];
  c.ssoil = s[NS_SSOIL][i]; c.sheat = s[NS_SHEAT][i]; c.runoff2 = s[NS_RUNOFF2][i];
  c.runoff3 = s[NS_RUNOFF3][i]; c.infil = s[NS_INFIL][i]; c.sncovr = s[NS_SNCOVR][i];
  c.beta_s = s[NS_BETA_S][i]; c.eta = s[NS_ETA][i]; c.soilm = s[NS_SOILM][i];
  c.etns = s[NS_ETNS][i];
}

// What a step changes: the state, the outputs and -- for urban land, where
// SFlx overrides them for good (src/noah/noah.c:201-212) -- the parameters.
__device__ void store_col(const NoahPlanes &P, int i, const Col &c) {
  const int ne = P.ne;
  for (int k = 0; k < c.nsoil; k++) {
    P.l[NL_SMC][k * ne + i] = c.smc[k];
    P.l[NL_SH2O][k * ne + i] = c.sh2o[k];
    P.l[NL_STC][k * ne + i] = c.stc[k];
    P.l[NL_ET][k * ne + i] = c.et[k];
    P.l[NL_RUNOFF2_LYR][k * ne + i] = c.runoff2_lyr[k];
    P.l[NL_SMFLXV][k * ne + i] = c.smflxv[k];
  }
  P.i[NI_NWTBL][i] = c.nwtbl;
  double *const *s = P.s;
  if (c.isurban) {
    s[NS_SHDFAC][i] = c.shdfac; s[NS_RSMIN][i] = c.rsmin; s[NS_SMCMAX][i] = c.smcmax;
    s[NS_SMCMIN][i] = c.smcmin; s[NS_SMCREF][i] = c.smcref; s[NS_SMCWLT][i] = c.smcwlt;
    s[NS_SMCDRY][i] = c.smcdry;
  }
  s[NS_T1][i] = c.t1; s[NS_CMC][i] = c.cmc; s[NS_SNEQV][i] = c.sneqv; s[NS_SNOWH][i] = c.snowh;
  s[NS_SNDENS][i] = c.sndens; s[NS_CH][i] = c.ch; s[NS_CM][i] = c.cm; s[NS_SNOTIME1][i] = c.snotime1;
  s[NS_ALBEDO][i] = c.albedo; s[NS_EMISSI][i] = c.emissi; s[NS_Q1][i] = c.q1; s[NS_RIBB][i] = c.ribb;
  s[NS_FCR][i] = c.fcr;
  s[NS_EDIR][i] = c.edir; s[NS_EC][i] = c.ec; s[NS_ETT][i] = c.ett; s[NS_ESNOW][i] = c.esnow;
  s[NS_ETP][i] = c.etp; s[NS_DRIP][i] = c.drip; s[NS_PCPDRP][i] = c.pcpdrp; s[NS_SNOMLT][i] = c.snomlt;
  s[NS_SSOIL][i] = c.ssoil; s[NS_SHEAT][i] = c.sheat; s[NS_RUNOFF2][i] = c.runoff2;
  s[NS_RUNOFF3][i] = c.runoff3; s[NS_INFIL][i] = c.infil; s[NS_SNCOVR][i] = c.sncovr;
  s[NS_BETA_S][i] = c.beta_s; s[NS_ETA][i] = c.eta; s[NS_SOILM][i] = c.soilm;
  s[NS_ETNS][i] = c.etns;
}

constexpr int kNoahBlock = 128;
constexpr int kNoahClasses = 8;

// The branch class of an element's next Noah() step: whether it will run the
// snowpack path (snow on the ground, or precipitation that may fall as snow
// or freezing rain), whether a soil layer or the skin is frozen (the
// iterative frozen-water solution of FrH2O), whether it has vegetation (the
// canopy resistance and transpiration).  Noah() is one thread per element and
// GB300 retires 2 FP64 lanes per clock per SM, so a warp whose lanes take
// different paths runs each path for all of them; grouping elements by class
// keeps warps on one path.  Only the order of work changes: every element's
// arithmetic, and so every result, is the same.
__device__ __forceinline__ int noah_class(const NoahPlanes &P, int i) {
  const double tf = 273.15;
  const bool snow = P.s[NS_SNEQV][i] > 0.0 || (P.s[NS_PRCP][i] > 0.0 && P.s[NS_SFCTMP][i] <= tf + 1.0);
  bool frozen = P.s[NS_T1][i] < tf;
  const int nsoil = P.i[NI_NSOIL][i];
  for (int k = 0; k < nsoil; k++) frozen = frozen || P.l[NL_STC][k * P.ne + i] < tf;
  const bool veg = P.s[NS_SHDFAC][i] > 0.0;
  return (snow ? 4 : 0) + (frozen ? 2 : 0) + (veg ? 1 : 0);
}

// class sizes (cls[0..7]; the caller zeroed cls)
__global__ void __launch_bounds__(256) k_noah_count(NoahPlanes P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.ne) return;
  atomicAdd(&P.cls[noah_class(P, i)], 1);
}

// each element's place: its class's start (the sizes summed in class order)
// plus a cursor; lanes of a warp in one class take consecutive places
__global__ void __launch_bounds__(256) k_noah_place(NoahPlanes P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = i < P.ne;
  const int c = in ? noah_class(P, i) : kNoahClasses;
  const unsigned mask = __match_any_sync(0xffffffffu, c);
  if (!in) return;
  const int lead = __ffs(mask) - 1, lane = threadIdx.x & 31;
  int base = 0;
  if (lane == lead) base = atomicAdd(&P.cls[kNoahClasses + c], __popc(mask));
  base = __shfl_sync(mask, base, lead);
  int start = 0;
  for (int k = 0; k < c; k++) start += P.cls[k];
  P.order[start + base + __popc(mask & ((1u << lane) - 1u))] = i;
}

__global__ void __launch_bounds__(kNoahBlock) k_noah_step(NoahPlanes P, double dt, unsigned int *err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.ne) return;
  const int i = P.order[t];
  Col c;
  load_col(P, i, c);
  noah::noah_step(c, dt);
  // the reference exits when the snow density exceeds one (SFlx) or a
  // state turns NaN; here the context's error word records it
  if (c.sneqv > 1.0e-7 && !(c.sndens <= 1.0)) atomicOr(err, 1u);
  if (c.t1 != c.t1 || c.edir != c.edir || c.ett != c.ett) atomicOr(err, 1u);
  store_col(P, i, c);
}

// y: the model state after the step (internal order); first: no previous
// state yet, ws0 is taken from y
__global__ void __launch_bounds__(kNoahBlock) k_noah_post(NoahPlanes P, NoahTargets o, const double *y, double dt,
                                                          int first) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.ne) return;
  const int ne = P.ne;
  Col c;
  load_col(P, i, c);
  // Summary, src/update.c:3-48: the element state from y, then MassBalance
  const double unsat = y[ne + i], gw = y[2 * ne + i];
  const double gw0 = first ? gw : P.s[NS_GW0][i];
  const double unsat0 = first ? unsat : P.s[NS_UNSAT0][i];
  double soilw0 = gw0 + unsat0;
  soilw0 = (soilw0 > c.depth) ? c.depth : soilw0;
  soilw0 = (soilw0 < 0.0) ? 0.0 : soilw0;
  double soilw1 = gw + unsat;
  soilw1 = (soilw1 > c.depth) ? c.depth : soilw1;
  soilw1 = (soilw1 < 0.0) ? 0.0 : soilw1;
  double subrunoff = 0.0;
  const int64_t ds = o.stride;
  for (int j = 0; j < 3; j++) subrunoff += o.d_sub[j * ds + i] / c.area;
  // the last evaluation's ET split: edir_unsat, edir_gw, ett_unsat, ett_gw
  c.infil = (soilw1 - soilw0) * c.porosity / dt + subrunoff + o.d_et[ds + i] + o.d_et[2 * ds + i] +
            o.d_et[3 * ds + i] + o.d_et[4 * ds + i];
  if (c.infil < 0.0) {
    subrunoff -= c.infil;
    c.infil = 0.0;
  }
  c.runoff2 = subrunoff;
  c.nwtbl = noah::find_water_table(c.sldpth, c.nsoil, gw, c.satdpth);
  noah::calc_lat_flx(c);
  P.s[NS_GW0][i] = gw;
  P.s[NS_UNSAT0][i] = unsat;
  // NoahHydrol
  noah::noah_hydrol(c, gw, dt);
  store_col(P, i, c);
}

// ws0 from the state a run starts from
__global__ void __launch_bounds__(256) k_noah_begin(NoahPlanes P, const double *y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.ne) return;
  P.s[NS_UNSAT0][i] = y[P.ne + i];
  P.s[NS_GW0][i] = y[2 * P.ne + i];
}

// The Flux-PIHM right-hand side's inputs from Noah's state and outputs.
__global__ void __launch_bounds__(256) k_noah_inputs(NoahPlanes P, NoahTargets o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.ne) return;
  const int ne = P.ne;
  const int top = P.i[NI_NWTBL][i], nr = P.i[NI_NROOT][i];
  double g = 0.0;
  if (top <= nr)
    for (int j = (top <= 0 ? 0 : top - 1); j < nr; j++) g += P.l[NL_ET][j * ne + i];
  const double smcmin = P.s[NS_SMCMIN][i], smcmax = P.s[NS_SMCMAX][i];
  o.etgw[i] = g;
  o.wtin[i] = top <= nr;
  o.satn[i] = (P.l[NL_SH2O][i] - smcmin) / (smcmax - smcmin);
  o.fcr[i] = P.s[NS_FCR][i];
  o.edir[i] = P.s[NS_EDIR][i];
  o.ett[i] = P.s[NS_ETT][i];
  o.pcpdrp[i] = P.s[NS_PCPDRP][i];
}

template <class T>
size_t padded(size_t n) {
  return (n * sizeof(T) + 255) & ~size_t(255);
}

int cuda_rc(cudaError_t e) { return e == cudaSuccess ? PIHM_GPU_OK : PIHM_GPU_ERR_CUDA; }

// reference-order [ne][per] host values -> internal-order [per][ne] device planes
int upload(const int32_t *perm, int ne, const double *src, int per, double *const *dst, cudaStream_t st) {
  std::vector<double> h((size_t)ne);
  for (int k = 0; k < per; k++) {
    for (int i = 0; i < ne; i++) h[i] = src[(size_t)per * perm[i] + k];
    if (cudaMemcpyAsync(dst[k], h.data(), sizeof(double) * ne, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return PIHM_GPU_ERR_CUDA;
  }
  return PIHM_GPU_OK;
}

int upload_layers(const int32_t *perm, int ne, const double *src, double *plane, cudaStream_t st) {
  double *dst[noah::L];
  for (int k = 0; k < noah::L; k++) dst[k] = plane + (size_t)k * ne;
  return upload(perm, ne, src, noah::L, dst, st);
}

int upload_int(const int32_t *perm, int ne, const int32_t *src, int32_t *dst) {
  std::vector<int32_t> h((size_t)ne);
  for (int i = 0; i < ne; i++) h[i] = src[perm[i]];
  return cuda_rc(cudaMemcpy(dst, h.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice));
}

int upload_scalar(const int32_t *perm, int ne, const double *src, double *dst, cudaStream_t st) {
  return src ? upload(perm, ne, src, 1, &dst, st) : 0;
}

int launch_inputs(NoahInstance &n, cudaStream_t st, int64_t *launches) {
  k_noah_inputs<<<(n.ne + 255) / 256, 256, 0, st>>>(*n.P, n.tg);
  ++*launches;
  return cuda_rc(cudaGetLastError());
}

}  // namespace

int noah_set_state(NoahInstance &n, const pihm_noah_state *s, const int32_t *perm, cudaStream_t st) {
  if (!n.alloc || !s) return PIHM_GPU_ERR_ARG;
  NoahPlanes &P = *n.P;
  const int ne = n.ne;
  int rc = PIHM_GPU_OK;
  if (s->smc) rc = rc ?: upload_layers(perm, ne, s->smc, P.l[NL_SMC], st);
  if (s->sh2o) rc = rc ?: upload_layers(perm, ne, s->sh2o, P.l[NL_SH2O], st);
  if (s->stc) rc = rc ?: upload_layers(perm, ne, s->stc, P.l[NL_STC], st);
  const double *src[] = {s->t1, s->cmc, s->sneqv, s->snowh, s->sndens, s->ch, s->cm, s->snotime1,
                         s->albedo, s->emissi, s->q1, s->ribb, s->fcr};
  const int dst[] = {NS_T1, NS_CMC, NS_SNEQV, NS_SNOWH, NS_SNDENS, NS_CH, NS_CM, NS_SNOTIME1,
                     NS_ALBEDO, NS_EMISSI, NS_Q1, NS_RIBB, NS_FCR};
  for (int k = 0; k < 13; k++) rc = rc ?: upload_scalar(perm, ne, src[k], P.s[dst[k]], st);
  int64_t launches = 0;
  return rc ?: launch_inputs(n, st, &launches) ?: cuda_rc(cudaStreamSynchronize(st));
}

int noah_build(const pihm_noah_params *p, const pihm_noah_state *s, const int32_t *perm, int ne,
               const NoahTargets &tg, cudaStream_t st, NoahInstance *out) {
  if (!p || !s || !out || p->nelem != ne || !p->nsoil || !p->sldpth || !p->nroot || !p->rtdis) return PIHM_GPU_ERR_ARG;
  for (int r = 0; r < ne; r++) {
    // HRT and SRT read the second layer: at least two
    if (p->nsoil[r] < 2 || p->nsoil[r] > noah::L || p->nroot[r] < 1 || p->nroot[r] > p->nsoil[r])
      return PIHM_GPU_ERR_ARG;
  }
  const double *params[] = {p->smcmax, p->smcmin, p->smcref, p->smcwlt, p->smcdry, p->quartz, p->csoil,
                            p->alpha, p->beta, p->ksatv, p->porosity, p->depth, p->area, p->shdfac,
                            p->cmcfactr, p->laimax, p->laimin, p->emissmax, p->emissmin, p->albedomax,
                            p->albedomin, p->z0max, p->z0min, p->snup, p->cfactr, p->rgl, p->rsmin,
                            p->rsmax, p->topt, p->hs, p->sbeta, p->salp, p->frzx, p->fxexp, p->czil,
                            p->lvcoef, p->zbot, p->tbot, p->zlvl, p->zlvl_wind, p->snoalb};
  constexpr int kParams = NS_SNOALB + 1;
  static_assert(sizeof(params) / sizeof(params[0]) == kParams, "parameter list");
  for (const double *q : params)
    if (!q) return PIHM_GPU_ERR_ARG;
  if (!s->smc || !s->sh2o || !s->stc || !s->t1 || !s->cmc || !s->sneqv || !s->snowh || !s->sndens || !s->ch ||
      !s->cm || !s->snotime1 || !s->albedo || !s->emissi || !s->q1 || !s->ribb || !s->fcr)
    return PIHM_GPU_ERR_ARG;
  const size_t NE = ne;
  const size_t bytes = NS_COUNT * padded<double>(NE) + NL_COUNT * padded<double>(noah::L * NE) +
                       NI_COUNT * padded<int32_t>(NE) + padded<int32_t>(NE) + padded<int32_t>(2 * kNoahClasses);
  NoahInstance n;
  if (cudaMalloc(&n.alloc, bytes) != cudaSuccess) return PIHM_GPU_ERR_NOMEM;
  n.P = new NoahPlanes();
  n.tg = tg;
  n.ne = ne;
  n.first = 1;
  if (cudaMemset(n.alloc, 0, bytes) != cudaSuccess) {
    noah_release(n);
    return PIHM_GPU_ERR_CUDA;
  }
  NoahPlanes &P = *n.P;
  P.ne = ne;
  char *cur = (char *)n.alloc;
  for (int k = 0; k < NS_COUNT; k++) {
    P.s[k] = (double *)cur;
    cur += padded<double>(NE);
  }
  for (int k = 0; k < NL_COUNT; k++) {
    P.l[k] = (double *)cur;
    cur += padded<double>(noah::L * NE);
  }
  for (int k = 0; k < NI_COUNT; k++) {
    P.i[k] = (int32_t *)cur;
    cur += padded<int32_t>(NE);
  }
  P.order = (int32_t *)cur;
  cur += padded<int32_t>(NE);
  P.cls = (int32_t *)cur;
  int rc = PIHM_GPU_OK;
  for (int k = 0; k < kParams && !rc; k++) rc = upload_scalar(perm, ne, params[k], P.s[k], st);
  // layer depths below the surface (DefSldpth, noah/lsm_func.c:152-156)
  std::vector<double> zsoil((size_t)noah::L * ne, 0.0);
  for (int r = 0; r < ne; r++) {
    const double *sl = p->sldpth + (size_t)noah::L * r;
    double *z = zsoil.data() + (size_t)noah::L * r;
    z[0] = -sl[0];
    for (int k = 1; k < p->nsoil[r]; k++) z[k] = -sl[k] + z[k - 1];
  }
  rc = rc ?: upload_layers(perm, ne, p->sldpth, P.l[NL_SLDPTH], st);
  rc = rc ?: upload_layers(perm, ne, zsoil.data(), P.l[NL_ZSOIL], st);
  rc = rc ?: upload_layers(perm, ne, p->rtdis, P.l[NL_RTDIS], st);
  rc = rc ?: upload_int(perm, ne, p->nsoil, P.i[NI_NSOIL]);
  rc = rc ?: upload_int(perm, ne, p->nroot, P.i[NI_NROOT]);
  if (p->isurban) rc = rc ?: upload_int(perm, ne, p->isurban, P.i[NI_ISURBAN]);
  // the water-table layer before the first post-step: below the column
  std::vector<int32_t> nw((size_t)ne);
  for (int r = 0; r < ne; r++) nw[r] = p->nsoil[r];
  rc = rc ?: upload_int(perm, ne, nw.data(), P.i[NI_NWTBL]);
  rc = rc ?: noah_set_state(n, s, perm, st);
  if (rc) {
    noah_release(n);
    return rc;
  }
  *out = n;
  return PIHM_GPU_OK;
}

int noah_set_forcing(NoahInstance &n, const pihm_noah_forcing *f, const int32_t *perm, cudaStream_t st) {
  if (!n.alloc || !f || !f->prcp || !f->sfctmp || !f->rh || !f->sfcspd || !f->soldn || !f->longwave ||
      !f->sfcprs || !f->lai)
    return PIHM_GPU_ERR_ARG;
  NoahPlanes &P = *n.P;
  const double *src[] = {f->prcp, f->sfctmp, f->rh, f->sfcspd, f->soldn, f->longwave, f->sfcprs, f->lai};
  int rc = PIHM_GPU_OK;
  for (int k = 0; k < 8 && !rc; k++) rc = upload_scalar(perm, n.ne, src[k], P.s[NS_PRCP + k], st);
  return rc;
}

int noah_launch_step(NoahInstance &n, double dt, unsigned int *err, cudaStream_t st, int64_t *launches) {
  if (!n.alloc || !(dt > 0.0)) return PIHM_GPU_ERR_ARG;
  if (n.ne == 0) return PIHM_GPU_OK;
  if (cudaMemsetAsync(n.P->cls, 0, sizeof(int32_t) * 2 * kNoahClasses, st) != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  k_noah_count<<<(n.ne + 255) / 256, 256, 0, st>>>(*n.P);
  k_noah_place<<<(n.ne + 255) / 256, 256, 0, st>>>(*n.P);
  k_noah_step<<<(n.ne + kNoahBlock - 1) / kNoahBlock, kNoahBlock, 0, st>>>(*n.P, dt, err);
  *launches += 3;
  return cuda_rc(cudaGetLastError()) ?: launch_inputs(n, st, launches);
}

int noah_launch_begin(NoahInstance &n, const double *y0, cudaStream_t st, int64_t *launches) {
  if (!n.alloc || !y0) return PIHM_GPU_ERR_ARG;
  k_noah_begin<<<(n.ne + 255) / 256, 256, 0, st>>>(*n.P, y0);
  n.first = 0;
  ++*launches;
  return cuda_rc(cudaGetLastError());
}

int noah_launch_post(NoahInstance &n, const double *y, double dt, cudaStream_t st, int64_t *launches) {
  if (!n.alloc || !y || !(dt > 0.0)) return PIHM_GPU_ERR_ARG;
  k_noah_post<<<(n.ne + kNoahBlock - 1) / kNoahBlock, kNoahBlock, 0, st>>>(*n.P, n.tg, y, dt, n.first);
  n.first = 0;
  ++*launches;
  return cuda_rc(cudaGetLastError()) ?: launch_inputs(n, st, launches);
}

int noah_get(NoahInstance &n, int field, const int32_t *perm, cudaStream_t st, double *out) {
  if (!n.alloc || !out || field < 0 || field >= PIHM_NOAH_NFIELDS) return PIHM_GPU_ERR_ARG;
  const NoahPlanes &P = *n.P;
  const int ne = n.ne;
  if (cudaStreamSynchronize(st) != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  static const int layer_of[] = {NL_SMC, NL_SH2O, NL_STC, NL_ET, NL_RUNOFF2_LYR, NL_SMFLXV};
  if (field < 6) {
    std::vector<double> h((size_t)noah::L * ne);
    if (cudaMemcpy(h.data(), P.l[layer_of[field]], sizeof(double) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
      return PIHM_GPU_ERR_CUDA;
    for (int k = 0; k < noah::L; k++)
      for (int i = 0; i < ne; i++) out[(size_t)noah::L * perm[i] + k] = h[(size_t)k * ne + i];
    return PIHM_GPU_OK;
  }
  static const int scalar_of[] = {NS_T1, NS_CMC, NS_SNEQV, NS_SNOWH, NS_SNDENS, NS_CH, NS_CM, NS_ALBEDO,
                                  NS_EMISSI, NS_Q1, NS_FCR, NS_EDIR, NS_EC, NS_ETT, NS_ESNOW, NS_ETP,
                                  NS_DRIP, NS_PCPDRP, NS_SNOMLT, NS_SSOIL, NS_SHEAT, NS_RUNOFF2, NS_RUNOFF3,
                                  NS_INFIL, -1, NS_SNOTIME1, NS_SNCOVR, NS_BETA_S, NS_ETA, NS_SOILM};
  const int idx = field - PIHM_NOAH_T1;
  if (field < PIHM_NOAH_T1 || idx >= (int)(sizeof(scalar_of) / sizeof(int))) return PIHM_GPU_ERR_ARG;
  std::vector<double> h((size_t)ne);
  if (scalar_of[idx] < 0) {  // nwtbl
    std::vector<int32_t> w((size_t)ne);
    if (cudaMemcpy(w.data(), P.i[NI_NWTBL], sizeof(int32_t) * ne, cudaMemcpyDeviceToHost) != cudaSuccess)
      return PIHM_GPU_ERR_CUDA;
    for (int i = 0; i < ne; i++) h[i] = w[i];
  } else if (cudaMemcpy(h.data(), P.s[scalar_of[idx]], sizeof(double) * ne, cudaMemcpyDeviceToHost) !=
             cudaSuccess) {
    return PIHM_GPU_ERR_CUDA;
  }
  for (int i = 0; i < ne; i++) out[perm[i]] = h[i];
  return PIHM_GPU_OK;
}

void noah_release(NoahInstance &n) {
  if (n.alloc) cudaFree(n.alloc);
  delete n.P;
  n = NoahInstance();
}

}  // namespace pihm

using namespace pihm;

extern "C" int pihm_gpu_noah_set_state(pihm_gpu_ctx *c, const pihm_noah_state *s) {
  if (!c || !c->noahlsm.alloc || !s) return PIHM_GPU_ERR_ARG;
  return noah_set_state(c->noahlsm, s, c->h_perm, c->stream);
}

extern "C" int pihm_gpu_noah_init(pihm_gpu_ctx *c, const pihm_noah_params *p, const pihm_noah_state *s) {
  if (!c || !p || !s || p->nelem != c->ne) return PIHM_GPU_ERR_ARG;
  const size_t NE = c->ne;
  // the right-hand side's Flux-PIHM input planes
  if (!c->d_noah) {
    const size_t nb = 3 * padded<double>(NE) + padded<int32_t>(NE);
    if (cudaMalloc(&c->d_noah, nb) != cudaSuccess) {
      c->d_noah = nullptr;
      return PIHM_GPU_ERR_NOMEM;
    }
    char *q = (char *)c->d_noah;
    c->m.noah_etgw = (double *)q; q += padded<double>(NE);
    c->m.noah_satn = (double *)q; q += padded<double>(NE);
    c->m.noah_fcr = (double *)q; q += padded<double>(NE);
    c->m.noah_wtin = (int32_t *)q;
  }
  NoahTargets tg{c->m.d_sub, c->m.d_et, (int64_t)c->ne, const_cast<double *>(c->m.noah_etgw),
                 const_cast<double *>(c->m.noah_satn), const_cast<double *>(c->m.noah_fcr),
                 const_cast<double *>(c->m.edir), const_cast<double *>(c->m.ett), const_cast<double *>(c->m.pcpdrp),
                 const_cast<int32_t *>(c->m.noah_wtin)};
  noah_release(c->noahlsm);
  const int rc = noah_build(p, s, c->h_perm, c->ne, tg, c->stream, &c->noahlsm);
  if (rc != PIHM_GPU_OK) return rc;
  c->m.noah = 1;
  c->diag = 1;  // MassBalance reads the last evaluation's fluxes
  return PIHM_GPU_OK;
}

extern "C" int pihm_gpu_noah_set_forcing(pihm_gpu_ctx *c, const pihm_noah_forcing *f) {
  if (!c || !c->noahlsm.alloc) return PIHM_GPU_ERR_ARG;
  return noah_set_forcing(c->noahlsm, f, c->h_perm, c->stream);
}

extern "C" int pihm_gpu_noah_step(pihm_gpu_ctx *c, double dt) {
  if (!c || !c->noahlsm.alloc) return PIHM_GPU_ERR_ARG;
  int64_t n = 0;
  const int rc = noah_launch_step(c->noahlsm, dt, c->m.err, c->stream, &n);
  c->launches += n;
  return rc;
}

extern "C" int pihm_gpu_noah_begin(pihm_gpu_ctx *c, const double *y0_dev) {
  if (!c || !c->noahlsm.alloc) return PIHM_GPU_ERR_ARG;
  int64_t n = 0;
  const int rc = noah_launch_begin(c->noahlsm, y0_dev, c->stream, &n);
  c->launches += n;
  return rc;
}

extern "C" int pihm_gpu_noah_post_step(pihm_gpu_ctx *c, const double *y_dev, double stepsize) {
  if (!c || !c->noahlsm.alloc) return PIHM_GPU_ERR_ARG;
  int64_t n = 0;
  const int rc = noah_launch_post(c->noahlsm, y_dev, stepsize, c->stream, &n);
  c->launches += n;
  return rc;
}

extern "C" int pihm_gpu_noah_get(pihm_gpu_ctx *c, int field, double *out) {
  if (!c || !c->noahlsm.alloc) return PIHM_GPU_ERR_ARG;
  return noah_get(c->noahlsm, field, c->h_perm, c->stream, out);
}
