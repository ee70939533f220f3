// Land-surface step on the device (include/pihm_land.h): ApplyForc's
// interpolation of the forcing series and IntcpSnowEt's snow, interception
// and evapotranspiration, one thread per element, writing the right-hand
// side's forcing planes in place.
//
// Numerics.  This file is compiled without multiply-add contraction
// (-fmad=false), so every product and sum rounds where the reference's C
// rounds; divisions and square roots are IEEE.  exp, log and pow go through
// the table-driven double-double routines of fp64_math.cuh (about 0.51 ulp,
// almost always the correctly rounded value the C library returns too);
// pow(x, 2) is x * x, the correctly rounded square; cos is CUDA's.  So the
// step reproduces the reference's values to the last bit on nearly every
// element, and within a few ulps of the affected terms elsewhere.
//
// Work is split by what it depends on: k_land_station interpolates each
// station's record and forms everything that depends on it alone (vapour
// pressure, snow fraction, melt, the temperature powers) once per station;
// k_land_month forms the aerodynamic term log(z/z0) log(10 z/z0) of every
// element when the month changes; k_land_step does the per-element rest,
// each value formed with the reference's operations in its order, so the
// split changes no result.
#include <cstdio>
#include <cstring>
#include <ctime>
#include <vector>

#include "fp64_math.cuh"
#include "land_tables.h"
#include "pihm_internal.h"
#include "pihm_land.h"

namespace pihm {

namespace {

__device__ const double g_monthly_lai[PIHM_LAND_NLC * 12] = {PIHM_MONTHLY_LAI};
__device__ const double g_monthly_rl[PIHM_LAND_NLC * 12] = {PIHM_MONTHLY_ROUGHNESS};
__device__ const double g_melt_factor[12] = {PIHM_MELT_FACTOR};

// Constants of IntcpSnowEt (src/is_sm_et.c:9-11) and of the model
// (src/include/pihm_const.h:9-15).
constexpr double kTSnow = -3.0, kTRain = 1.0, kT0 = 0.0;
constexpr double kCp = 1004.0, kLvH2O = 2.501e6, kSigma = 5.67e-8, kRd = 287.04, kRv = 461.5;

constexpr int kLandBlock = 256;

__device__ __forceinline__ double exp_l(double x) {
  double r;
  return exp_dd_checked(x, 0.0, r) ? r : exp(x);
}
__device__ __forceinline__ double log_l(double x) {
  double sh, lo;
  return log_dd_fast(x, sh, lo) ? sh + lo : log(x);
}

// IntrplForc's bisection (src/forcing.c:503-528): the knot `middle` with
// T[middle-1] <= t <= T[middle], or -1.  The host has checked that t lies in
// every series, whose times are non-decreasing, so the search ends in at most
// log2(len) + 1 rounds with a knot.
__device__ __forceinline__ int bracket(const int64_t *__restrict__ T, int len, int64_t t) {
  int first = 1, last = len - 1;
  while (first <= last) {
    const int middle = (first + last) >> 1;
    if (t >= __ldg(&T[middle - 1]) && t <= __ldg(&T[middle])) return middle;
    if (__ldg(&T[middle]) > t)
      last = middle - 1;
    else
      first = middle + 1;
  }
  return -1;
}

// The linear interpolation of IntrplForc (src/forcing.c:512-517), in its
// operation order.
__device__ __forceinline__ double lerp(const int64_t *__restrict__ T, const double *__restrict__ D, int nvar,
                                       int k, int var, int64_t t) {
  const int64_t t0 = __ldg(&T[k - 1]), t1 = __ldg(&T[k]);
  const double d0 = __ldg(&D[(size_t)(k - 1) * nvar + var]), d1 = __ldg(&D[(size_t)k * nvar + var]);
  return ((double)(t1 - t) * d0 + (double)(t - t0) * d1) / (double)(t1 - t0);
}

// Station values (ApplyMeteoForc's record, src/forcing.c:343-356, and the
// parts of IntcpSnowEt that depend on it alone), per station and step.
enum StationVal {
  SV_PRCP = 0,   // prcp / 1000 (m s-1)
  SV_TC,         // air temperature - 273.15 (C)
  SV_RH,         // relative humidity / 100
  SV_WIND016,    // wind speed * 0.16
  SV_SOLDN,      // solar radiation, negative as 0
  SV_VP,         // vapour pressure 611.2 exp(17.67 T / (T + 243.5)) rh
  SV_VPRH,       // vp / rh
  SV_GAMMAS,     // 1 / (1 + 0.00025 (vp / rh - vp)), at least 0.01
  SV_FRAC_SNOW,  // snow fraction of precipitation
  SV_MELT,       // degree-day melt rate before the snow store limits it
  SV_CGAMMA,     // 4 0.7 SIGMA RD / CP (T + 273.15)^4
  SV_CDELTA,     // LVH2O^2 0.622 / RV / CP / (T + 273.15)^2
  kStationVals
};

// One thread per station (then one per LAI series): the interpolation of
// IntrplForc and the station-only sub-expressions of IntcpSnowEt
// (src/is_sm_et.c:49-56, 70-77, 97-100, 149-150), in the reference's order.
__global__ void k_land_station(LandDev L, int64_t t, int month) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const double nan = __longlong_as_double(0x7ff8000000000000LL);
  if (k < L.nmeteo) {
    const int off = L.meteo_off[k];
    const int64_t *mt = L.meteo_time + off;
    const double *md = L.meteo_data + (size_t)off * PIHM_METEO_NVAR;
    const int km = bracket(mt, L.meteo_len[k], t);
    double prcp = nan, tk_in = nan, rh_pct = nan, wind = nan, soldn = nan;
    if (km > 0) {
      prcp = lerp(mt, md, PIHM_METEO_NVAR, km, PIHM_METEO_PRCP, t) / 1000.0;
      tk_in = lerp(mt, md, PIHM_METEO_NVAR, km, PIHM_METEO_SFCTMP, t);
      rh_pct = lerp(mt, md, PIHM_METEO_NVAR, km, PIHM_METEO_RH, t);
      wind = lerp(mt, md, PIHM_METEO_NVAR, km, PIHM_METEO_SFCSPD, t);
      soldn = lerp(mt, md, PIHM_METEO_NVAR, km, PIHM_METEO_SOLAR, t);
    }
    soldn = (soldn > 0.0) ? soldn : 0.0;
    const double sfctmp = tk_in - 273.15;
    const double rh = rh_pct / 100.0;
    const double vp = 611.2 * exp_l(17.67 * sfctmp / (sfctmp + 243.5)) * rh;
    const double vprh = vp / rh;
    double gammas = 1.0 / (1.0 + 0.00025 * (vp / rh - vp));
    gammas = (gammas < 0.01) ? 0.01 : gammas;
    const double frac_snow =
        (sfctmp < kTSnow) ? 1.0 : ((sfctmp > kTRain) ? 0.0 : (kTRain - sfctmp) / (kTRain - kTSnow));
    const double melt = (sfctmp > kT0) ? (sfctmp - kT0) * g_melt_factor[month] : 0.0;
    const double tk = sfctmp + 273.15;
    double *o = L.station + (size_t)k * kStationVals;
    o[SV_PRCP] = prcp;
    o[SV_TC] = sfctmp;
    o[SV_RH] = rh;
    o[SV_WIND016] = wind * 0.16;
    o[SV_SOLDN] = soldn;
    o[SV_VP] = vp;
    o[SV_VPRH] = vprh;
    o[SV_GAMMAS] = gammas;
    o[SV_FRAC_SNOW] = frac_snow;
    o[SV_MELT] = melt;
    o[SV_CGAMMA] = 4.0 * 0.7 * kSigma * kRd / kCp * pow_fast(tk, 4.0);
    o[SV_CDELTA] = kLvH2O * kLvH2O * 0.622 / kRv / kCp / (tk * tk);
  } else if (k < L.nmeteo + L.nlai) {
    const int s = k - L.nmeteo;
    const int off = L.lai_off[s];
    const int kl = bracket(L.lai_time + off, L.lai_len[s], t);
    L.lai_value[s] = kl > 0 ? lerp(L.lai_time + off, L.lai_data + off, 1, kl, 0, t) : nan;
  }
}

// log(zlvl / z0) log(10 zlvl / z0) of every element for a month (z0 from the
// monthly roughness table), the numerator of the aerodynamic resistance
// (src/is_sm_et.c:93-96); recomputed when the month changes.
__global__ void __launch_bounds__(kLandBlock) k_land_month(LandDev L, int ne, int month) {
  const int i = blockIdx.x * kLandBlock + threadIdx.x;
  if (i >= ne) return;
  const double z0 = g_monthly_rl[(__ldg(&L.lc[i]) - 1) * 12 + month];
  const double zlvl = __ldg(&L.zlvl[i]);
  L.ra_num[i] = log_l(zlvl / z0) * log_l(10.0 * zlvl / z0);
}

__global__ void __launch_bounds__(kLandBlock) k_land_step(LandDev L, const double *__restrict__ y, int ne,
                                                          int month, double dt) {
  const int i = blockIdx.x * kLandBlock + threadIdx.x;
  if (i >= ne) return;
  const double *sv = L.station + (size_t)(__ldg(&L.meteo[i]) - 1) * kStationVals;
  const int lc = __ldg(&L.lc[i]) - 1;
  const int lt = __ldg(&L.lai_type[i]);
  const double lai = lt > 0 ? L.lai_value[lt - 1] : g_monthly_lai[lc * 12 + month];

  // ---- IntcpSnowEt (src/is_sm_et.c:46-224) ----
  const double prcp = sv[SV_PRCP];
  const double sfctmp = sv[SV_TC];
  const double radnet = sv[SV_SOLDN] * (1.0 - __ldg(&L.albedo[i]));
  const double vp = sv[SV_VP];
  const double pres = __ldg(&L.pres[i]);
  const double qv = div_any(0.622 * vp, pres);
  const double qvsat = div_any(0.622 * sv[SV_VPRH], pres);

  // snow accumulation and melt
  const double frac_snow = sv[SV_FRAC_SNOW];
  double sneqv = L.sneqv[i];
  sneqv += frac_snow * prcp * dt;
  double melt_rate = sv[SV_MELT];
  if (sneqv > melt_rate * dt) {
    sneqv -= melt_rate * dt;
  } else {
    melt_rate = div_any(sneqv, dt);
    sneqv = 0.0;
  }

  // potential evaporation (Penman-Monteith)
  const double shdfac = __ldg(&L.shdfac[i]);
  const double intcp_max = __ldg(&L.cmcfactr[i]) * lai * shdfac;
  const double ra = div_any(L.ra_num[i], sv[SV_WIND016]);
  const double gamma = div_any(sv[SV_CGAMMA], div_any(pres, ra)) + 1.0;
  const double delta = sv[SV_CDELTA] * qvsat;
  const double etp = div_any(radnet * delta + gamma * div_any(1.2 * kLvH2O * (qvsat - qv), ra),
                             1000.0 * kLvH2O * (delta + gamma));

  // soil evaporation
  const double depth = __ldg(&L.depth[i]);
  const double unsat = y[ne + i], gw = y[2 * ne + i];
  double satn;
  if (depth - gw < __ldg(&L.rzd[i])) {
    satn = 1.0;
  } else {
    const double r = div_any(unsat, depth - gw);
    satn = (r > 1.0) ? 1.0 : ((r < 0.0) ? 0.0 : 0.5 * (1.0 - cos(3.14 * r)));
  }
  double betas = div_any(satn * __ldg(&L.porosity[i]) + __ldg(&L.smcmin[i]) - __ldg(&L.smcwlt[i]), __ldg(&L.dsmc[i]));
  betas = (betas < 0.0001) ? 0.0001 : ((betas > 1.0) ? 1.0 : betas);
  double edir = (1.0 - shdfac) * (betas * betas) * etp;
  edir *= L.cal_edir;
  edir = (edir < 0.0) ? 0.0 : edir;

  // canopy evaporation, transpiration and drip
  double cmc = L.cmc[i];
  double ec, ett, drip;
  if (lai > 0.0) {
    const double cfactr = __ldg(&L.cfactr[i]);
    const double cm = (cmc < 0.0) ? 0.0 : ((cmc > intcp_max) ? intcp_max : cmc);
    // ec divides the clamped storage by intcp_max; ett's expression divides
    // only the unclamped branch (src/is_sm_et.c:128-131, 164-168)
    const double base_ec = div_any(cm, intcp_max);
    const double base_ett = (cmc < 0.0) ? 0.0 : base_ec;
    const double pw_ec = pow_fast(base_ec, cfactr);
    const double pw_ett = (__double_as_longlong(base_ett) == __double_as_longlong(base_ec)) ? pw_ec
                                                                                           : pow_fast(base_ett, cfactr);
    ec = shdfac * pw_ec * etp;
    ec *= L.cal_ec;
    ec = (ec < 0.0) ? 0.0 : ec;

    double fr = div_any(1.1 * radnet, __ldg(&L.rgl[i]) * lai);
    fr = (fr < 0.0) ? 0.0 : fr;
    double alphar = div_any(1.0 + fr, fr + __ldg(&L.rs_ratio[i]));
    alphar = (alphar > 10000.0) ? 10000.0 : alphar;
    const double dtopt = __ldg(&L.topt_c[i]) - sfctmp;
    double etas = 1.0 - 0.0016 * (dtopt * dtopt);
    etas = (etas < 0.0001) ? 0.0001 : etas;
    const double gammas = sv[SV_GAMMAS];
    const double rsmax = __ldg(&L.rsmax[i]);
    double rs = div_any(__ldg(&L.rsmin[i]) * alphar, betas * lai * etas * gammas);
    rs = (rs > rsmax) ? rsmax : rs;
    const double dg = div_any(delta, gamma);  // the reference forms it twice
    const double pc = div_any(1.0 + dg, 1.0 + div_any(rs, ra) + dg);
    ett = shdfac * pc * (1.0 - pw_ett) * etp;
    ett *= L.cal_ett;
    ett = (ett < 0.0) ? 0.0 : ett;
    ett = ((gw < __ldg(&L.d_rzd[i])) && unsat <= 0.0) ? 0.0 : ett;
    // Rutter and Morton (1977): D0 = 6.52e-7 m s-1
    drip = (cmc <= 0.0) ? 0.0 : 6.52E-7 * intcp_max * exp_l(div_any(3.89 * cmc, intcp_max));
  } else {
    ett = 0.0;
    ec = 0.0;
    drip = 0.0;
  }
  if (drip < 0.0) drip = 0.0;
  if (drip * dt > cmc) drip = div_any(cmc, dt);

  const double isval = cmc + (1.0 - frac_snow) * prcp * shdfac * dt - ec * dt - drip * dt;
  if (isval > intcp_max) {
    cmc = intcp_max;
    drip += div_any(isval - intcp_max, dt);
  } else if (isval < 0.0) {
    cmc = 0.0;
    if (ec + drip > 0.0) {
      ec = div_any(ec, ec + drip) * (cmc + (1.0 - frac_snow) * prcp * shdfac * dt);
      drip = div_any(drip, ec + drip) * (cmc + (1.0 - frac_snow) * prcp * shdfac * dt);
    }
  } else {
    cmc = isval;
  }
  const double pcpdrp = (1.0 - shdfac) * (1.0 - frac_snow) * prcp + drip + melt_rate;

  L.cmc[i] = cmc;
  L.sneqv[i] = sneqv;
  L.prcp[i] = prcp;
  L.ec[i] = ec;
  L.drip[i] = drip;
  L.pcpdrp[i] = pcpdrp;
  L.edir[i] = edir;
  L.ett[i] = ett;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

int cuda_rc(cudaError_t e) { return e == cudaSuccess ? PIHM_GPU_OK : PIHM_GPU_ERR_CUDA; }

// Series checks of pihm_gpu_land_init: at least two knots, non-decreasing
// times; widens [lo, hi] to the times every series covers.
bool series_ok(int32_t n, const int32_t *len, const int64_t *time, int64_t *lo, int64_t *hi, size_t *knots) {
  size_t off = 0;
  for (int32_t k = 0; k < n; k++) {
    if (len[k] < 2) return false;
    for (int32_t j = 1; j < len[k]; j++)
      if (time[off + j] < time[off + j - 1]) return false;
    *lo = std::max(*lo, time[off]);
    *hi = std::min(*hi, time[off + len[k] - 1]);
    off += (size_t)len[k];
  }
  *knots = off;
  return true;
}

}  // namespace

}  // namespace pihm

using namespace pihm;

namespace pihm {

int land_build(const pihm_land_params *p, const pihm_forcing_series *s, const int32_t *perm, int ne,
               const double *zmax, const LandTargets &tg, LandInstance *out) {
  if (!p || !s || !out || p->nelem != ne || s->nmeteo < 1 || s->nlai < 0) return PIHM_GPU_ERR_ARG;
  const double *planes[] = {p->albedomin, p->albedomax, p->shdfac, p->cmcfactr, p->cfactr, p->rgl,
                            p->rsmin,     p->rsmax,     p->topt,   p->smcmin,   p->smcwlt, p->smcref,
                            p->zlvl_wind};
  for (const double *q : planes)
    if (!q) return PIHM_GPU_ERR_ARG;
  if (!p->lc_type || !p->meteo_type || !p->lai_type || !s->meteo_len || !s->meteo_time || !s->meteo_data ||
      (s->nlai > 0 && (!s->lai_len || !s->lai_time || !s->lai_data)))
    return PIHM_GPU_ERR_ARG;
  for (int r = 0; r < ne; r++)
    if (p->lc_type[r] < 1 || p->lc_type[r] > PIHM_LAND_NLC || p->meteo_type[r] < 1 ||
        p->meteo_type[r] > s->nmeteo || p->lai_type[r] < 0 || p->lai_type[r] > s->nlai)
      return PIHM_GPU_ERR_ARG;
  int64_t lo = INT64_MIN, hi = INT64_MAX;
  size_t nmk = 0, nlk = 0;
  if (!series_ok(s->nmeteo, s->meteo_len, s->meteo_time, &lo, &hi, &nmk) ||
      !series_ok(s->nlai, s->lai_len, s->lai_time, &lo, &hi, &nlk))
    return PIHM_GPU_ERR_ARG;
  if (nmk > (size_t)INT32_MAX || nlk > (size_t)INT32_MAX) return PIHM_GPU_ERR_ARG;

  // host planes in internal order, the derived ones with the reference's
  // operations (see LandDev)
  const size_t NE = ne;
  std::vector<double> hd[14];
  for (auto &v : hd) v.resize(NE);
  std::vector<int32_t> hi32[3];
  for (auto &v : hi32) v.resize(NE);
  for (int i = 0; i < ne; i++) {
    const int r = perm[i];
    hd[0][i] = 0.5 * (p->albedomin[r] + p->albedomax[r]);
    hd[1][i] = p->shdfac[r];
    hd[2][i] = p->cmcfactr[r];
    hd[3][i] = p->cfactr[r];
    hd[4][i] = p->rgl[r];
    hd[5][i] = p->rsmin[r];
    hd[6][i] = p->rsmin[r] / p->rsmax[r];
    hd[7][i] = p->rsmax[r];
    hd[8][i] = p->topt[r] - 273.15;
    hd[9][i] = p->smcmin[r];
    hd[10][i] = p->smcwlt[r];
    hd[11][i] = p->smcref[r] - p->smcwlt[r];
    hd[12][i] = p->zlvl_wind[r];
    hi32[0][i] = p->lc_type[r];
    hi32[1][i] = p->meteo_type[r];
    hi32[2][i] = p->lai_type[r];
  }
  for (int i = 0; i < ne; i++) hd[13][i] = 101.325 * 1.0e3 * std::pow((293.0 - 0.0065 * zmax[i]) / 293.0, 5.26);
  std::vector<int32_t> moff(s->nmeteo), loff(s->nlai > 0 ? s->nlai : 1);
  {
    int32_t o = 0;
    for (int k = 0; k < s->nmeteo; k++) moff[k] = o, o += s->meteo_len[k];
    o = 0;
    for (int k = 0; k < s->nlai; k++) loff[k] = o, o += s->lai_len[k];
  }

  // one allocation: parameters, series, state and outputs
  const size_t nm = (size_t)s->nmeteo, nl = (size_t)(s->nlai > 0 ? s->nlai : 1);
  const size_t bytes = 14 * align256(NE * 8) + 3 * align256(NE * 4) + 2 * align256(nm * 4) + 2 * align256(nl * 4) +
                       align256(nmk * 8) + align256(nmk * 8 * PIHM_METEO_NVAR) + align256((nlk ? nlk : 1) * 8) +
                       align256((nlk ? nlk : 1) * 8) + 5 * align256(NE * 8) + align256(nm * 8 * kStationVals) +
                       align256(nl * 8) + align256(NE * 8);
  void *alloc = nullptr;
  if (cudaMalloc(&alloc, bytes) != cudaSuccess) return PIHM_GPU_ERR_NOMEM;
  char *cur = (char *)alloc;
  auto take = [&](size_t b) {
    char *r = cur;
    cur += align256(b);
    return r;
  };
  LandDev L{};
  double *dd[14];
  for (int k = 0; k < 14; k++) dd[k] = (double *)take(NE * 8);
  int32_t *di[3];
  for (int k = 0; k < 3; k++) di[k] = (int32_t *)take(NE * 4);
  int32_t *d_moff = (int32_t *)take(nm * 4), *d_mlen = (int32_t *)take(nm * 4);
  int32_t *d_loff = (int32_t *)take(nl * 4), *d_llen = (int32_t *)take(nl * 4);
  int64_t *d_mt = (int64_t *)take(nmk * 8);
  double *d_md = (double *)take(nmk * 8 * PIHM_METEO_NVAR);
  int64_t *d_lt = (int64_t *)take((nlk ? nlk : 1) * 8);
  double *d_ld = (double *)take((nlk ? nlk : 1) * 8);
  double *state[5];
  for (int k = 0; k < 5; k++) state[k] = (double *)take(NE * 8);
  double *d_station = (double *)take(nm * 8 * kStationVals);
  double *d_laival = (double *)take(nl * 8);
  double *d_ranum = (double *)take(NE * 8);

  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 14 && e == cudaSuccess; k++) e = cudaMemcpy(dd[k], hd[k].data(), NE * 8, cudaMemcpyHostToDevice);
  for (int k = 0; k < 3 && e == cudaSuccess; k++) e = cudaMemcpy(di[k], hi32[k].data(), NE * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_moff, moff.data(), nm * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_mlen, s->meteo_len, nm * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_mt, s->meteo_time, nmk * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_md, s->meteo_data, nmk * 8 * PIHM_METEO_NVAR, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && s->nlai > 0) {
    e = cudaMemcpy(d_loff, loff.data(), nl * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_llen, s->lai_len, nl * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_lt, s->lai_time, nlk * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_ld, s->lai_data, nlk * 8, cudaMemcpyHostToDevice);
  }
  for (int k = 0; k < 5 && e == cudaSuccess; k++) e = cudaMemset(state[k], 0, NE * 8);
  if (e != cudaSuccess) {
    cudaFree(alloc);
    return PIHM_GPU_ERR_CUDA;
  }
  L.albedo = dd[0];
  L.shdfac = dd[1];
  L.cmcfactr = dd[2];
  L.cfactr = dd[3];
  L.rgl = dd[4];
  L.rsmin = dd[5];
  L.rs_ratio = dd[6];
  L.rsmax = dd[7];
  L.topt_c = dd[8];
  L.smcmin = dd[9];
  L.smcwlt = dd[10];
  L.dsmc = dd[11];
  L.zlvl = dd[12];
  L.pres = dd[13];
  L.lc = di[0];
  L.meteo = di[1];
  L.lai_type = di[2];
  L.depth = tg.depth;
  L.porosity = tg.porosity;
  L.rzd = tg.rzd;
  L.d_rzd = tg.d_rzd;
  L.cal_edir = p->cal_edir;
  L.cal_ec = p->cal_ec;
  L.cal_ett = p->cal_ett;
  L.meteo_off = d_moff;
  L.meteo_len = d_mlen;
  L.lai_off = d_loff;
  L.lai_len = d_llen;
  L.meteo_time = d_mt;
  L.meteo_data = d_md;
  L.lai_time = d_lt;
  L.lai_data = d_ld;
  L.cmc = state[0];
  L.sneqv = state[1];
  L.prcp = state[2];
  L.ec = state[3];
  L.drip = state[4];
  L.station = d_station;
  L.lai_value = d_laival;
  L.ra_num = d_ranum;
  L.nmeteo = s->nmeteo;
  L.nlai = s->nlai;
  L.pcpdrp = tg.pcpdrp;
  L.edir = tg.edir;
  L.ett = tg.ett;
  out->alloc = alloc;
  out->L = L;
  out->t_lo = lo;
  out->t_hi = hi;
  out->month = -1;
  out->ne = ne;
  return PIHM_GPU_OK;
}

int land_set_state(LandInstance &li, const int32_t *perm, const double *cmc, const double *sneqv,
                   cudaStream_t st) {
  const int ne = li.ne;
  std::vector<double> a(ne, 0.0), b(ne, 0.0);
  for (int i = 0; i < ne; i++) {
    const int r = perm[i];
    if (cmc) a[i] = cmc[r];
    if (sneqv) b[i] = sneqv[r];
  }
  return cuda_rc(cudaMemcpyAsync(li.L.cmc, a.data(), sizeof(double) * ne, cudaMemcpyHostToDevice, st)) ?:
         cuda_rc(cudaMemcpyAsync(li.L.sneqv, b.data(), sizeof(double) * ne, cudaMemcpyHostToDevice, st)) ?:
         cuda_rc(cudaStreamSynchronize(st));
}

int land_launch(LandInstance &li, int64_t t, double stepsize, const double *y_dev, cudaStream_t st,
                int64_t *launches) {
  if (!li.alloc || !y_dev || !(stepsize > 0.0)) return PIHM_GPU_ERR_ARG;
  if (t < li.t_lo || t > li.t_hi) return PIHM_GPU_ERR_ARG;
  // the month of PIHMTime (src/time_func.c:3-22), from gmtime like the reference
  const time_t raw = (time_t)t;
  std::tm tm{};
  if (!gmtime_r(&raw, &tm)) return PIHM_GPU_ERR_ARG;
  const int ne = li.ne;
  if (ne == 0) return PIHM_GPU_OK;
  const unsigned grid = (unsigned)((ne + kLandBlock - 1) / kLandBlock);
  if (tm.tm_mon != li.month) {
    k_land_month<<<grid, kLandBlock, 0, st>>>(li.L, ne, tm.tm_mon);
    (*launches)++;
    li.month = tm.tm_mon;
  }
  const int nser = li.L.nmeteo + li.L.nlai;
  k_land_station<<<(nser + 127) / 128, 128, 0, st>>>(li.L, t, tm.tm_mon);
  k_land_step<<<grid, kLandBlock, 0, st>>>(li.L, y_dev, ne, tm.tm_mon, stepsize);
  *launches += 2;
  return cuda_rc(cudaGetLastError());
}

void land_release(LandInstance &li) {
  if (li.alloc) cudaFree(li.alloc);
  li = LandInstance();
}

}  // namespace pihm

extern "C" {

int pihm_gpu_land_init(pihm_gpu_ctx *c, const pihm_land_params *p, const pihm_forcing_series *s) {
  if (!c || !p || p->nelem != c->ne) return PIHM_GPU_ERR_ARG;
  std::vector<double> zmax((size_t)c->ne);  // the surface elevation plane, read back from the device
  if (c->ne > 0 && cudaMemcpy(zmax.data(), c->m.zmax, sizeof(double) * c->ne, cudaMemcpyDeviceToHost) != cudaSuccess)
    return PIHM_GPU_ERR_CUDA;
  LandTargets tg{c->m.depth, c->m.porosity, c->m.rzd, c->m.d_rzd, const_cast<double *>(c->m.pcpdrp),
                 const_cast<double *>(c->m.edir), const_cast<double *>(c->m.ett)};
  LandInstance li;
  const int rc = land_build(p, s, c->h_perm, c->ne, zmax.data(), tg, &li);
  if (rc != PIHM_GPU_OK) return rc;
  land_release(c->land);
  c->land = li;
  c->m.land_prcp = li.L.prcp;
  c->m.land_ec = li.L.ec;
  c->m.land_cmc = li.L.cmc;
  c->m.land_sneqv = li.L.sneqv;
  return PIHM_GPU_OK;
}

int pihm_gpu_land_set_state(pihm_gpu_ctx *c, const double *cmc, const double *sneqv) {
  if (!c || !c->land.alloc) return PIHM_GPU_ERR_ARG;
  return land_set_state(c->land, c->h_perm, cmc, sneqv, c->stream);
}

int pihm_gpu_land_step(pihm_gpu_ctx *c, int64_t t, double stepsize, const double *y_dev) {
  if (!c || !c->land.alloc) return PIHM_GPU_ERR_ARG;
  int64_t n = 0;
  const int rc = land_launch(c->land, t, stepsize, y_dev, c->stream, &n);
  c->launches += n;
  return rc;
}

int pihm_gpu_land_get(pihm_gpu_ctx *c, int field, double *out) {
  if (!c || !c->land.alloc || !out || field < 0 || field >= PIHM_LAND_NFIELD) return PIHM_GPU_ERR_ARG;
  const LandDev &L = c->land.L;
  const double *src[PIHM_LAND_NFIELD] = {L.prcp, L.pcpdrp, L.edir, L.ett,
                                         L.ec,   L.drip,   L.cmc,  L.sneqv};
  const int ne = c->ne;
  std::vector<double> tmp(ne);
  const int rc = cuda_rc(cudaMemcpyAsync(tmp.data(), src[field], sizeof(double) * ne, cudaMemcpyDeviceToHost,
                                         c->stream)) ?:
                 cuda_rc(cudaStreamSynchronize(c->stream));
  if (rc != PIHM_GPU_OK) return rc;
  for (int i = 0; i < ne; i++) out[c->h_perm[i]] = tmp[i];
  return PIHM_GPU_OK;
}

}  // extern "C"
