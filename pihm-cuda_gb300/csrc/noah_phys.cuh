// Noah land-surface physics of Flux-PIHM for one element column, on the
// device.  A restatement of src/noah/noah.c and src/noah/lsm_func.c (the
// functions below name their reference and its lines): the same operations
// in the same order, so that, with the file compiled without multiply-add
// contraction, each element follows the reference's arithmetic; powers go
// through pow_any (within 0.502 ulp of the exact power, as glibc's), the
// other elementary functions are CUDA's.
//
// A column carries the element's parameters, forcing and state in a
// per-thread struct (the layer arrays in local memory); the kernels in
// noah.cu load it from the structure-of-arrays planes, run a step and store
// what persists.
#pragma once

#include <cmath>

#include "fp64_math.cuh"

namespace pihm {
namespace noah {

constexpr int L = 11;  // MAXLYR, src/include/pihm_const.h:84

// src/include/pihm_const.h
constexpr double kPi = 3.14159265;
constexpr double kGrav = 9.80665;
constexpr double kCp = 1004.0;
constexpr double kLvh2o = 2.501e6;
constexpr double kSigma = 5.67e-8;
constexpr double kRd = 287.04;
constexpr double kCph2o = 4.218e3;
constexpr double kCpice = 2.106e3;
constexpr double kLsubf = 3.335e5;
constexpr double kEmissiS = 0.95;
constexpr double kTfreez = 273.15;
constexpr double kLsubs = 2.83e6;
constexpr double kSh2oMin = 0.02;
constexpr double kBadVal = -999.0;

struct Col {
  // geometry and parameters
  int nsoil, nroot, isurban;
  double sldpth[L], zsoil[L], rtdis[L];
  double smcmax, smcmin, smcref, smcwlt, smcdry, quartz, csoil, alpha, beta, ksatv, porosity, depth, area;
  double shdfac, cmcfactr, laimax, laimin, emissmax, emissmin, albedomax, albedomin, z0max, z0min, snup,
      cfactr, rgl, rsmin, rsmax, topt, hs;
  double sbeta, salp, frzx, fxexp, czil, lvcoef, zbot, tbot, zlvl, zlvl_wind, snoalb;
  // forcing
  double prcp, sfctmp, rh, sfcspd, soldn, longwave, sfcprs, proj_lai;
  // state carried between steps
  double smc[L], sh2o[L], stc[L];
  double t1, cmc, sneqv, snowh, sndens, ch, cm, snotime1, albedo, emissi, q1, ribb, fcr;
  int nwtbl;
  double satdpth[L];
  // per-step quantities
  double cmcmax, embrd, alb, z0brd, sncond, sncovr, z0, th2, q2, q2sat, dqsdt2, ffrozp;
  double rr, rch, epsca, rc, pc, rcs, rct, rcq, rcsoil, beta_s, eta_kinematic, soilw, soilm;
  double solnet, lwdn, fdown, ssoil, flx1, flx2, flx3, sheat;
  double et[L], runoff2_lyr[L], smflxv[L];
  double edir, ec, ett, esnow, etp, eta, etns, dew, drip, pcpdrp, snomlt;
  double runoff2, runoff3, infil;
  // energy-unit fluxes of SFlx (W/m2)
  double ef_edir, ef_ec, ef_ett, ef_esnow, ef_etp, ef_eta;
};

// ---------------------------------------------------------------------------
// lsm_func.c
// ---------------------------------------------------------------------------

// FindWaterTable, src/noah/lsm_func.c:4-55
__device__ inline int find_water_table(const double *sldpth, int nsoil, double gw, double *satdpth) {
  int layer = -999;
  double dsum = 0.0, depth = 0.0;
  for (int j = 0; j < L; j++) satdpth[j] = 0.0;
  for (int j = 0; j < nsoil; j++) depth += sldpth[j];
  if (gw <= 0.0) {
    layer = nsoil;
    satdpth[nsoil - 1] = 1.0E-3;
  } else if (gw > depth) {
    layer = 0;
    for (int j = 0; j < nsoil; j++) satdpth[j] = sldpth[j];
  } else {
    for (int j = nsoil - 1; j >= 0; j--) {
      if (dsum + sldpth[j] > gw) {
        satdpth[j] = gw - dsum;
        layer = j + 1;
        break;
      }
      satdpth[j] = sldpth[j];
      dsum += sldpth[j];
    }
  }
  return layer;
}

// CalcLatFlx, src/noah/lsm_func.c:207-257 (the Flux-PIHM part)
__device__ inline void calc_lat_flx(Col &c) {
  double sattot = 0.0;
  for (int ks = 0; ks < c.nsoil; ks++) sattot += c.satdpth[ks];
  if (sattot <= 0.0) {
    c.runoff2_lyr[c.nsoil - 1] = c.runoff2;
  } else {
    for (int ks = 0; ks < c.nsoil; ks++) c.runoff2_lyr[ks] = c.satdpth[ks] / sattot * c.runoff2;
  }
}

// ---------------------------------------------------------------------------
// noah.c: helpers
// ---------------------------------------------------------------------------

// CalHum, :659-702
__device__ inline void cal_hum(Col &c) {
  const double A2 = 17.67, A3 = 273.15, A4 = 29.65, ELWV = 2.501e6, E0 = 611.0, RVV = 461.0,
               EPSILON = 0.622, SVP1 = 611.2, SVP2 = 17.67, SVP3 = 29.65, SVPT0 = 273.15;
  const double rh = c.rh / 100.0;
  const double svp = SVP1 * exp(SVP2 * (c.sfctmp - SVPT0) / (c.sfctmp - SVP3));
  const double e = rh * svp;
  c.q2 = (0.622 * e) / (c.sfcprs - (1.0 - 0.622) * e);
  c.th2 = c.sfctmp + (0.0098 * c.zlvl);
  const double a23m4 = A2 * (A3 - A4);
  const double esat = E0 * exp(ELWV / RVV * (1.0 / A3 - 1.0 / c.sfctmp));
  c.q2sat = EPSILON * esat / (c.sfcprs - (1.0 - EPSILON) * esat);
  c.dqsdt2 = c.q2sat * a23m4 / ((c.sfctmp - A4) * (c.sfctmp - A4));
}

// FrozRain, :961-976
__device__ inline double froz_rain(double prcp, double sfctmp) {
  return (prcp > 0.0 && sfctmp < kTfreez) ? 1.0 : 0.0;
}

// CSnow, :811-839
__device__ inline double csnow(double dsnow) {
  const double UNIT = 0.11631;
  const double cc = 0.328 * pow_any(10.0, 2.25 * dsnow);
  return 2.0 * UNIT * cc;
}

// SnFrac, :1713-1744
__device__ inline double snfrac(double sneqv, double snup, double salp) {
  if (sneqv < snup) {
    const double rsnow = sneqv / snup;
    return 1.0 - (exp(-salp * rsnow) - rsnow * exp(-salp));
  }
  return 1.0;
}

// Snowz0, :2202-2220
__device__ inline double snowz0(double sncovr, double z0brd, double snowh) {
  const double Z0S = 0.001;
  const double burial = 7.0 * z0brd - snowh;
  const double z0eff = (burial <= 0.0007) ? Z0S : (burial / 7.0);
  return (1.0 - sncovr) * z0brd + sncovr * z0eff;
}

// SnowNew, :2222-2268
__device__ inline void snow_new(Col &c, double newsn) {
  double snowhc = c.snowh * 100.0;
  const double newsnc = newsn * 100.0;
  const double tempc = c.sfctmp - 273.15;
  double dsnew;
  if (tempc <= -15.0) dsnew = 0.05;
  else dsnew = 0.05 + 0.0017 * pow_any(tempc + 15.0, 1.5);
  const double hnewc = newsnc / dsnew;
  if (snowhc + hnewc < 0.001) c.sndens = (dsnew > c.sndens) ? dsnew : c.sndens;
  else c.sndens = (snowhc * c.sndens + hnewc * dsnew) / (snowhc + hnewc);
  snowhc = snowhc + hnewc;
  c.snowh = snowhc * 0.01;
}

// AlCalc, :610-657
__device__ inline void al_calc(Col &c, double dt, int snowng) {
  const double SNACCA = 0.94, SNACCB = 0.58;
  c.albedo = c.alb + c.sncovr * (c.snoalb - c.alb);
  c.emissi = c.embrd + c.sncovr * (kEmissiS - c.embrd);
  const double snoalb1 = c.snoalb + c.lvcoef * (0.85 - c.snoalb);
  double snoalb2 = snoalb1;
  if (snowng) {
    c.snotime1 = 0.0;
  } else {
    c.snotime1 += dt;
    snoalb2 = snoalb1 * pow_any(SNACCA, pow_any(c.snotime1 / 86400.0, SNACCB));
  }
  snoalb2 = (snoalb2 > c.alb) ? snoalb2 : c.alb;
  c.albedo = c.alb + c.sncovr * (snoalb2 - c.alb);
  c.albedo = (c.albedo > snoalb2) ? snoalb2 : c.albedo;
}

// TDfCnd, :2520-2619
__device__ inline double tdf_cnd(double smc, double qz, double smcmax, double smcmin, double sh2o) {
  const double THKICE = 2.2, THKQTZ = 7.7, THKW = 0.57;
  const double satratio = (smc - smcmin) / (smcmax - smcmin);
  const double thko = 2.0;
  const double thks = pow_any(THKQTZ, qz) * pow_any(thko, 1.0 - qz);
  const double xunfroz = sh2o / smc;
  const double xu = xunfroz * smcmax;
  const double thksat = pow_any(thks, 1.0 - smcmax) * pow_any(THKICE, smcmax - xu) * pow_any(THKW, xu);
  const double gammd = (1.0 - smcmax) * 2700.0;
  const double thkdry = (0.135 * gammd + 64.7) / (2700.0 - 0.947 * gammd);
  double ake;
  if ((sh2o + 0.0005) < smc) ake = satratio;
  else ake = (satratio > 0.1) ? log10(satratio) + 1.0 : 0.0;
  return ake * (thksat - thkdry) + thkdry;
}

// The surface-layer stability functions, :3173-3223
__device__ inline double pslmu(double zz) { return -0.96 * log(1.0 - 4.5 * zz); }
__device__ inline double pslms(double zz) {
  const double RIC = 0.183;
  const double rric = 1.0 / RIC;
  return zz * rric - 2.076 * (1.0 - 1.0 / (zz + 1.0));
}
__device__ inline double pslhu(double zz) { return -0.96 * log(1.0 - 4.5 * zz); }
__device__ inline double pslhs(double zz) {
  const double RIC = 0.183, FHNEU = 0.8, RFC = 0.191;
  const double rfac = RIC / (FHNEU * RFC * RFC);
  return zz * rfac - 2.076 * (1.0 - exp(-1.2 * zz));
}
__device__ inline double pspmu(double xx) {
  return -2.0 * log((xx + 1.0) * 0.5) - log((xx * xx + 1.0) * 0.5) + 2.0 * atan(xx) - kPi * 0.5;
}
__device__ inline double pspms(double yy) { return 5.0 * yy; }
__device__ inline double psphu(double xx) { return -2.0 * log((xx * xx + 1.0) * 0.5); }
__device__ inline double psphs(double yy) { return 5.0 * yy; }

// SfcDifOff, :2862-3079 (iz0tlnd = 0 as SFlx calls it)
__device__ inline void sfcdif_off(Col &c, double t1v, double th2v) {
  const double WWST = 1.2, VKRM = 0.40, EXCM = 0.001, BETA = 1.0 / 270.0, WOLD = 0.15, EPSU2 = 1.0e-4,
               EPSUST = 0.07, ZTMIN = -5.0, ZTMAX = 1.0, HPBL = 1000.0, SQVISC = 258.2;
  const int ITRMX = 5;
  const double wwst2 = WWST * WWST;
  const double btg = BETA * kGrav;
  const double elfc = VKRM * btg;
  const double wnew = 1.0 - WOLD;
  const int ilech = 0;
  const double zilfc = -c.czil * VKRM * SQVISC;
  const double zu = c.z0;
  const double rdz = 1.0 / c.zlvl_wind;
  const double cxch = EXCM * rdz;
  const double dthv = th2v - t1v;
  double du2 = c.sfcspd * c.sfcspd;
  du2 = (du2 > EPSU2) ? du2 : EPSU2;
  const double btgh = btg * HPBL;
  double wstar2;
  if (btgh * c.ch * dthv != 0.0) wstar2 = wwst2 * pow_any(fabs(btgh * c.ch * dthv), 2.0 / 3.0);
  else wstar2 = 0.0;
  double ustar = sqrt(c.cm * sqrt(du2 + wstar2));
  ustar = (ustar > EPSUST) ? ustar : EPSUST;
  double zt = exp(zilfc * sqrt(ustar * c.z0)) * c.z0;
  const double zslu = c.zlvl_wind + zu;
  double zslt = c.zlvl + zt;
  const double rlogu = log(zslu / zu);
  double rlogt = log(zslt / zt);
  double rlmo = elfc * c.ch * dthv / pow_any(ustar, 3);
  for (int itr = 0; itr < ITRMX; itr++) {
    double zetalt = zslt * rlmo;
    zetalt = zetalt > ZTMIN ? zetalt : ZTMIN;
    rlmo = zetalt / zslt;
    double zetalu = zslu * rlmo;
    const double zetau = zu * rlmo;
    const double zetat = zt * rlmo;
    double psmz, simm, pshz, simh;
    if (ilech == 0) {
      if (rlmo < 0.0) {
        const double xlu4 = 1.0 - 16.0 * zetalu;
        const double xlt4 = 1.0 - 16.0 * zetalt;
        const double xu4 = 1.0 - 16.0 * zetau;
        const double xt4 = 1.0 - 16.0 * zetat;
        const double xlu = sqrt(sqrt(xlu4));
        const double xlt = sqrt(sqrt(xlt4));
        const double xu = sqrt(sqrt(xu4));
        const double xt = sqrt(sqrt(xt4));
        psmz = pspmu(xu);
        simm = pspmu(xlu) - psmz + rlogu;
        pshz = psphu(xt);
        simh = psphu(xlt) - pshz + rlogt;
      } else {
        zetalu = (zetalu < ZTMAX) ? zetalu : ZTMAX;
        zetalt = (zetalt < ZTMAX) ? zetalt : ZTMAX;
        psmz = pspms(zetau);
        simm = pspms(zetalu) - psmz + rlogu;
        pshz = psphs(zetat);
        simh = psphs(zetalt) - pshz + rlogt;
      }
    } else {
      if (rlmo < 0.0) {
        psmz = pslmu(zetau);
        simm = pslmu(zetalu) - psmz + rlogu;
        pshz = pslhu(zetat);
        simh = pslhu(zetalt) - pshz + rlogt;
      } else {
        zetalu = zetalu < ZTMAX ? zetalu : ZTMAX;
        zetalt = zetalt < ZTMAX ? zetalt : ZTMAX;
        psmz = pslms(zetau);
        simm = pslms(zetalu) - psmz + rlogu;
        pshz = pslhs(zetat);
        simh = pslhs(zetalt) - pshz + rlogt;
      }
    }
    ustar = sqrt(c.cm * sqrt(du2 + wstar2));
    ustar = (ustar > EPSUST) ? ustar : EPSUST;
    zt = exp(zilfc * sqrt(ustar * c.z0)) * c.z0;
    zslt = c.zlvl + zt;
    rlogt = log(zslt / zt);
    const double ustark = ustar * VKRM;
    c.cm = (ustark / simm > cxch) ? ustark / simm : cxch;
    c.ch = (ustark / simh > cxch) ? ustark / simh : cxch;
    if (btgh * c.ch * dthv != 0.0) wstar2 = wwst2 * pow_any(fabs(btgh * c.ch * dthv), 2.0 / 3.0);
    else wstar2 = 0.0;
    const double rlmn = elfc * c.ch * dthv / pow_any(ustar, 3.0);
    const double rlma = rlmo * WOLD + rlmn * wnew;
    rlmo = rlma;
  }
}

// Penman, :1508-1570
__device__ inline void penman(Col &c, double *t24, double t2v, int snowng, int frzgra) {
  const double ELCP = 2.4888e+3, LSUBC = 2.501000e+6;
  const double emissi = c.emissi;
  const double elcp1 = (1.0 - c.sncovr) * ELCP + c.sncovr * ELCP * kLsubs / LSUBC;
  const double lvs = (1.0 - c.sncovr) * LSUBC + c.sncovr * kLsubs;
  c.flx2 = 0.0;
  const double delta = elcp1 * c.dqsdt2;
  *t24 = c.sfctmp * c.sfctmp * c.sfctmp * c.sfctmp;
  c.rr = emissi * *t24 * 6.48e-8 / (c.sfcprs * c.ch) + 1.0;
  const double rho = c.sfcprs / (kRd * t2v);
  c.rch = rho * kCp * c.ch;
  if (!snowng) {
    if (c.prcp > 0.0) c.rr += kCph2o * c.prcp * 1000.0 / c.rch;
  } else {
    c.rr += kCpice * c.prcp * 1000.0 / c.rch;
  }
  double fnet = c.fdown - emissi * kSigma * *t24 - c.ssoil;
  if (frzgra) {
    c.flx2 = -kLsubf * c.prcp * 1000.0;
    fnet -= c.flx2;
  }
  const double rad = fnet / c.rch + c.th2 - c.sfctmp;
  const double a = elcp1 * (c.q2sat - c.q2);
  c.epsca = (a * c.rr + rad * delta) / (delta + c.rr);
  c.etp = c.epsca * c.rch / lvs / 1000.0;
}

// CanRes, :704-809 (Flux-PIHM, not Cycles)
__device__ inline void can_res(Col &c) {
  const double SLV = 2.501000e6;
  double part[L];
  c.rcs = 0.0;
  c.rct = 0.0;
  c.rcq = 0.0;
  c.rcsoil = 0.0;
  c.rc = 0.0;
  const double ff = 0.55 * 2.0 * c.soldn / (c.rgl * c.proj_lai);
  c.rcs = (ff + c.rsmin / c.rsmax) / (1.0 + ff);
  c.rcs = (c.rcs > 0.0001) ? c.rcs : 0.0001;
  c.rct = 1.0 - 0.0016 * pow_any(c.topt - c.sfctmp, 2.0);
  c.rct = (c.rct > 0.0001) ? c.rct : 0.0001;
  c.rcq = 1.0 / (1.0 + c.hs * (c.q2sat - c.q2));
  c.rcq = (c.rcq > 0.01) ? c.rcq : 0.01;
  double gx = (c.sh2o[0] - c.smcwlt) / (c.smcref - c.smcwlt);
  gx = (gx > 1.0) ? 1.0 : gx;
  gx = (gx < 0.0) ? 0.0 : gx;
  part[0] = (c.zsoil[0] / c.zsoil[c.nroot - 1]) * gx;
  for (int k = 1; k < c.nroot; k++) {
    gx = (c.sh2o[k] - c.smcwlt) / (c.smcref - c.smcwlt);
    gx = (gx > 1.0) ? 1.0 : gx;
    gx = (gx < 0.0) ? 0.0 : gx;
    part[k] = ((c.zsoil[k] - c.zsoil[k - 1]) / c.zsoil[c.nroot - 1]) * gx;
  }
  for (int k = 0; k < c.nroot; k++) c.rcsoil += part[k];
  c.rcsoil = (c.rcsoil > 0.0001) ? c.rcsoil : 0.0001;
  c.rc = c.rsmin / (c.proj_lai * c.rcs * c.rct * c.rcq * c.rcsoil);
  const double rr = (4.0 * c.emissi * kSigma * kRd / kCp) * pow_any(c.sfctmp, 4.0) / (c.sfcprs * c.ch) + 1.0;
  const double delta = (SLV / kCp) * c.dqsdt2;
  c.pc = (rr + delta) / (rr * (1.0 + c.rc * c.ch) + delta);
}

// DEvap, :841-870
__device__ inline void devap(Col &c) {
  double fx;
  const double sratio = (c.sh2o[0] - c.smcdry) / (c.smcmax - c.smcdry);
  if (sratio > 0.0) {
    fx = pow_any(sratio, c.fxexp);
    fx = (fx > 1.0) ? 1.0 : fx;
    fx = (fx < 0.0) ? 0.0 : fx;
  } else {
    fx = 0.0;
  }
  c.edir = fx * (1.0 - c.shdfac) * c.etp;
}

// Transp, :2725-2811
__device__ inline void transp(Col &c) {
  double gx[L];
  for (int k = 0; k < c.nsoil; k++) c.et[k] = 0.0;
  double etpa;
  if (c.cmc != 0.0) etpa = c.shdfac * c.pc * c.etp * (1.0 - pow_any(c.cmc / c.cmcmax, c.cfactr));
  else etpa = c.shdfac * c.pc * c.etp;
  double sgx = 0.0;
  for (int i = 0; i < c.nroot; i++) {
    gx[i] = (c.smc[i] - c.smcwlt) / (c.smcref - c.smcwlt);
    gx[i] = (gx[i] < 0.0) ? 0.0 : gx[i];
    gx[i] = (gx[i] > 1.0) ? 1.0 : gx[i];
    sgx += gx[i];
  }
  sgx /= (double)c.nroot;
  double denom = 0.0;
  for (int i = 0; i < c.nroot; i++) {
    const double rtx = c.rtdis[i] + gx[i] - sgx;
    gx[i] *= ((rtx > 0.0) ? rtx : 0.0);
    denom += gx[i];
  }
  denom = (denom <= 0.0) ? 1.0 : denom;
  for (int i = 0; i < c.nroot; i++) c.et[i] = etpa * gx[i] / denom;
}

// Evapo, :872-959 (Flux-PIHM)
__device__ inline void evapo(Col &c, double dt) {
  c.edir = 0.0;
  c.ec = 0.0;
  c.ett = 0.0;
  for (int k = 0; k < c.nsoil; k++) c.et[k] = 0.0;
  if (c.etp > 0.0) {
    if (c.shdfac < 1.0) devap(c);
    if (c.shdfac > 0.0) {
      transp(c);
      for (int k = 0; k < c.nsoil; k++) c.ett += c.et[k];
      if (c.cmc > 0.0)
        c.ec = c.shdfac * pow_any((c.cmc / c.cmcmax > 1.0) ? 1.0 : c.cmc / c.cmcmax, c.cfactr) * c.etp;
      else
        c.ec = 0.0;
      const double cmc2ms = c.cmc / dt;
      c.ec = (cmc2ms < c.ec) ? cmc2ms : c.ec;
    }
  }
  c.etns = c.edir + c.ett + c.ec;
}

// PcpDrp, :1451-1506
__device__ inline void pcp_drp(Col &c, double prcp, double dt) {
  const double KD = 6.54e-7, BFACTR = 3.89;
  double rhsct = c.shdfac * prcp - c.ec;
  c.drip = 0.0;
  const double trhsct = dt * rhsct;
  const double excess = c.cmc + trhsct;
  if (excess > 0.0) {
    if (excess >= c.cmcmax) c.drip = (KD * c.cmcmax * exp(BFACTR)) + (excess - c.cmcmax) / dt;
    else c.drip = (KD * c.cmcmax * exp(BFACTR * excess / c.cmcmax));
    c.drip = (c.drip > excess / dt) ? excess / dt : c.drip;
  }
  rhsct -= c.drip;
  c.pcpdrp = (1.0 - c.shdfac) * prcp + c.drip;
  c.cmc += dt * rhsct;
  if (c.cmc < 1.0e-20) c.cmc = 0.0;
  c.cmc = (c.cmc < c.cmcmax) ? c.cmc : c.cmcmax;
}

// Rosr12, :1572-1619: tridiagonal solve, p receives the solution
__device__ inline void rosr12(double *p, const double *a, const double *b, double *cc, const double *d,
                              double *delta, int nsoil) {
  cc[nsoil - 1] = 0.0;
  p[0] = -cc[0] / b[0];
  delta[0] = d[0] / b[0];
  for (int k = 1; k < nsoil; k++) {
    p[k] = -cc[k] * (1.0 / (b[k] + a[k] * p[k - 1]));
    delta[k] = (d[k] - a[k] * delta[k - 1]) * (1.0 / (b[k] + a[k] * p[k - 1]));
  }
  p[nsoil - 1] = delta[nsoil - 1];
  for (int k = 1; k < nsoil; k++) {
    const int kk = nsoil - k - 1;
    p[kk] = p[kk] * p[kk + 1] + delta[kk];
  }
}

// FrH2O, :978-1090: supercooled liquid water (Newton iteration, at most 10
// steps, as the reference)
__device__ inline double frh2o(const Col &c, double tkelv, double smc, double sh2o) {
  const double CK = 8.0, ERROR = 0.005;
  int nlog = 0, kcount = 0;
  double freew, mx = 0.0;
  if (tkelv > (kTfreez - 1.0e-3)) {
    freew = smc;
  } else {
    double swl = smc - sh2o;
    swl = (swl > smc - kSh2oMin) ? (smc - kSh2oMin) : swl;
    swl = (swl < 0.0) ? 0.0 : swl;
    while (nlog < 10 && kcount == 0) {
      nlog++;
      const double satn = (smc - swl - c.smcmin) / (c.smcmax - c.smcmin);
      mx = c.beta / (1.0 - c.beta);
      const double df = log(kGrav / c.alpha / kLsubf) + 1.0 / c.beta * log(pow_any(satn, mx) - 1.0) +
                        2.0 * log(1.0 + CK * swl) - log(-(tkelv - kTfreez) / tkelv);
      const double denom = 1.0 / (c.beta - 1.0) / (c.smcmax - c.smcmin) * pow_any(satn, mx - 1.0) /
                               (pow_any(satn, mx) - 1.0) +
                           2.0 * CK / (1.0 + CK * swl);
      double swlk = swl - df / denom;
      swlk = (swlk > smc - kSh2oMin) ? (smc - kSh2oMin) : swlk;
      swlk = (swlk < 0.0) ? 0.0 : swlk;
      const double dswl = fabs(swlk - swl);
      swl = swlk;
      if (dswl <= ERROR) kcount++;
    }
    freew = smc - swl;
    if (kcount == 0) {
      double fk = pow_any(pow_any(-(tkelv - kTfreez) / tkelv * c.alpha * kLsubf / kGrav, c.beta), 1.0 / mx) *
                      (c.smcmax - c.smcmin) -
                  c.smcmin;
      fk = (fk < kSh2oMin) ? kSh2oMin : fk;
      freew = (fk < smc) ? fk : smc;
    }
  }
  return freew;
}

// SnkSrc, :1746-1811
__device__ inline double snk_src(const Col &c, double tavg, double smc, double *sh2o, double dt, int k,
                                 double qtot) {
  const double DH2O = 1.0000e3;
  const double dz = (0 == k) ? -c.zsoil[0] : c.zsoil[k - 1] - c.zsoil[k];
  const double freew = frh2o(c, tavg, smc, *sh2o);
  double xh2o = *sh2o + qtot * dt / (DH2O * kLsubf * dz);
  if (xh2o < *sh2o && xh2o < freew) xh2o = (freew > *sh2o) ? *sh2o : freew;
  if (xh2o > *sh2o && xh2o > freew) xh2o = (freew < *sh2o) ? *sh2o : freew;
  xh2o = (xh2o < 0.0) ? 0.0 : xh2o;
  xh2o = (xh2o > smc) ? smc : xh2o;
  const double tsnsr = -DH2O * kLsubf * dz * (xh2o - *sh2o) / dt;
  *sh2o = xh2o;
  return tsnsr;
}

// TBnd, :2482-2518
__device__ inline double tbnd(double tu, double tb, const double *zsoil, double zbot, int k, int nsoil) {
  const double zup = (k == 0) ? 0.0 : zsoil[k - 1];
  const double zb = (k == nsoil - 1) ? 2.0 * zbot - zsoil[k] : zsoil[k + 1];
  return tu + (tb - tu) * (zup - zsoil[k]) / (zup - zb);
}

// TmpAvg, :2621-2723
__device__ inline double tmp_avg(double tup, double tm, double tdn, const double *zsoil, int k) {
  const double dz = (k == 0) ? -zsoil[0] : zsoil[k - 1] - zsoil[k];
  const double dzh = dz * 0.5;
  double x0, xdn, xup, tavg;
  if (tup < kTfreez) {
    if (tm < kTfreez) {
      if (tdn < kTfreez) {
        tavg = (tup + 2.0 * tm + tdn) / 4.0;
      } else {
        x0 = (kTfreez - tm) * dzh / (tdn - tm);
        tavg = 0.5 * (tup * dzh + tm * (dzh + x0) + kTfreez * (2.0 * dzh - x0)) / dz;
      }
    } else {
      if (tdn < kTfreez) {
        xup = (kTfreez - tup) * dzh / (tm - tup);
        xdn = dzh - (kTfreez - tm) * dzh / (tdn - tm);
        tavg = 0.5 * (tup * xup + kTfreez * (2.0 * dz - xup - xdn) + tdn * xdn) / dz;
      } else {
        xup = (kTfreez - tup) * dzh / (tm - tup);
        tavg = 0.5 * (tup * xup + kTfreez * (2.0 * dz - xup)) / dz;
      }
    }
  } else {
    if (tm < kTfreez) {
      if (tdn < kTfreez) {
        xup = dzh - (kTfreez - tup) * dzh / (tm - tup);
        tavg = 0.5 * (kTfreez * (dz - xup) + tm * (dzh + xup) + tdn * dzh) / dz;
      } else {
        xup = dzh - (kTfreez - tup) * dzh / (tm - tup);
        xdn = (kTfreez - tm) * dzh / (tdn - tm);
        tavg = 0.5 * (kTfreez * (2.0 * dz - xup - xdn) + tm * (xup + xdn)) / dz;
      }
    } else {
      if (tdn < kTfreez) {
        xdn = dzh - (kTfreez - tm) * dzh / (tdn - tm);
        tavg = (kTfreez * (dz - xdn) + 0.5 * (kTfreez + tdn) * xdn) / dz;
      } else {
        tavg = (tup + 2.0 * tm + tdn) / 4.0;
      }
    }
  }
  return tavg;
}

// HRT, :1092-1299 (temperature averaging on, as the reference sets it)
__device__ inline void hrt(Col &c, double *rhsts, double yy, double zz1, double dt, double df1, double *ai,
                           double *bi, double *ci) {
  const double CH2O = 4.2e6;
  const double csoil_loc = (c.isurban) ? 3.0e6 : c.csoil;
  double hcpct = c.sh2o[0] * CH2O + (1.0 - c.smcmax) * csoil_loc + (c.smcmax - c.smc[0]) * kCp +
                 (c.smc[0] - c.sh2o[0]) * kCpice;
  double ddz = 1.0 / (-0.5 * c.zsoil[1]);
  ai[0] = 0.0;
  ci[0] = (df1 * ddz) / (c.zsoil[0] * hcpct);
  bi[0] = -ci[0] + df1 / (0.5 * c.zsoil[0] * c.zsoil[0] * hcpct * zz1);
  double dtsdz = (c.stc[0] - c.stc[1]) / (-0.5 * c.zsoil[1]);
  c.ssoil = df1 * (c.stc[0] - yy) / (0.5 * c.zsoil[0] * zz1);
  double denom = c.zsoil[0] * hcpct;
  rhsts[0] = (df1 * dtsdz - c.ssoil) / denom;
  double qtot = -1.0 * rhsts[0] * denom;
  double sice = c.smc[0] - c.sh2o[0];
  const double tsurf = (yy + (zz1 - 1.0) * c.stc[0]) / zz1;
  double tbk = tbnd(c.stc[0], c.stc[1], c.zsoil, c.zbot, 0, c.nsoil);
  if ((sice > 0.0) || (c.stc[0] < kTfreez) || (tsurf < kTfreez) || (tbk < kTfreez)) {
    const double tavg = tmp_avg(tsurf, c.stc[0], tbk, c.zsoil, 0);
    const double tsnsr = snk_src(c, tavg, c.smc[0], &c.sh2o[0], dt, 0, qtot);
    rhsts[0] -= tsnsr / denom;
  }
  double ddz2 = 0.0;
  double df1k = df1, df1n, dtsdz2, tbk1 = 0.0;
  for (int k = 1; k < c.nsoil; k++) {
    hcpct = c.sh2o[k] * CH2O + (1.0 - c.smcmax) * csoil_loc + (c.smcmax - c.smc[k]) * kCp +
            (c.smc[k] - c.sh2o[k]) * kCpice;
    if (k != c.nsoil - 1) {
      df1n = tdf_cnd(c.smc[k], c.quartz, c.smcmax, c.smcmin, c.sh2o[k]);
      df1n = (c.isurban) ? 3.24 : df1n;
      denom = 0.5 * (c.zsoil[k - 1] - c.zsoil[k + 1]);
      dtsdz2 = (c.stc[k] - c.stc[k + 1]) / denom;
      ddz2 = 2.0 / (c.zsoil[k - 1] - c.zsoil[k + 1]);
      ci[k] = -df1n * ddz2 / ((c.zsoil[k - 1] - c.zsoil[k]) * hcpct);
      tbk1 = tbnd(c.stc[k], c.stc[k + 1], c.zsoil, c.zbot, k, c.nsoil);
    } else {
      df1n = tdf_cnd(c.smc[k], c.quartz, c.smcmax, c.smcmin, c.sh2o[k]);
      df1n = (c.isurban) ? 3.24 : df1n;
      denom = 0.5 * (c.zsoil[k - 1] + c.zsoil[k]) - c.zbot;
      dtsdz2 = (c.stc[k] - c.tbot) / denom;
      ci[k] = 0.0;
      tbk1 = tbnd(c.stc[k], c.tbot, c.zsoil, c.zbot, k, c.nsoil);
    }
    denom = (c.zsoil[k] - c.zsoil[k - 1]) * hcpct;
    rhsts[k] = (df1n * dtsdz2 - df1k * dtsdz) / denom;
    qtot = -1.0 * denom * rhsts[k];
    sice = c.smc[k] - c.sh2o[k];
    const double tavg = tmp_avg(tbk, c.stc[k], tbk1, c.zsoil, k);
    if ((sice > 0.0) || (c.stc[k] < kTfreez) || (tbk < kTfreez) || (tbk1 < kTfreez)) {
      const double tsnsr = snk_src(c, tavg, c.smc[k], &c.sh2o[k], dt, k, qtot);
      rhsts[k] = rhsts[k] - tsnsr / denom;
    }
    ai[k] = -df1k * ddz / ((c.zsoil[k - 1] - c.zsoil[k]) * hcpct);
    bi[k] = -(ai[k] + ci[k]);
    tbk = tbk1;
    df1k = df1n;
    dtsdz = dtsdz2;
    ddz = ddz2;
  }
}

// HStep, :1301-1341
__device__ inline void hstep(Col &c, double *rhsts, double dt, double *ai, double *bi, double *ci) {
  double rhstsin[L], ciin[L];
  const int n = c.nsoil;
  for (int k = 0; k < n; k++) {
    rhsts[k] *= dt;
    ai[k] *= dt;
    bi[k] = 1.0 + bi[k] * dt;
    ci[k] *= dt;
  }
  for (int k = 0; k < n; k++) rhstsin[k] = rhsts[k];
  for (int k = 0; k < n; k++) ciin[k] = ci[k];
  rosr12(ci, ai, bi, ciin, rhstsin, rhsts, n);
  for (int k = 0; k < n; k++) c.stc[k] += ci[k];
}

// ShFlx, :1621-1652
__device__ inline void shflx(Col &c, double dt, double yy, double zz1, double df1) {
  double ai[L], bi[L], ci[L], rhsts[L];
  hrt(c, rhsts, yy, zz1, dt, df1, ai, bi, ci);
  hstep(c, rhsts, dt, ai, bi, ci);
  c.t1 = (yy + (zz1 - 1.0) * c.stc[0]) / zz1;
  c.ssoil = df1 * (c.stc[0] - c.t1) / (0.5 * c.zsoil[0]);
}

// NoPac, :1343-1449
__device__ inline void nopac(Col &c, double dt, double t24) {
  double prcpf = c.prcp;
  c.dew = 0.0;
  c.edir = 0.0;
  c.ec = 0.0;
  for (int k = 0; k < c.nsoil; k++) c.et[k] = 0.0;
  c.ett = 0.0;
  if (c.etp > 0.0) {
    evapo(c, dt);
    c.eta = c.etns;
  } else {
    c.dew = -c.etp;
    prcpf += c.dew;
  }
  pcp_drp(c, prcpf, dt);
  if (c.etp <= 0.0) {
    c.beta_s = 0.0;
    c.eta = c.etp;
    if (c.etp < 0.0) c.beta_s = 1.0;
  } else {
    c.beta_s = c.eta / c.etp;
  }
  double df1 = tdf_cnd(c.smc[0], c.quartz, c.smcmax, c.smcmin, c.sh2o[0]);
  df1 = (c.isurban) ? 3.24 : df1;
  df1 *= exp(c.sbeta * c.shdfac);
  const double yynum = c.fdown - c.emissi * kSigma * t24;
  const double yy = c.sfctmp + (yynum / c.rch + c.th2 - c.sfctmp - c.beta_s * c.epsca) / c.rr;
  const double zz1 = df1 / (-0.5 * c.zsoil[0] * c.rch * c.rr) + 1.0;
  shflx(c, dt, yy, zz1, df1);
  c.flx1 = kCph2o * c.prcp * 1000.0 * (c.t1 - c.sfctmp);
  c.flx3 = 0.0;
}

// SnowPack, :2100-2200
__device__ inline void snow_pack(double esd, double dtsec, double *snowh, double *sndens, double tsnow,
                                 double tsoil) {
  const double C1 = 0.01, C2 = 21.0;
  const double esdc = esd * 100.0;
  const double dthr = dtsec / 3600.0;
  const double tsnowc = tsnow - 273.15;
  const double tsoilc = tsoil - 273.15;
  const double tavgc = 0.5 * (tsnowc + tsoilc);
  const double esdcx = (esdc > 1.0e-2) ? esdc : 1.0e-2;
  const double bfac = dthr * C1 * exp(0.08 * tavgc - C2 * *sndens);
  const int ipol = 4;
  double pexp = 0.0;
  for (int j = ipol; j > 0; j--) pexp = (1.0 + pexp) * bfac * esdcx / (double)(j + 1);
  pexp += 1.0;
  double dsx = *sndens * pexp;
  dsx = (dsx > 0.40) ? 0.40 : dsx;
  dsx = (dsx < 0.05) ? 0.05 : dsx;
  *sndens = dsx;
  if (tsnowc >= 0.0) {
    const double dw = 0.13 * dthr / 24.0;
    *sndens = *sndens * (1.0 - dw) + dw;
    if (*sndens >= 0.40) *sndens = 0.40;
  }
  const double snowhc = esdc / *sndens;
  *snowh = snowhc * 0.01;
}

// SnoPac, :1813-2098
__device__ inline void snopac(Col &c, int snowng, double dt, double t24, double prcpf, double df1) {
  const double ESDMIN = 1.0e-6, SNOEXP = 2.0;
  c.dew = 0.0;
  c.edir = 0.0;
  c.ec = 0.0;
  for (int k = 0; k < c.nsoil; k++) c.et[k] = 0.0;
  c.ett = 0.0;
  c.esnow = 0.0;
  double esnow2 = 0.0, etanrg, ex;
  c.beta_s = 1.0;
  if (c.etp <= 0.0) {
    if ((c.ribb >= 0.1) && (c.fdown > 150.0)) {
      c.etp = (((c.etp * (1.0 - c.ribb) < 0.0) ? c.etp * (1.0 - c.ribb) : 0.0) * c.sncovr / 0.980 +
               c.etp * (0.980 - c.sncovr)) /
              0.980;
    }
    if (c.etp == 0.0) c.beta_s = 0.0;
    c.dew = -c.etp;
    esnow2 = c.etp * dt;
    etanrg = c.etp * 1000.0 * ((1.0 - c.sncovr) * kLvh2o + c.sncovr * kLsubs);
  } else {
    if (c.sncovr < 1.0) {
      evapo(c, dt);
      c.edir *= (1.0 - c.sncovr);
      c.ec *= (1.0 - c.sncovr);
      for (int k = 0; k < c.nsoil; k++) c.et[k] = c.et[k] * (1.0 - c.sncovr);
      c.ett *= (1.0 - c.sncovr);
      c.etns *= (1.0 - c.sncovr);
    }
    c.esnow = c.etp * c.sncovr;
    esnow2 = c.esnow * dt;
    etanrg = c.esnow * 1000.0 * kLsubs + c.etns * 1000.0 * kLvh2o;
  }
  c.flx1 = 0.0;
  if (snowng) {
    c.flx1 = kCpice * c.prcp * 1000.0 * (c.t1 - c.sfctmp);
  } else {
    if (c.prcp > 0.0) c.flx1 = kCph2o * c.prcp * 1000.0 * (c.t1 - c.sfctmp);
  }
  const double dsoil = -0.5 * c.zsoil[0];
  const double dtot = c.snowh + dsoil;
  const double denom = 1.0 + df1 / (dtot * c.rr * c.rch);
  const double t12a =
      ((c.fdown - c.flx1 - c.flx2 - c.emissi * kSigma * t24) / c.rch + c.th2 - c.sfctmp - etanrg / c.rch) / c.rr;
  const double t12b = df1 * c.stc[0] / (dtot * c.rr * c.rch);
  const double t12 = (c.sfctmp + t12a + t12b) / denom;
  if (t12 <= kTfreez) {
    c.t1 = t12;
    c.ssoil = df1 * (c.t1 - c.stc[0]) / dtot;
    if (c.sneqv - esnow2 > 0.0) {
      c.sneqv -= esnow2;
    } else {
      c.sneqv = 0.0;
      esnow2 = c.sneqv;
      c.esnow = esnow2 / dt;
    }
    c.flx3 = 0.0;
    ex = 0.0;
    c.snomlt = 0.0;
  } else {
    c.t1 = kTfreez * pow_any(c.sncovr, SNOEXP) + t12 * (1.0 - pow_any(c.sncovr, SNOEXP));
    c.beta_s = 1.0;
    c.ssoil = df1 * (c.t1 - c.stc[0]) / dtot;
    if (c.sneqv - esnow2 <= ESDMIN) {
      c.sneqv = 0.0;
      ex = 0.0;
      c.snomlt = 0.0;
      c.flx3 = 0.0;
    } else {
      c.sneqv -= esnow2;
      const double seh = c.rch * (c.t1 - c.th2);
      double t14 = c.t1 * c.t1;
      t14 = t14 * t14;
      c.flx3 = c.fdown - c.flx1 - c.flx2 - c.emissi * kSigma * t14 - c.ssoil - seh - etanrg;
      c.flx3 = (c.flx3 <= 0.0) ? 0.0 : c.flx3;
      ex = c.flx3 * 0.001 / kLsubf;
      c.snomlt = ex;
      if (c.sneqv - c.snomlt * dt >= ESDMIN) {
        c.sneqv -= c.snomlt * dt;
      } else {
        ex = c.sneqv / dt;
        c.flx3 = ex * 1000.0 * kLsubf;
        c.snomlt = c.sneqv / dt;
        c.sneqv = 0.0;
      }
    }
    prcpf += ex;
  }
  pcp_drp(c, prcpf, dt);
  const double zz1 = 1.0;
  const double yy = c.stc[0] - 0.5 * c.ssoil * c.zsoil[0] * zz1 / df1;
  const double t11 = c.t1;
  const double ssoil1 = c.ssoil;
  shflx(c, dt, yy, zz1, df1);
  c.t1 = t11;
  c.ssoil = ssoil1;
  if (c.sneqv > 0.0) {
    snow_pack(c.sneqv, dt, &c.snowh, &c.sndens, c.t1, yy);
  } else {
    c.sneqv = 0.0;
    c.snowh = 0.0;
    c.sndens = 0.0;
    c.sncovr = 0.0;
  }
}

// SFlx, :166-608 (Flux-PIHM, not Cycles)
__device__ inline void sflx(Col &c, double dt) {
  c.snomlt = 0.0;
  c.pcpdrp = 0.0;
  if (c.isurban) {
    c.shdfac = 0.05;
    c.rsmin = 400.0;
    c.smcmax = 0.45;
    c.smcmin = 0.0;
    c.smcref = 0.42;
    c.smcwlt = 0.40;
    c.smcdry = 0.40;
  }
  if (c.shdfac > 0.0) c.proj_lai = (c.proj_lai > 0.5) ? c.proj_lai : 0.5;
  c.cmcmax = c.shdfac * c.cmcfactr * c.proj_lai;
  if (c.proj_lai >= c.laimax) {
    c.embrd = c.emissmax;
    c.alb = c.albedomin;
    c.z0brd = c.z0max;
  } else if (c.proj_lai <= c.laimin) {
    c.embrd = c.emissmin;
    c.alb = c.albedomax;
    c.z0brd = c.z0min;
  } else {
    if (c.laimax > c.laimin) {
      double f = (c.proj_lai - c.laimin) / (c.laimax - c.laimin);
      f = (f < 1.0) ? f : 1.0;
      f = (f > 0.0) ? f : 0.0;
      c.embrd = ((1.0 - f) * c.emissmin) + (f * c.emissmax);
      c.alb = ((1.0 - f) * c.albedomax) + (f * c.albedomin);
      c.z0brd = ((1.0 - f) * c.z0min) + (f * c.z0max);
    } else {
      c.embrd = 0.5 * c.emissmin + 0.5 * c.emissmax;
      c.alb = 0.5 * c.albedomin + 0.5 * c.albedomax;
      c.z0brd = 0.5 * c.z0min + 0.5 * c.z0max;
    }
  }
  int snowng = 0, frzgra = 0;
  if (c.sneqv <= 1.0e-7) {
    c.sneqv = 0.0;
    c.sndens = 0.0;
    c.snowh = 0.0;
    c.sncond = 1.0;
  } else {
    // the reference exits when the snow density exceeds one; the kernel
    // reports it through the context's error word
    c.sndens = c.sneqv / c.snowh;
    c.sncond = csnow(c.sndens);
  }
  if (c.prcp > 0.0) {
    if (c.ffrozp > 0.5) snowng = 1;
    else if (c.t1 <= kTfreez) frzgra = 1;
  }
  double prcpf;
  if (snowng || frzgra) {
    const double sn_new = c.prcp * dt;
    c.sneqv += sn_new;
    prcpf = 0.0;
    snow_new(c, sn_new);
    c.sncond = csnow(c.sndens);
  } else {
    prcpf = c.prcp;
  }
  if (c.sneqv == 0.0) {
    c.sncovr = 0.0;
    c.albedo = c.alb;
    c.emissi = c.embrd;
  } else {
    c.sncovr = snfrac(c.sneqv, c.snup, c.salp);
    c.sncovr = (c.sncovr < 0.98) ? c.sncovr : 0.98;
    al_calc(c, dt, snowng);
  }
  double df1 = tdf_cnd(c.smc[0], c.quartz, c.smcmax, c.smcmin, c.sh2o[0]);
  if (c.isurban) df1 = 3.24;
  df1 *= exp(c.sbeta * c.shdfac);
  if (c.sncovr > 0.97) df1 = c.sncond;
  const double dsoil = -(0.5 * c.zsoil[0]);
  if (c.sneqv == 0.0) {
    c.ssoil = df1 * (c.t1 - c.stc[0]) / dsoil;
  } else {
    const double dtot = c.snowh + dsoil;
    const double frcsno = c.snowh / dtot;
    const double frcsoi = dsoil / dtot;
    const double df1a = frcsno * c.sncond + frcsoi * df1;
    df1 = df1a * c.sncovr + df1 * (1.0 - c.sncovr);
    c.ssoil = df1 * (c.t1 - c.stc[0]) / dtot;
  }
  if (c.sncovr > 0.0) c.z0 = snowz0(c.sncovr, c.z0brd, c.snowh);
  else c.z0 = c.z0brd;
  const double t1v = c.t1 * (1.0 + 0.61 * c.q2);
  const double th2v = c.th2 * (1.0 + 0.61 * c.q2);
  sfcdif_off(c, t1v, th2v);
  c.fdown = c.solnet + c.lwdn;
  const double t2v = c.sfctmp * (1.0 + 0.61 * c.q2);
  double t24;
  penman(c, &t24, t2v, snowng, frzgra);
  if (c.shdfac > 0.0) can_res(c);
  else c.rc = 0.0;
  c.esnow = 0.0;
  if (c.sneqv == 0.0) {
    nopac(c, dt, t24);
    c.eta_kinematic = c.eta * 1000.0;
  } else {
    snopac(c, snowng, dt, t24, prcpf, df1);
    c.eta_kinematic = (c.esnow + c.etns) * 1000.0;
  }
  c.q1 = c.q2 + c.eta_kinematic * kCp / c.rch;
  c.sheat = -(c.ch * kCp * c.sfcprs) / (kRd * t2v) * (c.th2 - c.t1);
  c.ef_edir = c.edir * 1000.0 * kLvh2o;
  c.ef_ec = c.ec * 1000.0 * kLvh2o;
  c.ef_ett = c.ett * 1000.0 * kLvh2o;
  c.ef_esnow = c.esnow * 1000.0 * kLsubs;
  c.ef_etp = c.etp * 1000.0 * ((1.0 - c.sncovr) * kLvh2o + c.sncovr * kLsubs);
  if (c.ef_etp > 0.0) c.ef_eta = c.ef_edir + c.ef_ec + c.ef_ett + c.ef_esnow;
  else c.ef_eta = c.ef_etp;
  c.beta_s = (c.ef_etp == 0.0) ? 0.0 : (c.ef_eta / c.ef_etp);
  c.ssoil *= -1.0;
  c.soilm = -1.0 * c.smc[0] * c.zsoil[0];
  for (int k = 1; k < c.nsoil; k++) c.soilm += c.smc[k] * (c.zsoil[k - 1] - c.zsoil[k]);
  double soilwm = -1.0 * (c.smcmax - c.smcwlt) * c.zsoil[0];
  double soilww = -1.0 * (c.smc[0] - c.smcwlt) * c.zsoil[0];
  if (c.nroot > 1) {
    for (int k = 1; k < c.nroot; k++) {
      soilwm += (c.smcmax - c.smcwlt) * (c.zsoil[k - 1] - c.zsoil[k]);
      soilww += (c.smc[k] - c.smcwlt) * (c.zsoil[k - 1] - c.zsoil[k]);
    }
  }
  if (soilwm < 1.0e-6) {
    soilwm = 0.0;
    c.soilw = 0.0;
    c.soilm = 0.0;
  } else {
    c.soilw = soilww / soilwm;
  }
}

// Noah's per-element body, src/noah/noah.c:3-55: humidity, frozen
// precipitation, net radiation with the previous step's albedo and
// emissivity, the moisture clamps, SFlx, and the evaporation terms back
// from energy units (as the reference converts them)
__device__ inline void noah_step(Col &c, double dt) {
  cal_hum(c);
  c.ffrozp = froz_rain(c.prcp, c.sfctmp);
  c.alb = kBadVal;
  if (c.q1 == kBadVal) c.q1 = c.q2;
  c.solnet = c.soldn * (1.0 - c.albedo);
  c.lwdn = c.longwave * c.emissi;
  for (int j = 0; j < c.nsoil; j++) {
    c.smc[j] = (c.smc[j] > c.smcmin + kSh2oMin) ? c.smc[j] : c.smcmin + kSh2oMin;
    c.smc[j] = (c.smc[j] < c.smcmax) ? c.smc[j] : c.smcmax;
    c.sh2o[j] = (c.sh2o[j] < c.smc[j]) ? c.sh2o[j] : c.smc[j];
  }
  sflx(c, dt);
  c.ec = c.ef_ec / kLvh2o / 1000.0;
  c.ett = c.ef_ett / kLvh2o / 1000.0;
  c.edir = c.ef_edir / kLvh2o / 1000.0;
}

// ---------------------------------------------------------------------------
// Soil moisture: SmFlx and what it calls
// ---------------------------------------------------------------------------

// KrFunc, src/soil.c:8-13
__device__ inline double kr_func(double beta, double satn) {
  return sqrt(satn) * (1.0 - pow_any(1.0 - pow_any(satn, beta / (beta - 1.0)), (beta - 1.0) / beta)) *
         (1.0 - pow_any(1.0 - pow_any(satn, beta / (beta - 1.0)), (beta - 1.0) / beta));
}

// WDfCnd, :2813-2860
__device__ inline void wdf_cnd(const Col &c, double *wdf, double *wcnd, double smc, double sicemax) {
  double factr1 = 0.05 / (c.smcmax - c.smcmin);
  double factr2 = (smc - c.smcmin) / (c.smcmax - c.smcmin);
  factr2 = (factr2 > 1.0 - 5.0e-4) ? 1.0 - 5.0e-4 : factr2;
  factr2 = (factr2 < 0.0 + 5.0e-4) ? 5.0e-4 : factr2;
  factr1 = (factr1 < factr2) ? factr1 : factr2;
  const double expon = 1.0 - 1.0 / c.beta;
  double satkfunc = kr_func(c.beta, factr2);
  double dpsidsm = (1.0 - expon) / c.alpha / expon / (c.smcmax - c.smcmin) *
                   pow_any(pow_any(factr2, -1.0 / expon) - 1.0, -expon) * pow_any(factr2, -(1.0 / expon + 1.0));
  *wcnd = c.ksatv * satkfunc;
  *wdf = *wcnd * dpsidsm;
  if (sicemax > 0.0) {
    const double vkwgt = 1.0 / (1.0 + pow_any(500.0 * sicemax, 3.0));
    satkfunc = kr_func(c.beta, factr1);
    dpsidsm = (1.0 - expon) / c.alpha / expon / (c.smcmax - c.smcmin) *
              pow_any(pow_any(factr1, -1.0 / expon) - 1.0, -expon) * pow_any(factr1, -(1.0 / expon + 1.0));
    *wdf = vkwgt * *wdf + (1.0 - vkwgt) * dpsidsm * satkfunc * c.ksatv;
  }
}

// SRT, :2270-2425 (Flux-PIHM: the infiltration is MassBalance's, the
// lateral runoff of each layer is CalcLatFlx's)
__device__ inline void srt(Col &c, double *rhstt, const double *sice, double *ai, double *bi, double *ci) {
  const double CVFRZ = 3.0;
  double sicemax = 0.0;
  for (int ks = 0; ks < c.nsoil; ks++) sicemax = (sice[ks] > sicemax) ? sice[ks] : sicemax;
  double dice = -c.zsoil[0] * sice[0];
  for (int ks = 1; ks < c.nsoil; ks++) dice += (c.zsoil[ks - 1] - c.zsoil[ks]) * sice[ks];
  c.fcr = 1.0;
  if (dice > 1.0e-2) {
    const double acrt = CVFRZ * c.frzx / dice;
    double sum = 1.0;
    const int ialp1 = (int)round(CVFRZ) - 1;
    for (int j = 1; j < ialp1 + 1; j++) {
      int k = 1;
      for (int jj = j + 1; jj < ialp1; jj++) k *= jj;
      sum += pow_any(acrt, CVFRZ - (double)j) / (double)k;
    }
    c.fcr = 1.0 - exp(-acrt) * sum;
  }
  const double pddum = c.infil;
  const double mxsmc = c.sh2o[0];
  double dsmdz = (c.sh2o[0] - c.sh2o[1]) / (-0.5 * c.zsoil[1]);
  double wdf, wcnd;
  wdf_cnd(c, &wdf, &wcnd, mxsmc, sicemax);
  double ddz = 1.0 / (-0.5 * c.zsoil[1]);
  ai[0] = 0.0;
  bi[0] = wdf * ddz / (-c.zsoil[0]);
  ci[0] = -bi[0];
  rhstt[0] = (wdf * dsmdz + wcnd - pddum + c.edir + c.et[0]) / c.zsoil[0];
  rhstt[0] += c.runoff2_lyr[0] / c.zsoil[0];
  double ddz2 = 0.0;
  for (int k = 1; k < c.nsoil; k++) {
    const double denom2 = (c.zsoil[k - 1] - c.zsoil[k]);
    double wdf2, wcnd2, dsmdz2;
    if (k < c.nsoil - 1) {
      const double mxsmc2 = c.sh2o[k];
      const double denom = c.zsoil[k - 1] - c.zsoil[k + 1];
      dsmdz2 = (c.sh2o[k] - c.sh2o[k + 1]) / (denom * 0.5);
      wdf_cnd(c, &wdf2, &wcnd2, mxsmc2, sicemax);
      ddz2 = 2.0 / denom;
      ci[k] = -wdf2 * ddz2 / denom2;
    } else {
      wdf2 = 0.0;
      wcnd2 = 0.0;
      dsmdz2 = 0.0;
      ci[k] = 0.0;
    }
    double numer = (wdf2 * dsmdz2) + wcnd2 - (wdf * dsmdz) - wcnd + c.et[k];
    numer += c.runoff2_lyr[k];
    rhstt[k] = numer / (-denom2);
    ai[k] = -wdf * ddz / denom2;
    bi[k] = -(ai[k] + ci[k]);
    if (k != c.nsoil - 1) {
      wdf = wdf2;
      wcnd = wcnd2;
      dsmdz = dsmdz2;
      ddz = ddz2;
    }
  }
}

// AdjSmProf, :3081-3171
__device__ inline void adj_sm_prof(Col &c, const double *sice, double dt) {
  double sh2omid[L];
  double wplus = 0.0, ddz;
  c.runoff3 = 0.0;
  for (int k = c.nsoil - 1; k >= 0; k--) {
    ddz = (k != 0) ? c.zsoil[k - 1] - c.zsoil[k] : -c.zsoil[0];
    sh2omid[k] = c.sh2o[k] + wplus / ddz;
    const double stot = sh2omid[k] + sice[k];
    if (stot > c.smcmax) {
      c.smc[k] = c.smcmax;
      wplus = (stot - c.smcmax) * ddz;
    } else {
      double stotmin = (c.satdpth[k] * c.smcmax + (c.sldpth[k] - c.satdpth[k]) * (c.smcmin + kSh2oMin)) / c.sldpth[k];
      stotmin = (stotmin > c.smcmax) ? c.smcmax : stotmin;
      stotmin = (stotmin < c.smcmin + kSh2oMin) ? (c.smcmin + kSh2oMin) : stotmin;
      if (stot < stotmin) {
        c.smc[k] = stotmin;
        wplus = (stot - stotmin) * ddz;
      } else {
        c.smc[k] = stot;
        wplus = 0.0;
      }
    }
    sh2omid[k] = c.smc[k] - sice[k];
  }
  ddz = -c.zsoil[0];
  for (int k = 0; k < c.nsoil; k++) {
    if (k != 0) ddz = c.zsoil[k - 1] - c.zsoil[k];
    c.sh2o[k] = sh2omid[k] + wplus / ddz;
    const double stot = c.sh2o[k] + sice[k];
    wplus = (stot > c.smcmax) ? (stot - c.smcmax) * ddz : 0.0;
    c.smc[k] = (stot < c.smcmax) ? stot : c.smcmax;
    c.smc[k] = (c.smc[k] > c.smcmin + kSh2oMin) ? c.smc[k] : (c.smcmin + kSh2oMin);
    c.sh2o[k] = c.smc[k] - sice[k];
    c.sh2o[k] = (c.sh2o[k] > 0.0) ? c.sh2o[k] : 0.0;
  }
  c.runoff3 = wplus / dt;
}

// SStep, :2427-2480
__device__ inline void sstep(Col &c, double *rhstt, const double *sice, double *ai, double *bi, double *ci,
                             double dt) {
  double rhsttin[L], ciin[L], sh2o0[L];
  const int n = c.nsoil;
  for (int k = 0; k < n; k++) {
    rhstt[k] *= dt;
    ai[k] *= dt;
    bi[k] = 1.0 + bi[k] * dt;
    ci[k] *= dt;
    sh2o0[k] = c.sh2o[k];
    c.smflxv[k] = 0.0;
  }
  for (int k = 0; k < n; k++) {
    rhsttin[k] = rhstt[k];
    ciin[k] = ci[k];
  }
  rosr12(ci, ai, bi, ciin, rhsttin, rhstt, n);
  for (int k = 0; k < n; k++) c.sh2o[k] += ci[k];
  adj_sm_prof(c, sice, dt);
  for (int k = n - 1; k > 0; k--)
    c.smflxv[k - 1] = (c.sh2o[k] - sh2o0[k]) * c.sldpth[k] / dt + c.runoff2_lyr[k] + c.et[k] + c.smflxv[k];
}

// SmFlx, :1654-1711
__device__ inline void smflx(Col &c, double dt) {
  double ai[L], bi[L], ci[L], rhstt[L], sice[L];
  for (int i = 0; i < c.nsoil; i++) sice[i] = c.smc[i] - c.sh2o[i];
  if (0 == c.nwtbl) {
    for (int i = 0; i < c.nsoil; i++) {
      c.smc[i] = c.smcmax;
      c.sh2o[i] = c.smc[i] - sice[i];
    }
  } else {
    srt(c, rhstt, sice, ai, bi, ci);
    sstep(c, rhstt, sice, ai, bi, ci, dt);
  }
}

// NoahHydrol's per-element body, src/noah/noah.c:57-97
__device__ inline void noah_hydrol(Col &c, double gw, double dt) {
  c.nwtbl = find_water_table(c.sldpth, c.nsoil, gw, c.satdpth);
  for (int k = 0; k < c.nsoil; k++) {
    c.smc[k] = (c.smc[k] > c.smcmin + kSh2oMin) ? c.smc[k] : c.smcmin + kSh2oMin;
    c.smc[k] = (c.smc[k] < c.smcmax) ? c.smc[k] : c.smcmax;
    c.sh2o[k] = (c.sh2o[k] < c.smc[k]) ? c.sh2o[k] : c.smc[k];
  }
  smflx(c, dt);
}

}  // namespace noah
}  // namespace pihm
