// Derived from SUNDIALS 2.7.0 (CVODE 2.9.0). Copyright (c) 2002-2016,
// Lawrence Livermore National Security; produced at the Lawrence Livermore
// National Laboratory (UCRL-CODE-155951). Redistributed under the SUNDIALS
// BSD-3 licence: its full text, conditions and disclaimer are in
// pihm-cuda_gb300/NOTICE.SUNDIALS.
//
// Variable-order BDF integrator with Newton iteration and unpreconditioned
// GMRES, restating the algorithm of CVODE 2.9.0 (SUNDIALS 2.7.0) as PIHM
// configures it (src/ode.c:413-529: CV_BDF, CV_NEWTON, scalar tolerances,
// initial step, stability limit detection on, max step = model step,
// CVSpgmr with PREC_NONE and maxl = 5).
//
// BdfCore<Ops> is written as C++20 coroutines over an operations policy: every
// vector operation and every right-hand-side evaluation is `co_await`ed.  The
// single-system entry points (bdf.cpp) use operations that complete at once,
// so a solve runs straight through; the batch engine (batch.cu) uses
// operations that suspend, so hundreds of systems -- each with its own step
// size, order and Newton/Krylov history -- advance together while their
// identical operations are executed as one launch.
//
// Function-by-function correspondence (cvode/src/cvode/cvode.c of the
// reference tree unless noted):
//   solve            CVode                       :1074-1500
//   ewt_set          cvEwtSetSS                  :4081-4090
//   hin / upper_bound_h0 / ydd_norm              :1812-2003
//   step             cvStep                      :2005-2076
//   adjust_params / increase_bdf / decrease_bdf / rescale  :2078-2275
//   predict / set_bdf / set_tq_bdf               :2277-2537
//   nls_newton / newton_iteration                :2651-2832
//   handle_nflag / restore / do_error_test       :2834-2994
//   complete_step / prepare_next_step / set_eta / compute_etaqm1 /
//   compute_etaqp1 / choose_eta                  :2996-3247
//   bdf_stab / sl_det                            :3249-3600
//   get_dky          CVodeGetDky                 :1509-1560
//   lsolve / spgmr   CVSpgmrSolve (cvode_spgmr.c:366-420), SpgmrSolve
//                    (sundials/sundials_spgmr.c:165-405), ModifiedGS, QRfact,
//                    QRsol (sundials/sundials_iterative.c)
//   dq_atimes        CVSpilsDQJtimes + CVSpilsAtimes (cvode_spils.c:665-705)
// The constants are CVODE's (cvode.c:206-240, cvode_spils.h:52-64).
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdlib>

#include "coro.h"

namespace pihm {
namespace bdf {

constexpr double ZERO = 0.0, ONE = 1.0, TWO = 2.0, HALF = 0.5, FOUR = 4.0, FOURTH = 0.25, THREE = 3.0;
constexpr double HUNDRED = 100.0, TINY = 1.0e-10, POINT2 = 0.2, PT25 = 0.25;
constexpr double FUZZ_FACTOR = 100.0, HLB_FACTOR = 100.0, HUB_FACTOR = 0.1, H_BIAS = 0.5;
constexpr int MAX_ITERS = 4;
constexpr double CORTES = 0.1, THRESH = 1.5, ETAMX1 = 10000.0, ETAMX2 = 10.0, ETAMX3 = 10.0;
constexpr double ETAMXF = 0.2, ETAMIN = 0.1, ETACF = 0.25, ADDON = 0.000001;
constexpr double BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0, ONEPSM = 1.000001;
constexpr int SMALL_NST = 10, MXNCF = 10, MXNEF = 7, MXNEF1 = 3, SMALL_NEF = 2, LONG_WAIT = 10;
constexpr int NLS_MAXCOR = 3;
constexpr double CRDOWN = 0.3, RDIV = TWO;
constexpr double GS_FACTOR = 1000.0;
constexpr int QMAX = 5, L_MAX = QMAX + 1, NUM_TESTS = 5;
constexpr int MAXL = 5;
constexpr double EPLIN = 0.05;

// return codes (CVODE's values)
enum {
  SUCCESS = 0, TSTOP_RETURN = 1, TOO_MUCH_WORK = -1, TOO_MUCH_ACC = -2, ERR_FAILURE = -3,
  CONV_FAILURE = -4, LSOLVE_FAIL = -7, RHSFUNC_FAIL = -8, FIRST_RHSFUNC_ERR = -9,
  REPTD_RHSFUNC_ERR = -10, UNREC_RHSFUNC_ERR = -11, MEM_FAIL = -20, ILL_INPUT = -22, TOO_CLOSE = -27
};
// internal flags (cvode_impl.h / cvode.c)
enum { FIRST_CALL = 123, PREV_CONV_FAIL = 124, PREV_ERR_FAIL = 125 };
enum { DO_ERROR_TEST = 2, PREDICT_AGAIN = 3, CONV_FAIL = 4, TRY_AGAIN = 5, RHSFUNC_RECVR = 9 };
enum { SPGMR_SUCCESS = 0, SPGMR_RES_REDUCED = 1, SPGMR_CONV_FAIL = 2, SPGMR_QRFACT_FAIL = 3,
       SPGMR_ATIMES_FAIL_REC = 5, SPGMR_ATIMES_FAIL_UNREC = -2, SPGMR_GS_FAIL = -4,
       SPGMR_QRSOL_FAIL = -5 };

inline double sun_sqrt(double x) { return (x <= ZERO) ? ZERO : std::sqrt(x); }
inline double sun_powr(double b, double e) { return (b <= ZERO) ? ZERO : std::pow(b, e); }
inline double sun_powi(double b, int e) {
  double prod = ONE;
  const int expt = std::abs(e);
  for (int i = 1; i <= expt; i++) prod *= b;
  if (e < 0) prod = ONE / prod;
  return prod;
}
inline double sun_max(double a, double b) { return (a > b) ? a : b; }
inline double sun_min(double a, double b) { return (a < b) ? a : b; }

// A linear-sum coefficient held as a reduction result on the vectors' side
// (policies with device-resident scalars): a constant, or -s, 1/s, 1/(1/s),
// -(1/(1/s)) of slot s.
enum CoefKind { COEF_HOST = 0, COEF_NEG, COEF_INV, COEF_INV_INV, COEF_NEG_INV_INV };
struct Coef {
  int kind, slot;
  double value;
};
constexpr Coef host_coef(double v) { return {COEF_HOST, 0, v}; }

struct Stats {
  long nst, nfe, nni, ncfn, netf, nli, nfes, njtimes, ncfl, nor;
  int qlast, qcur;
  double hlast, hcur, tcur;
};

template <class Ops>
struct BdfCore {
  using Vec = typename Ops::Vec;
  Ops ops;
  // ---- configuration ----
  double reltol = 0, abstol = 0;
  bool tol_set = false;
  double hin = ZERO, hmin = ZERO, hmax_inv = ZERO;
  long mxstep = 500;
  bool sldeton = false;
  int qmax = QMAX, maxcor = NLS_MAXCOR, maxnef = MXNEF, maxncf = MXNCF;
  double nlscoef = CORTES;
  double tstop = ZERO;
  bool tstopset = false;
  int maxl = MAXL;
  double eplifac = EPLIN;
  double uround = DBL_EPSILON;
  // ---- vectors ----
  Vec zn[L_MAX]{};
  Vec ewt{}, y{}, acor{}, tempv{}, ftemp{};
  Vec V[MAXL + 1]{};
  Vec xcor{}, vtemp{}, xsol{}, ytemp{};
  Vec ycur{}, fcur{};
  double Hes[MAXL + 1][MAXL] = {{0}};
  double givens[2 * MAXL] = {0};
  double yg[MAXL + 1] = {0};
  // ---- step state ----
  double tn = 0, h = 0, hprime = 0, next_h = 0, eta = 0, etaqm1 = 0, etaq = 0, etaqp1 = 0;
  double hscale = 0, hu = 0, h0u = 0, tolsf = 1, etamax = ETAMX1, saved_tq5 = 0;
  double crate = 0, acnrm = 0, gamma = 0, gammap = 0, gamrat = 0, rl1 = 0;
  double tretlast = 0;
  double tau[L_MAX + 1] = {0};
  double tq[NUM_TESTS + 1] = {0};
  double l[L_MAX] = {0};
  int q = 1, qprime = 1, next_q = 0, qwait = 2, L = 2, qu = 0, indx_acor = QMAX, mnewt = 0;
  long nst = 0, nfe = 0, ncfn = 0, netf = 0, nni = 0, nhnil = 0, nscon = 0, nor = 0;
  double ssdat[6][4] = {{0}};
  long nli = 0, njtimes = 0, nfes = 0, ncfl = 0;
  double sqrtN = 0;
  bool alloc_done = false;

  // ---------------------------------------------------------------- setup
  // CVodeInit (cvode.c:420-520) + CVSpgmr's sqrtN (cvode_spgmr.c:201-203)
  Task<int> init(double t0, Vec y0) {
    if (!alloc_done) {
      ewt = ops.clone(y0);
      acor = ops.clone(y0);
      tempv = ops.clone(y0);
      ftemp = ops.clone(y0);
      for (int j = 0; j <= qmax; j++) zn[j] = ops.clone(y0);
      for (int i = 0; i <= maxl; i++) V[i] = ops.clone(y0);
      xcor = ops.clone(y0);
      vtemp = ops.clone(y0);
      xsol = ops.clone(y0);
      ytemp = ops.clone(y0);
      alloc_done = true;
      bool ok = ops.valid(ewt) && ops.valid(acor) && ops.valid(tempv) && ops.valid(ftemp) &&
                ops.valid(xcor) && ops.valid(vtemp) && ops.valid(xsol) && ops.valid(ytemp);
      for (int j = 0; j <= qmax; j++) ok = ok && ops.valid(zn[j]);
      for (int i = 0; i <= maxl; i++) ok = ok && ops.valid(V[i]);
      if (!ok) {
        release();
        co_return MEM_FAIL;
      }
      // sqrtN from a dot product of ones (CVSpgmr, cvode_spgmr.c:201-203)
      co_await ops.const_(ONE, ytemp);
      sqrtN = sun_sqrt(co_await ops.dot(ytemp, ytemp));
    }
    tn = t0;
    q = 1;
    L = 2;
    qwait = L;
    etamax = ETAMX1;
    qu = 0;
    hu = ZERO;
    tolsf = ONE;
    co_await ops.scale(ONE, y0, zn[0]);
    nst = nfe = ncfn = netf = nni = nhnil = nscon = 0;
    nli = njtimes = nfes = ncfl = 0;
    h0u = ZERO;
    next_h = ZERO;
    next_q = 0;
    nor = 0;
    for (int i = 1; i <= 5; i++)
      for (int k = 1; k <= 3; k++) ssdat[i][k] = ZERO;
    co_return SUCCESS;
  }

  void release() {
    if (!alloc_done) return;
    alloc_done = false;
    ops.destroy(ewt);
    ops.destroy(acor);
    ops.destroy(tempv);
    ops.destroy(ftemp);
    for (int j = 0; j <= qmax; j++) ops.destroy(zn[j]);
    for (int i = 0; i <= maxl; i++) ops.destroy(V[i]);
    ops.destroy(xcor);
    ops.destroy(vtemp);
    ops.destroy(xsol);
    ops.destroy(ytemp);
  }

  Stats stats() const {
    return Stats{nst, nfe, nni, ncfn, netf, nli, nfes, njtimes, ncfl, nor, qu, next_q, hu, next_h, tn};
  }

  // ---------------------------------------------------------------- weights
  Task<int> ewt_set(Vec ycur_, Vec weight) {
    co_await ops.abs_(ycur_, tempv);
    co_await ops.scale(reltol, tempv, tempv);
    co_await ops.addconst(tempv, abstol, tempv);
    if ((co_await ops.vmin(tempv)) <= ZERO) co_return -1;
    co_await ops.inv(tempv, weight);
    co_return 0;
  }

  // ---------------------------------------------------------------- initial step
  Task<double> upper_bound_h0(double tdist) {
    Vec temp1 = tempv, temp2 = acor;
    co_await ops.abs_(zn[0], temp2);
    (void)co_await ewt_set(zn[0], temp1);
    co_await ops.inv(temp1, temp1);
    co_await ops.linear_sum(HUB_FACTOR, temp2, ONE, temp1, temp1);
    co_await ops.abs_(zn[1], temp2);
    co_await ops.div(temp2, temp1, temp1);
    const double hub_inv = co_await ops.maxnorm(temp1);
    double hub = HUB_FACTOR * tdist;
    if (hub * hub_inv > ONE) hub = ONE / hub_inv;
    co_return hub;
  }

  Task<int> ydd_norm(double hg, double *yddnrm) {
    co_await ops.linear_sum(hg, zn[1], ONE, zn[0], y);
    const int retval = co_await ops.rhs(tn + hg, y, tempv);
    nfe++;
    if (retval < 0) co_return RHSFUNC_FAIL;
    if (retval > 0) co_return RHSFUNC_RECVR;
    co_await ops.linear_sum(ONE, tempv, -ONE, zn[1], tempv);
    co_await ops.scale(ONE / hg, tempv, tempv);
    *yddnrm = co_await ops.wrms(tempv, ewt);
    co_return SUCCESS;
  }

  Task<int> hin_estimate(double tout) {
    const double tdiff = tout - tn;
    if (tdiff == ZERO) co_return TOO_CLOSE;
    const int sign = (tdiff > ZERO) ? 1 : -1;
    const double tdist = std::fabs(tdiff);
    const double tround = uround * sun_max(std::fabs(tn), std::fabs(tout));
    if (tdist < TWO * tround) co_return TOO_CLOSE;
    const double hlb = HLB_FACTOR * tround;
    const double hub = co_await upper_bound_h0(tdist);
    double hg = sun_sqrt(hlb * hub);
    if (hub < hlb) {
      h = (sign == -1) ? -hg : hg;
      co_return SUCCESS;
    }
    bool hnewOK = false;
    double hs = hg, hnew = hg, yddnrm = 0;
    for (int count1 = 1; count1 <= MAX_ITERS; count1++) {
      bool hgOK = false;
      for (int count2 = 1; count2 <= MAX_ITERS; count2++) {
        const double hgs = hg * sign;
        const int retval = co_await ydd_norm(hgs, &yddnrm);
        if (retval < 0) co_return RHSFUNC_FAIL;
        if (retval == SUCCESS) {
          hgOK = true;
          break;
        }
        hg *= POINT2;
      }
      if (!hgOK) {
        if (count1 <= 2) co_return REPTD_RHSFUNC_ERR;
        hnew = hs;
        break;
      }
      hs = hg;
      if (hnewOK || count1 == MAX_ITERS) {
        hnew = hg;
        break;
      }
      hnew = (yddnrm * hub * hub > TWO) ? sun_sqrt(TWO / yddnrm) : sun_sqrt(hg * hub);
      const double hrat = hnew / hg;
      if (hrat > HALF && hrat < TWO) hnewOK = true;
      if (count1 > 1 && hrat > TWO) {
        hnew = hg;
        hnewOK = true;
      }
      hg = hnew;
    }
    double h0 = H_BIAS * hnew;
    if (h0 < hlb) h0 = hlb;
    if (h0 > hub) h0 = hub;
    if (sign == -1) h0 = -h0;
    h = h0;
    co_return SUCCESS;
  }

  // ---------------------------------------------------------------- history array
  Task<void> increase_bdf() {
    for (int i = 0; i <= qmax; i++) l[i] = ZERO;
    double alpha1, prod, xiold;
    l[2] = alpha1 = prod = xiold = ONE;
    double alpha0 = -ONE;
    double hsum = hscale;
    if (q > 1) {
      for (int j = 1; j < q; j++) {
        hsum += tau[j + 1];
        const double xi = hsum / hscale;
        prod *= xi;
        alpha0 -= ONE / (j + 1);
        alpha1 += ONE / xi;
        for (int i = j + 2; i >= 2; i--) l[i] = l[i] * xiold + l[i - 1];
        xiold = xi;
      }
    }
    const double A1 = (-alpha0 - alpha1) / prod;
    co_await ops.scale(A1, zn[indx_acor], zn[L]);
    for (int j = 2; j <= q; j++) co_await ops.linear_sum(l[j], zn[L], ONE, zn[j], zn[j]);
  }

  Task<void> decrease_bdf() {
    for (int i = 0; i <= qmax; i++) l[i] = ZERO;
    l[2] = ONE;
    double hsum = ZERO;
    for (int j = 1; j <= q - 2; j++) {
      hsum += tau[j];
      const double xi = hsum / hscale;
      for (int i = j + 2; i >= 2; i--) l[i] = l[i] * xi + l[i - 1];
    }
    for (int j = 2; j < q; j++) co_await ops.linear_sum(-l[j], zn[q], ONE, zn[j], zn[j]);
  }

  Task<void> adjust_order(int deltaq) {
    if (q == 2 && deltaq != 1) co_return;
    if (deltaq == 1) co_await increase_bdf();
    else if (deltaq == -1) co_await decrease_bdf();
  }

  Task<void> rescale() {
    double factor = eta;
    for (int j = 1; j <= q; j++) {
      co_await ops.scale(factor, zn[j], zn[j]);
      factor *= eta;
    }
    h = hscale * eta;
    next_h = h;
    hscale = h;
    nscon = 0;
  }

  Task<void> adjust_params() {
    if (qprime != q) {
      co_await adjust_order(qprime - q);
      q = qprime;
      L = q + 1;
      qwait = L;
    }
    co_await rescale();
  }

  Task<void> predict() {
    tn += h;
    if (tstopset) {
      if ((tn - tstop) * h > ZERO) tn = tstop;
    }
    for (int k = 1; k <= q; k++)
      for (int j = q; j >= k; j--) co_await ops.linear_sum(ONE, zn[j - 1], ONE, zn[j], zn[j - 1]);
  }

  void set_tq_bdf(double hsum, double alpha0, double alpha0_hat, double xi_inv, double xistar_inv) {
    const double A1 = ONE - alpha0_hat + alpha0;
    const double A2 = ONE + q * A1;
    tq[2] = std::fabs(A1 / (alpha0 * A2));
    tq[5] = std::fabs(A2 * xistar_inv / (l[q] * xi_inv));
    if (qwait == 1) {
      if (q > 1) {
        const double C = xistar_inv / l[q];
        const double A3 = alpha0 + ONE / q;
        const double A4 = alpha0_hat + xi_inv;
        const double Cpinv = (ONE - A4 + A3) / A3;
        tq[1] = std::fabs(C * Cpinv);
      } else {
        tq[1] = ONE;
      }
      hsum += tau[q];
      xi_inv = h / hsum;
      const double A5 = alpha0 - (ONE / (q + 1));
      const double A6 = alpha0_hat - xi_inv;
      const double Cppinv = (ONE - A6 + A5) / A2;
      tq[3] = std::fabs(Cppinv / (xi_inv * (q + 2) * A5));
    }
    tq[4] = nlscoef / tq[2];
  }

  void set_bdf() {
    double xi_inv, xistar_inv, alpha0, alpha0_hat, hsum;
    l[0] = l[1] = xi_inv = xistar_inv = ONE;
    for (int i = 2; i <= q; i++) l[i] = ZERO;
    alpha0 = alpha0_hat = -ONE;
    hsum = h;
    if (q > 1) {
      for (int j = 2; j < q; j++) {
        hsum += tau[j - 1];
        xi_inv = h / hsum;
        alpha0 -= ONE / j;
        for (int i = j; i >= 1; i--) l[i] += l[i - 1] * xi_inv;
      }
      alpha0 -= ONE / q;
      xistar_inv = -l[1] - alpha0;
      hsum += tau[q - 1];
      xi_inv = h / hsum;
      alpha0_hat = -l[1] - xi_inv;
      for (int i = q; i >= 1; i--) l[i] += l[i - 1] * xistar_inv;
    }
    set_tq_bdf(hsum, alpha0, alpha0_hat, xi_inv, xistar_inv);
  }

  void set_coefficients() {
    set_bdf();
    rl1 = ONE / l[1];
    gamma = h * rl1;
    if (nst == 0) gammap = gamma;
    gamrat = (nst > 0) ? gamma / gammap : ONE;
  }

  // ---------------------------------------------------------------- GMRES
  Task<int> dq_atimes(Vec v, Vec z) {
    double sig = ONE / (co_await ops.wrms(v, ewt));
    int retval = 0;
    for (int iter = 0; iter < MAX_ITERS; iter++) {
      co_await ops.linear_sum(sig, v, ONE, ycur, ytemp);
      retval = co_await ops.rhs(tn, ytemp, z);
      nfes++;
      if (retval == 0) break;
      if (retval < 0) co_return -1;
      sig *= PT25;
    }
    if (retval > 0) co_return +1;
    const double siginv = ONE / sig;
    co_await ops.linear_sum(siginv, z, -siginv, fcur, z);
    njtimes++;
    co_await ops.linear_sum(ONE, v, -gamma, z, z);
    co_return 0;
  }

  Task<int> modified_gs(int k, int p, double *new_vk_norm) {
    const double vk_norm = sun_sqrt(co_await ops.dot(V[k], V[k]));
    const int k_minus_1 = k - 1;
    const int i0 = (k - p > 0) ? k - p : 0;
    for (int i = i0; i < k; i++) {
      Hes[i][k_minus_1] = co_await ops.dot(V[i], V[k]);
      co_await ops.linear_sum(ONE, V[k], -Hes[i][k_minus_1], V[i], V[k]);
    }
    *new_vk_norm = sun_sqrt(co_await ops.dot(V[k], V[k]));
    co_return co_await gs_reorthogonalize(k, i0, vk_norm, new_vk_norm);
  }

  // ModifiedGS after the first pass: reorthogonalise V[k] against V[i0..k-1]
  // when its norm dropped by more than GS_FACTOR
  Task<int> gs_reorthogonalize(int k, int i0, double vk_norm, double *new_vk_norm) {
    const int k_minus_1 = k - 1;
    double temp = GS_FACTOR * vk_norm;
    if ((temp + (*new_vk_norm)) != temp) co_return 0;
    double new_norm_2 = ZERO;
    for (int i = i0; i < k; i++) {
      const double new_product = co_await ops.dot(V[i], V[k]);
      temp = GS_FACTOR * Hes[i][k_minus_1];
      if ((temp + new_product) == temp) continue;
      Hes[i][k_minus_1] += new_product;
      co_await ops.linear_sum(ONE, V[k], -new_product, V[i], V[k]);
      new_norm_2 += new_product * new_product;
    }
    if (new_norm_2 != ZERO) {
      const double new_product = (*new_vk_norm) * (*new_vk_norm) - new_norm_2;
      *new_vk_norm = (new_product > ZERO) ? sun_sqrt(new_product) : ZERO;
    }
    co_return 0;
  }

  // ---- GMRES with device-resident scalars (policies that provide them) ----
  // Slots: the norm that sets the difference-quotient increment, ||V[k]||^2
  // before and after Gram-Schmidt, and the Hessenberg column.
  enum { SLOT_VNORM = 0, SLOT_VK = 1, SLOT_NEW = 2, SLOT_H = 3 };
  static constexpr bool kDeferredOps = requires(Ops &o, Vec v) { o.deferred_scalars(v); };

  bool deferred_scalars() {
    if constexpr (kDeferredOps) return ops.deferred_scalars(V[0]);
    else return false;
  }

  // One GMRES iteration: V[li] unscaled, the difference-quotient product
  // (dq_atimes), rescaled, and modified_gs's first pass, with the norm that
  // sets sig and the Gram-Schmidt dot products used where the vectors are
  // and read back together (with a deferred right-hand side's status) once.
  // The operations, their order and every value are those of the plain
  // iteration; only the round trips are fewer.
  Task<int> atimes_gs_deferred(int li, Vec weight, double *new_vk_norm) {
    const int k = li + 1;
    co_await ops.div(V[li], weight, vtemp);
    // dq_atimes(vtemp, V[k]): sig = 1/||vtemp||_wrms
    co_await ops.wrms_slot(vtemp, ewt, SLOT_VNORM);
    co_await ops.linear_sum_coef({COEF_INV, SLOT_VNORM, 0}, vtemp, host_coef(ONE), ycur, ytemp);
    int retval = co_await ops.rhs_deferred(tn, ytemp, V[k]);
    nfes++;
    if (retval == 0) {
      co_await ops.linear_sum_coef({COEF_INV_INV, SLOT_VNORM, 0}, V[k], {COEF_NEG_INV_INV, SLOT_VNORM, 0}, fcur,
                                   V[k]);
    } else {
      // a right-hand side that reports at once and failed: dq_atimes's
      // retries with sig read back
      if (retval < 0) co_return -1;
      double s0[1];
      (void)co_await ops.fetch_slots(1, s0);
      double sig = ONE / s0[0];
      for (int iter = 1; iter < MAX_ITERS && retval > 0; iter++) {
        sig *= PT25;
        co_await ops.linear_sum(sig, vtemp, ONE, ycur, ytemp);
        retval = co_await ops.rhs(tn, ytemp, V[k]);
        nfes++;
        if (retval < 0) co_return -1;
      }
      if (retval > 0) co_return +1;
      const double siginv = ONE / sig;
      co_await ops.linear_sum(siginv, V[k], -siginv, fcur, V[k]);
    }
    njtimes++;
    co_await ops.linear_sum(ONE, vtemp, -gamma, V[k], V[k]);
    co_await ops.prod(weight, V[k], V[k]);
    // modified_gs(k, maxl): the first pass
    const int i0 = (k - maxl > 0) ? k - maxl : 0;
    co_await ops.dot_slot(V[k], V[k], SLOT_VK);
    for (int i = i0; i < k; i++) {
      co_await ops.dot_slot(V[i], V[k], SLOT_H + i);
      co_await ops.linear_sum_coef(host_coef(ONE), V[k], {COEF_NEG, SLOT_H + i, 0}, V[i], V[k]);
    }
    co_await ops.dot_slot(V[k], V[k], SLOT_NEW);
    double s[SLOT_H + MAXL];
    if ((co_await ops.fetch_slots(SLOT_H + k, s)) < 0) {
      njtimes--;  // the deferred evaluation failed: dq_atimes returns before counting it
      co_return -1;
    }
    for (int i = i0; i < k; i++) Hes[i][k - 1] = s[SLOT_H + i];
    *new_vk_norm = sun_sqrt(s[SLOT_NEW]);
    (void)co_await gs_reorthogonalize(k, i0, sun_sqrt(s[SLOT_VK]), new_vk_norm);
    co_return 0;
  }

  static void givens_pair(double temp1, double temp2, double *c, double *s) {
    if (temp2 == ZERO) {
      *c = ONE;
      *s = ZERO;
    } else if (std::fabs(temp2) >= std::fabs(temp1)) {
      const double temp3 = temp1 / temp2;
      *s = -ONE / sun_sqrt(ONE + temp3 * temp3);
      *c = -(*s) * temp3;
    } else {
      const double temp3 = temp2 / temp1;
      *c = ONE / sun_sqrt(ONE + temp3 * temp3);
      *s = -(*c) * temp3;
    }
  }

  // QRfact (sundials_iterative.c): job 0 factors the first column, otherwise
  // the new last column of an n-column Hessenberg matrix
  int qr_fact(int n, int job) {
    if (job == 0) {
      double c, s;
      givens_pair(Hes[0][0], Hes[1][0], &c, &s);
      const double temp1 = Hes[0][0], temp2 = Hes[1][0];
      givens[0] = c;
      givens[1] = s;
      return ((Hes[0][0] = c * temp1 - s * temp2) == ZERO) ? 1 : 0;
    }
    const int n_minus_1 = n - 1;
    for (int k = 0; k < n_minus_1; k++) {
      const int i = 2 * k;
      const double temp1 = Hes[k][n_minus_1], temp2 = Hes[k + 1][n_minus_1];
      const double c = givens[i], s = givens[i + 1];
      Hes[k][n_minus_1] = c * temp1 - s * temp2;
      Hes[k + 1][n_minus_1] = s * temp1 + c * temp2;
    }
    const double temp1 = Hes[n_minus_1][n_minus_1], temp2 = Hes[n][n_minus_1];
    double c, s;
    givens_pair(temp1, temp2, &c, &s);
    givens[2 * n_minus_1] = c;
    givens[2 * n_minus_1 + 1] = s;
    return ((Hes[n_minus_1][n_minus_1] = c * temp1 - s * temp2) == ZERO) ? n : 0;
  }

  int qr_sol(int n) {
    for (int k = 0; k < n; k++) {
      const double c = givens[2 * k], s = givens[2 * k + 1];
      const double temp1 = yg[k], temp2 = yg[k + 1];
      yg[k] = c * temp1 - s * temp2;
      yg[k + 1] = s * temp1 + c * temp2;
    }
    for (int k = n - 1; k >= 0; k--) {
      if (Hes[k][k] == ZERO) return k + 1;
      yg[k] /= Hes[k][k];
      for (int i = 0; i < k; i++) yg[i] -= yg[k] * Hes[i][k];
    }
    return 0;
  }

  // SpgmrSolve with x = 0 initially, s1 = s2 = weight, no preconditioning and
  // no restarts.  The solution is left in xsol.
  Task<int> spgmr(Vec b, Vec weight, double delta, int *nli_inc) {
    const int l_max = maxl;
    const bool deferred = deferred_scalars();
    int l_plus_1 = 0, krydim = 0;
    bool converged = false;
    *nli_inc = 0;
    // the initial guess is x = 0 (lsolve zeroes it), so r0 = b; SpgmrSolve
    // tests N_VDotProd(x, x) == 0 to find that out, a reduction skipped here.
    // SpgmrSolve then copies r0 through vtemp and V[0] (its preconditioning
    // stubs) before scaling, V[0] = s2 r0; the copies change no value and
    // vtemp is written before it is next read, so only the product is made.
    co_await ops.prod(weight, b, V[0]);
    double r_norm, beta, rho;
    r_norm = beta = sun_sqrt(co_await ops.dot(V[0], V[0]));
    if (r_norm <= delta) co_return SPGMR_SUCCESS;
    rho = beta;
    co_await ops.const_(ZERO, xcor);
    for (int i = 0; i <= l_max; i++)
      for (int j = 0; j < l_max; j++) Hes[i][j] = ZERO;
    double rotation_product = ONE;
    co_await ops.scale(ONE / r_norm, V[0], V[0]);
    for (int li = 0; li < l_max; li++) {
      (*nli_inc)++;
      krydim = l_plus_1 = li + 1;
      double hnorm = 0;
      bool iterated = false;
      if constexpr (kDeferredOps) {
        if (deferred) {
          const int ier = co_await atimes_gs_deferred(li, weight, &hnorm);
          if (ier != 0) co_return (ier < 0) ? SPGMR_ATIMES_FAIL_UNREC : SPGMR_ATIMES_FAIL_REC;
          iterated = true;
        }
      }
      if (!iterated) {
        co_await ops.div(V[li], weight, vtemp);
        const int ier = co_await dq_atimes(vtemp, V[l_plus_1]);
        if (ier != 0) co_return (ier < 0) ? SPGMR_ATIMES_FAIL_UNREC : SPGMR_ATIMES_FAIL_REC;
        // SpgmrSolve's copy through vtemp before the scaling changes no value
        co_await ops.prod(weight, V[l_plus_1], V[l_plus_1]);
        (void)co_await modified_gs(l_plus_1, l_max, &hnorm);
      }
      Hes[l_plus_1][li] = hnorm;
      if (qr_fact(krydim, li) != 0) co_return SPGMR_QRFACT_FAIL;
      rotation_product *= givens[2 * li + 1];
      rho = std::fabs(rotation_product * r_norm);
      if (rho <= delta) {
        converged = true;
        break;
      }
      co_await ops.scale(ONE / Hes[l_plus_1][li], V[l_plus_1], V[l_plus_1]);
    }
    yg[0] = r_norm;
    for (int i = 1; i <= krydim; i++) yg[i] = ZERO;
    if (qr_sol(krydim) != 0) co_return SPGMR_QRSOL_FAIL;
    for (int k = 0; k < krydim; k++) co_await ops.linear_sum(yg[k], V[k], ONE, xcor, xcor);
    if (converged || rho < beta) {
      co_await ops.div(xcor, weight, xcor);
      // SpgmrSolve's copy of xcor through vtemp changes no value
      co_await ops.linear_sum(ONE, xsol, ONE, xcor, xsol);
      co_return converged ? SPGMR_SUCCESS : SPGMR_RES_REDUCED;
    }
    co_return SPGMR_CONV_FAIL;
  }

  // CVSpgmrSolve, cvode_spgmr.c:366-420: solve (I - gamma J) x = b in place
  Task<int> lsolve(Vec b, Vec weight, Vec ynow, Vec fnow) {
    const double deltar = eplifac * tq[4];
    const double bnorm = co_await ops.wrms(b, weight);
    if (bnorm <= deltar) {
      if (mnewt > 0) co_await ops.const_(ZERO, b);
      co_return 0;
    }
    ycur = ynow;
    fcur = fnow;
    const double delta = deltar * sqrtN;
    co_await ops.const_(ZERO, xsol);
    int nli_inc = 0;
    const int retval = co_await spgmr(b, weight, delta, &nli_inc);
    co_await ops.scale(ONE, xsol, b);
    nli += nli_inc;
    if (retval != SPGMR_SUCCESS) ncfl++;
    switch (retval) {
      case SPGMR_SUCCESS: co_return 0;
      case SPGMR_RES_REDUCED: co_return (mnewt == 0) ? 0 : 1;
      case SPGMR_CONV_FAIL:
      case SPGMR_QRFACT_FAIL:
      case SPGMR_ATIMES_FAIL_REC: co_return 1;
      default: co_return -1;
    }
  }

  // ---------------------------------------------------------------- Newton
  Task<int> newton_iteration() {
    int m_it = 0;
    double del = ZERO, delp = ZERO;
    mnewt = 0;
    for (;;) {
      co_await ops.linear_sum(rl1, zn[1], ONE, acor, tempv);
      co_await ops.linear_sum(gamma, ftemp, -ONE, tempv, tempv);
      const int retval = co_await lsolve(tempv, ewt, y, ftemp);
      nni++;
      if (retval < 0) co_return LSOLVE_FAIL;
      if (retval > 0) co_return CONV_FAIL;
      del = co_await ops.wrms(tempv, ewt);
      co_await ops.linear_sum(ONE, acor, ONE, tempv, acor);
      co_await ops.linear_sum(ONE, zn[0], ONE, acor, y);
      if (m_it > 0) crate = sun_max(CRDOWN * crate, del / delp);
      const double dcon = del * sun_min(ONE, crate) / tq[4];
      if (dcon <= ONE) {
        acnrm = (m_it == 0) ? del : co_await ops.wrms(acor, ewt);
        co_return SUCCESS;
      }
      mnewt = ++m_it;
      if ((m_it == maxcor) || ((m_it >= 2) && (del > RDIV * delp))) co_return CONV_FAIL;
      delp = del;
      const int rv = co_await ops.rhs(tn, y, ftemp);
      nfe++;
      if (rv < 0) co_return RHSFUNC_FAIL;
      if (rv > 0) co_return RHSFUNC_RECVR;
    }
  }

  Task<int> nls_newton() {
    crate = ONE;  // PREC_NONE: no linear-solver setup
    const int retval = co_await ops.rhs(tn, zn[0], ftemp);
    nfe++;
    if (retval < 0) co_return RHSFUNC_FAIL;
    if (retval > 0) co_return RHSFUNC_RECVR;
    co_await ops.const_(ZERO, acor);
    co_await ops.scale(ONE, zn[0], y);
    co_return co_await newton_iteration();
  }

  Task<void> restore(double saved_t) {
    tn = saved_t;
    for (int k = 1; k <= q; k++)
      for (int j = q; j >= k; j--) co_await ops.linear_sum(ONE, zn[j - 1], -ONE, zn[j], zn[j - 1]);
  }

  Task<int> handle_nflag(int *nflagPtr, double saved_t, int *ncfPtr) {
    const int nflag = *nflagPtr;
    if (nflag == SUCCESS) co_return DO_ERROR_TEST;
    ncfn++;
    co_await restore(saved_t);
    if (nflag == LSOLVE_FAIL) co_return LSOLVE_FAIL;
    if (nflag == RHSFUNC_FAIL) co_return RHSFUNC_FAIL;
    (*ncfPtr)++;
    etamax = ONE;
    if ((std::fabs(h) <= hmin * ONEPSM) || (*ncfPtr == maxncf)) {
      if (nflag == CONV_FAIL) co_return CONV_FAILURE;
      if (nflag == RHSFUNC_RECVR) co_return REPTD_RHSFUNC_ERR;
    }
    eta = sun_max(ETACF, hmin / std::fabs(h));
    *nflagPtr = PREV_CONV_FAIL;
    co_await rescale();
    co_return PREDICT_AGAIN;
  }

  Task<int> do_error_test(int *nflagPtr, double saved_t, int *nefPtr, double *dsmPtr) {
    const double dsm = acnrm * tq[2];
    *dsmPtr = dsm;
    if (dsm <= ONE) co_return SUCCESS;
    (*nefPtr)++;
    netf++;
    *nflagPtr = PREV_ERR_FAIL;
    co_await restore(saved_t);
    if ((std::fabs(h) <= hmin * ONEPSM) || (*nefPtr == maxnef)) co_return ERR_FAILURE;
    etamax = ONE;
    if (*nefPtr <= MXNEF1) {
      eta = ONE / (sun_powr(BIAS2 * dsm, ONE / L) + ADDON);
      eta = sun_max(ETAMIN, sun_max(eta, hmin / std::fabs(h)));
      if (*nefPtr >= SMALL_NEF) eta = sun_min(eta, ETAMXF);
      co_await rescale();
      co_return TRY_AGAIN;
    }
    if (q > 1) {
      eta = sun_max(ETAMIN, hmin / std::fabs(h));
      co_await adjust_order(-1);
      L = q;
      q--;
      qwait = L;
      co_await rescale();
      co_return TRY_AGAIN;
    }
    eta = sun_max(ETAMIN, hmin / std::fabs(h));
    h *= eta;
    next_h = h;
    hscale = h;
    qwait = LONG_WAIT;
    nscon = 0;
    const int retval = co_await ops.rhs(tn, zn[0], tempv);
    nfe++;
    if (retval < 0) co_return RHSFUNC_FAIL;
    if (retval > 0) co_return UNREC_RHSFUNC_ERR;
    co_await ops.scale(h, tempv, zn[1]);
    co_return TRY_AGAIN;
  }

  Task<void> complete_step() {
    nst++;
    nscon++;
    hu = h;
    qu = q;
    for (int i = q; i >= 2; i--) tau[i] = tau[i - 1];
    if ((q == 1) && (nst > 1)) tau[2] = tau[1];
    tau[1] = h;
    for (int j = 0; j <= q; j++) co_await ops.linear_sum(l[j], acor, ONE, zn[j], zn[j]);
    qwait--;
    if ((qwait == 1) && (q != qmax)) {
      co_await ops.scale(ONE, acor, zn[qmax]);
      saved_tq5 = tq[5];
      indx_acor = qmax;
    }
  }

  void set_eta() {
    if (eta < THRESH) {
      eta = ONE;
      hprime = h;
    } else {
      eta = sun_min(eta, etamax);
      eta /= sun_max(ONE, std::fabs(h) * hmax_inv * eta);
      hprime = h * eta;
      if (qprime < q) nscon = 0;
    }
  }

  Task<double> compute_etaqm1() {
    etaqm1 = ZERO;
    if (q > 1) {
      const double ddn = (co_await ops.wrms(zn[q], ewt)) * tq[1];
      etaqm1 = ONE / (sun_powr(BIAS1 * ddn, ONE / q) + ADDON);
    }
    co_return etaqm1;
  }

  Task<double> compute_etaqp1() {
    etaqp1 = ZERO;
    if (q != qmax) {
      if (saved_tq5 == ZERO) co_return etaqp1;
      const double cquot = (tq[5] / saved_tq5) * sun_powi(h / tau[2], L);
      co_await ops.linear_sum(-cquot, zn[qmax], ONE, acor, tempv);
      const double dup = (co_await ops.wrms(tempv, ewt)) * tq[3];
      etaqp1 = ONE / (sun_powr(BIAS3 * dup, ONE / (L + 1)) + ADDON);
    }
    co_return etaqp1;
  }

  Task<void> choose_eta() {
    const double etam = sun_max(etaqm1, sun_max(etaq, etaqp1));
    if (etam < THRESH) {
      eta = ONE;
      qprime = q;
      co_return;
    }
    if (etam == etaq) {
      eta = etaq;
      qprime = q;
    } else if (etam == etaqm1) {
      eta = etaqm1;
      qprime = q - 1;
    } else {
      eta = etaqp1;
      qprime = q + 1;
      co_await ops.scale(ONE, acor, zn[qmax]);
    }
  }

  Task<void> prepare_next_step(double dsm) {
    if (etamax == ONE) {
      qwait = (qwait > 2) ? qwait : 2;
      qprime = q;
      hprime = h;
      eta = ONE;
      co_return;
    }
    etaq = ONE / (sun_powr(BIAS2 * dsm, ONE / L) + ADDON);
    if (qwait != 0) {
      eta = etaq;
      qprime = q;
      set_eta();
      co_return;
    }
    qwait = 2;
    etaqm1 = co_await compute_etaqm1();
    etaqp1 = co_await compute_etaqp1();
    co_await choose_eta();
    set_eta();
  }

  // cvSLdet, cvode.c:3336-3600
  int sl_det() {
    int kmin = 0, kflag = 0;
    double rat[5][4], rav[4], qkr[4], sigsq[4], smax[4], ssmax[4];
    double drr[4], rrc[4], sqmx[4], qjk[4][4], vrat[5], qc[6][4], qco[6][4];
    const double rrcut = 0.98, vrrtol = 1.0e-4, vrrt2 = 5.0e-4, sqtol = 1.0e-3, rrtol = 1.0e-2;
    double rr = ZERO, sqmin = ZERO;
    for (int k = 1; k <= 3; k++) {
      double smink = ssdat[1][k], smaxk = ZERO;
      for (int i = 1; i <= 5; i++) {
        smink = sun_min(smink, ssdat[i][k]);
        smaxk = sun_max(smaxk, ssdat[i][k]);
      }
      if (smink < TINY * smaxk) return -1;
      smax[k] = smaxk;
      ssmax[k] = smaxk * smaxk;
      double sumrat = ZERO, sumrsq = ZERO;
      for (int i = 1; i <= 4; i++) {
        rat[i][k] = ssdat[i][k] / ssdat[i + 1][k];
        sumrat = sumrat + rat[i][k];
        sumrsq = sumrsq + rat[i][k] * rat[i][k];
      }
      rav[k] = FOURTH * sumrat;
      vrat[k] = std::fabs(FOURTH * sumrsq - rav[k] * rav[k]);
      qc[5][k] = ssdat[1][k] * ssdat[3][k] - ssdat[2][k] * ssdat[2][k];
      qc[4][k] = ssdat[2][k] * ssdat[3][k] - ssdat[1][k] * ssdat[4][k];
      qc[3][k] = ZERO;
      qc[2][k] = ssdat[2][k] * ssdat[5][k] - ssdat[3][k] * ssdat[4][k];
      qc[1][k] = ssdat[4][k] * ssdat[4][k] - ssdat[3][k] * ssdat[5][k];
      for (int i = 1; i <= 5; i++) qco[i][k] = qc[i][k];
    }
    const double vmin = sun_min(vrat[1], sun_min(vrat[2], vrat[3]));
    const double vmax = sun_max(vrat[1], sun_max(vrat[2], vrat[3]));
    if (vmin < vrrtol * vrrtol) {
      if (vmax > vrrt2 * vrrt2) return -2;
      rr = (rav[1] + rav[2] + rav[3]) / THREE;
      double drrmax = ZERO;
      for (int k = 1; k <= 3; k++) {
        const double adrr = std::fabs(rav[k] - rr);
        drrmax = sun_max(drrmax, adrr);
      }
      if (drrmax > vrrt2) kflag = -3;
      kflag = 1;
    } else {
      if (std::fabs(qco[1][1]) < TINY * ssmax[1]) return -4;
      double tem = qco[1][2] / qco[1][1];
      for (int i = 2; i <= 5; i++) qco[i][2] = qco[i][2] - tem * qco[i][1];
      qco[1][2] = ZERO;
      tem = qco[1][3] / qco[1][1];
      for (int i = 2; i <= 5; i++) qco[i][3] = qco[i][3] - tem * qco[i][1];
      qco[1][3] = ZERO;
      if (std::fabs(qco[2][2]) < TINY * ssmax[2]) return -4;
      tem = qco[2][3] / qco[2][2];
      for (int i = 3; i <= 5; i++) qco[i][3] = qco[i][3] - tem * qco[i][2];
      if (std::fabs(qco[4][3]) < TINY * ssmax[3]) return -4;
      rr = -qco[5][3] / qco[4][3];
      if (rr < TINY || rr > HUNDRED) return -5;
      for (int k = 1; k <= 3; k++) qkr[k] = qc[5][k] + rr * (qc[4][k] + rr * rr * (qc[2][k] + rr * qc[1][k]));
      double sqmax = ZERO;
      for (int k = 1; k <= 3; k++) {
        const double saqk = std::fabs(qkr[k]) / ssmax[k];
        if (saqk > sqmax) sqmax = saqk;
      }
      if (sqmax < sqtol) {
        kflag = 2;
      } else {
        for (int it = 1; it <= 3; it++) {
          for (int k = 1; k <= 3; k++) {
            const double qp = qc[4][k] + rr * rr * (THREE * qc[2][k] + rr * FOUR * qc[1][k]);
            drr[k] = ZERO;
            if (std::fabs(qp) > TINY * ssmax[k]) drr[k] = -qkr[k] / qp;
            rrc[k] = rr + drr[k];
          }
          for (int k = 1; k <= 3; k++) {
            const double s = rrc[k];
            double sqmaxk = ZERO;
            for (int j = 1; j <= 3; j++) {
              qjk[j][k] = qc[5][j] + s * (qc[4][j] + s * s * (qc[2][j] + s * qc[1][j]));
              const double saqj = std::fabs(qjk[j][k]) / ssmax[j];
              if (saqj > sqmaxk) sqmaxk = saqj;
            }
            sqmx[k] = sqmaxk;
          }
          sqmin = sqmx[1] + ONE;
          for (int k = 1; k <= 3; k++) {
            if (sqmx[k] < sqmin) {
              kmin = k;
              sqmin = sqmx[k];
            }
          }
          rr = rrc[kmin];
          if (sqmin < sqtol) {
            kflag = 3;
            break;
          } else {
            for (int j = 1; j <= 3; j++) qkr[j] = qjk[j][kmin];
          }
        }
        if (sqmin > sqtol) return -6;
      }
    }
    for (int k = 1; k <= 3; k++) {
      const double rsa = ssdat[1][k];
      const double rsb = ssdat[2][k] * rr;
      const double rsc = ssdat[3][k] * rr * rr;
      const double rsd = ssdat[4][k] * rr * rr * rr;
      const double rd1a = rsa - rsb;
      const double rd1b = rsb - rsc;
      const double rd1c = rsc - rsd;
      const double rd2a = rd1a - rd1b;
      const double rd2b = rd1b - rd1c;
      const double rd3a = rd2a - rd2b;
      if (std::fabs(rd1b) < TINY * smax[k]) return -7;
      const double cest1 = -rd3a / rd1b;
      if (cest1 < TINY || cest1 > FOUR) return -7;
      const double corr1 = (rd2b / cest1) / (rr * rr);
      sigsq[k] = ssdat[3][k] + corr1;
    }
    if (sigsq[2] < TINY) return -8;
    const double ratp = sigsq[3] / sigsq[2];
    const double ratm = sigsq[1] / sigsq[2];
    const double qfac1 = FOURTH * (q * q - ONE);
    const double qfac2 = TWO / (q - ONE);
    const double bb = ratp * ratm - ONE - qfac1 * ratp;
    const double tem = ONE - qfac2 * bb;
    if (std::fabs(tem) < TINY) return -8;
    const double rrb = ONE / tem;
    if (std::fabs(rrb - rr) > rrtol) return -9;
    if (rr > rrcut) {
      if (kflag == 1) kflag = 4;
      if (kflag == 2) kflag = 5;
      if (kflag == 3) kflag = 6;
    }
    return kflag;
  }

  Task<void> bdf_stab() {
    if (q >= 3) {
      for (int k = 1; k <= 3; k++)
        for (int i = 5; i >= 2; i--) ssdat[i][k] = ssdat[i - 1][k];
      int factorial = 1;
      for (int i = 1; i <= q - 1; i++) factorial *= i;
      const double sq = factorial * q * (q + 1) * acnrm / sun_max(tq[5], TINY);
      const double sqm1 = factorial * q * (co_await ops.wrms(zn[q], ewt));
      const double sqm2 = factorial * (co_await ops.wrms(zn[q - 1], ewt));
      ssdat[1][1] = sqm2 * sqm2;
      ssdat[1][2] = sqm1 * sqm1;
      ssdat[1][3] = sq * sq;
    }
    if (qprime >= q) {
      if ((q >= 3) && (nscon >= q + 5)) {
        const int ldflag = sl_det();
        if (ldflag > 3) {
          qprime = q - 1;
          eta = etaqm1;
          eta = sun_min(eta, etamax);
          eta = eta / sun_max(ONE, std::fabs(h) * hmax_inv * eta);
          hprime = h * eta;
          nor = nor + 1;
        }
      }
    } else {
      nscon = 0;
    }
  }

  Task<int> step() {
    const double saved_t = tn;
    int ncf = 0, nef = 0;
    int nflag = FIRST_CALL;
    double dsm = 0;
    if ((nst > 0) && (hprime != h)) co_await adjust_params();
    for (;;) {
      co_await predict();
      set_coefficients();
      nflag = co_await nls_newton();
      const int kflag = co_await handle_nflag(&nflag, saved_t, &ncf);
      if (kflag == PREDICT_AGAIN) continue;
      if (kflag != DO_ERROR_TEST) co_return kflag;
      const int eflag = co_await do_error_test(&nflag, saved_t, &nef, &dsm);
      if (eflag == TRY_AGAIN) continue;
      if (eflag != SUCCESS) co_return eflag;
      break;
    }
    co_await complete_step();
    co_await prepare_next_step(dsm);
    if (sldeton) co_await bdf_stab();
    etamax = (nst <= SMALL_NST) ? ETAMX2 : ETAMX3;
    co_await ops.scale(tq[2], acor, acor);
    co_return SUCCESS;
  }

  Task<int> get_dky(double t, Vec dky) {
    double tfuzz = FUZZ_FACTOR * uround * (std::fabs(tn) + std::fabs(hu));
    if (hu < ZERO) tfuzz = -tfuzz;
    const double tp = tn - hu - tfuzz;
    const double tn1 = tn + tfuzz;
    if ((t - tp) * (t - tn1) > ZERO) co_return ILL_INPUT;
    const double s = (t - tn) / h;
    for (int j = q; j >= 0; j--) {
      if (j == q) co_await ops.scale(ONE, zn[q], dky);
      else co_await ops.linear_sum(ONE, zn[j], s, dky, dky);
    }
    co_return SUCCESS;
  }

  int set_stop_time(double t) {
    if (nst > 0 && (t - tn) * h < ZERO) return ILL_INPUT;
    tstop = t;
    tstopset = true;
    return SUCCESS;
  }

  int set_max_step(double hmax) {
    if (hmax < 0) return ILL_INPUT;
    if (hmax == ZERO) {
      hmax_inv = ZERO;
      return SUCCESS;
    }
    const double inv = ONE / hmax;
    if (inv * hmin > ONE) return ILL_INPUT;
    hmax_inv = inv;
    return SUCCESS;
  }

  // CVode(..., CV_NORMAL), cvode.c:1074-1500 (no root finding)
  Task<int> solve(double tout, Vec yout, double *tret) {
    if (!alloc_done || !tol_set) co_return ILL_INPUT;
    y = yout;
    int istate = SUCCESS;
    if (nst == 0) {
      tretlast = *tret = tn;
      if ((co_await ewt_set(zn[0], ewt)) != 0) co_return ILL_INPUT;
      const int retval = co_await ops.rhs(tn, zn[0], zn[1]);
      nfe++;
      if (retval < 0) co_return RHSFUNC_FAIL;
      if (retval > 0) co_return FIRST_RHSFUNC_ERR;
      if (tstopset && (tstop - tn) * (tout - tn) <= ZERO) co_return ILL_INPUT;
      h = hin;
      if (h != ZERO && (tout - tn) * h < ZERO) co_return ILL_INPUT;
      if (h == ZERO) {
        double tout_hin = tout;
        if (tstopset && (tout - tn) * (tout - tstop) > ZERO) tout_hin = tstop;
        const int hflag = co_await hin_estimate(tout_hin);
        if (hflag != SUCCESS) co_return hflag;
      }
      const double rh = std::fabs(h) * hmax_inv;
      if (rh > ONE) h /= rh;
      if (std::fabs(h) < hmin) h *= hmin / std::fabs(h);
      if (tstopset) {
        if ((tn + h - tstop) * h > ZERO) h = (tstop - tn) * (ONE - FOUR * uround);
      }
      hscale = h;
      h0u = h;
      hprime = h;
      co_await ops.scale(h, zn[1], zn[1]);
    }
    if (nst > 0) {
      const double troundoff = FUZZ_FACTOR * uround * (std::fabs(tn) + std::fabs(h));
      if ((tn - tout) * h >= ZERO) {
        tretlast = *tret = tout;
        if ((co_await get_dky(tout, yout)) != SUCCESS) co_return ILL_INPUT;
        co_return SUCCESS;
      }
      if (tstopset) {
        if (std::fabs(tn - tstop) <= troundoff) {
          if ((co_await get_dky(tstop, yout)) != SUCCESS) co_return ILL_INPUT;
          tretlast = *tret = tstop;
          tstopset = false;
          co_return TSTOP_RETURN;
        }
        if ((tn + hprime - tstop) * h > ZERO) {
          hprime = (tstop - tn) * (ONE - FOUR * uround);
          eta = hprime / h;
        }
      }
    }
    long nstloc = 0;
    for (;;) {
      next_h = h;
      next_q = q;
      if (nst > 0) {
        if ((co_await ewt_set(zn[0], ewt)) != 0) {
          istate = ILL_INPUT;
          tretlast = *tret = tn;
          co_await ops.scale(ONE, zn[0], yout);
          break;
        }
      }
      if ((mxstep > 0) && (nstloc >= mxstep)) {
        istate = TOO_MUCH_WORK;
        tretlast = *tret = tn;
        co_await ops.scale(ONE, zn[0], yout);
        break;
      }
      const double nrm = co_await ops.wrms(zn[0], ewt);
      tolsf = uround * nrm;
      if (tolsf > ONE) {
        istate = TOO_MUCH_ACC;
        tretlast = *tret = tn;
        co_await ops.scale(ONE, zn[0], yout);
        tolsf *= TWO;
        break;
      } else {
        tolsf = ONE;
      }
      if (tn + h == tn) nhnil++;
      const int kflag = co_await step();
      if (kflag != SUCCESS) {
        istate = kflag;
        tretlast = *tret = tn;
        co_await ops.scale(ONE, zn[0], yout);
        break;
      }
      nstloc++;
      if ((tn - tout) * h >= ZERO) {
        istate = SUCCESS;
        tretlast = *tret = tout;
        (void)co_await get_dky(tout, yout);
        next_q = qprime;
        next_h = hprime;
        break;
      }
      if (tstopset) {
        const double troundoff = FUZZ_FACTOR * uround * (std::fabs(tn) + std::fabs(h));
        if (std::fabs(tn - tstop) <= troundoff) {
          (void)co_await get_dky(tstop, yout);
          tretlast = *tret = tstop;
          tstopset = false;
          istate = TSTOP_RETURN;
          break;
        }
        if ((tn + hprime - tstop) * h > ZERO) {
          hprime = (tstop - tn) * (ONE - FOUR * uround);
          eta = hprime / h;
        }
      }
    }
    co_return istate;
  }
};

}  // namespace bdf
}  // namespace pihm
