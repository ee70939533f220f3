// Variable-order BDF integrator with Newton iteration and unpreconditioned
// GMRES, restating the algorithm of CVODE 2.9.0 (SUNDIALS 2.7.0) as PIHM
// configures it (src/ode.c:413-529: CV_BDF, CV_NEWTON, scalar tolerances,
// initial step, stability limit detection on, max step = model step,
// CVSpgmr with PREC_NONE and maxl = 5).  It drives any N_Vector through its
// operations table -- the device N_Vector of this library on the GPU, a host
// serial vector in the tests -- and calls the right-hand side through a
// CVRhsFn, so the sequence of right-hand-side evaluations (and therefore the
// carried river-edge flux of the PIHM right-hand side) is the one CVODE makes.
//
// Function-by-function correspondence (cvode/src/cvode/cvode.c of the
// reference tree unless noted):
//   solve            CVode                       :1074-1500
//   initial_setup    cvInitialSetup, cvEwtSetSS  :1730, :4081
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
//   spgmr_solve      CVSpgmrSolve (cvode_spgmr.c:366-420) + SpgmrSolve
//                    (sundials/sundials_spgmr.c:165-405), ModifiedGS, QRfact,
//                    QRsol (sundials/sundials_iterative.c)
//   dq_jtimes        CVSpilsDQJtimes, CVSpilsAtimes (cvode_spils.c:665-705)
// The constants are CVODE's (cvode.c:206-240, cvode_spils.h:52-64).
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "pihm_bdf.h"

namespace {

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
constexpr int MAXL_DEFAULT = 5;
constexpr double EPLIN = 0.05;

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

// N_Vector operations through the vector's own table
inline void NVLinearSum(double a, N_Vector x, double b, N_Vector y, N_Vector z) {
  z->ops->nvlinearsum(a, x, b, y, z);
}
inline void NVConst(double c, N_Vector z) { z->ops->nvconst(c, z); }
inline void NVScale(double c, N_Vector x, N_Vector z) { z->ops->nvscale(c, x, z); }
inline void NVAbs(N_Vector x, N_Vector z) { z->ops->nvabs(x, z); }
inline void NVInv(N_Vector x, N_Vector z) { z->ops->nvinv(x, z); }
inline void NVDiv(N_Vector x, N_Vector y, N_Vector z) { z->ops->nvdiv(x, y, z); }
inline void NVAddConst(N_Vector x, double b, N_Vector z) { z->ops->nvaddconst(x, b, z); }
inline double NVDot(N_Vector x, N_Vector y) { return x->ops->nvdotprod(x, y); }
inline double NVMaxNorm(N_Vector x) { return x->ops->nvmaxnorm(x); }
inline double NVWrms(N_Vector x, N_Vector w) { return x->ops->nvwrmsnorm(x, w); }
inline double NVMin(N_Vector x) { return x->ops->nvmin(x); }
inline N_Vector NVClone(N_Vector w) { return w->ops->nvclone(w); }
inline void NVDestroy(N_Vector v) {
  if (v) v->ops->nvdestroy(v);
}

}  // namespace

struct pihm_bdf {
  // ---- configuration ----
  pihm_bdf_rhs_fn f = nullptr;
  void *user_data = nullptr;
  double reltol = 0, abstol = 0;
  bool tol_set = false;
  double hin = ZERO, hmin = ZERO, hmax_inv = ZERO;
  long mxstep = 500;
  int mxhnil = 10;
  bool sldeton = false;
  int qmax = QMAX, maxcor = NLS_MAXCOR, maxnef = MXNEF, maxncf = MXNCF;
  double nlscoef = CORTES;
  double tstop = ZERO;
  bool tstopset = false;
  int maxl = MAXL_DEFAULT;
  double eplifac = EPLIN;
  double uround = DBL_EPSILON;
  // ---- vectors ----
  N_Vector zn[L_MAX] = {nullptr};
  N_Vector ewt = nullptr, y = nullptr, acor = nullptr, tempv = nullptr, ftemp = nullptr;
  N_Vector V[MAXL_DEFAULT + 1] = {nullptr};
  N_Vector xcor = nullptr, vtemp = nullptr, xsol = nullptr, ytemp = nullptr;
  N_Vector ycur = nullptr, fcur = nullptr;
  double Hes[MAXL_DEFAULT + 1][MAXL_DEFAULT] = {{0}};
  double givens[2 * MAXL_DEFAULT] = {0};
  double yg[MAXL_DEFAULT + 1] = {0};
  // ---- step state ----
  double tn = 0, h = 0, hprime = 0, next_h = 0, eta = 0, etaqm1 = 0, etaq = 0, etaqp1 = 0;
  double hscale = 0, hu = 0, h0u = 0, tolsf = 1, etamax = ETAMX1, saved_tq5 = 0;
  double crate = 0, acnrm = 0, gamma = 0, gammap = 0, gamrat = 0, rl1 = 0;
  double tretlast = 0, toutc = 0;
  double tau[L_MAX + 1] = {0};
  double tq[NUM_TESTS + 1] = {0};
  double l[L_MAX] = {0};
  int q = 1, qprime = 1, next_q = 0, qwait = 2, L = 2, qu = 0, indx_acor = QMAX, mnewt = 0;
  long nst = 0, nfe = 0, ncfn = 0, netf = 0, nni = 0, nhnil = 0, nstlp = 0, nscon = 0, nor = 0;
  double ssdat[6][4] = {{0}};
  // ---- linear solver statistics ----
  long nli = 0, njtimes = 0, nfes = 0, ncfl = 0;
  double sqrtN = 0;
  bool malloc_done = false;
};

namespace {

using Mem = pihm_bdf;

int ewt_set(Mem *m, N_Vector ycur, N_Vector weight) {
  // cvEwtSetSS, cvode.c:4081-4090
  NVAbs(ycur, m->tempv);
  NVScale(m->reltol, m->tempv, m->tempv);
  NVAddConst(m->tempv, m->abstol, m->tempv);
  if (NVMin(m->tempv) <= ZERO) return -1;
  NVInv(m->tempv, weight);
  return 0;
}

// ---------------------------------------------------------------------------
// initial step size
// ---------------------------------------------------------------------------
double upper_bound_h0(Mem *m, double tdist) {
  N_Vector temp1 = m->tempv, temp2 = m->acor;
  NVAbs(m->zn[0], temp2);
  ewt_set(m, m->zn[0], temp1);
  NVInv(temp1, temp1);
  NVLinearSum(HUB_FACTOR, temp2, ONE, temp1, temp1);
  NVAbs(m->zn[1], temp2);
  NVDiv(temp2, temp1, temp1);
  const double hub_inv = NVMaxNorm(temp1);
  double hub = HUB_FACTOR * tdist;
  if (hub * hub_inv > ONE) hub = ONE / hub_inv;
  return hub;
}

int ydd_norm(Mem *m, double hg, double *yddnrm) {
  NVLinearSum(hg, m->zn[1], ONE, m->zn[0], m->y);
  const int retval = m->f(m->tn + hg, m->y, m->tempv, m->user_data);
  m->nfe++;
  if (retval < 0) return PIHM_BDF_RHSFUNC_FAIL;
  if (retval > 0) return RHSFUNC_RECVR;
  NVLinearSum(ONE, m->tempv, -ONE, m->zn[1], m->tempv);
  NVScale(ONE / hg, m->tempv, m->tempv);
  *yddnrm = NVWrms(m->tempv, m->ewt);
  return PIHM_BDF_SUCCESS;
}

int hin_estimate(Mem *m, double tout) {
  double tdiff = tout - m->tn;
  if (tdiff == ZERO) return PIHM_BDF_TOO_CLOSE;
  const int sign = (tdiff > ZERO) ? 1 : -1;
  const double tdist = std::fabs(tdiff);
  const double tround = m->uround * sun_max(std::fabs(m->tn), std::fabs(tout));
  if (tdist < TWO * tround) return PIHM_BDF_TOO_CLOSE;
  const double hlb = HLB_FACTOR * tround;
  const double hub = upper_bound_h0(m, tdist);
  double hg = sun_sqrt(hlb * hub);
  if (hub < hlb) {
    m->h = (sign == -1) ? -hg : hg;
    return PIHM_BDF_SUCCESS;
  }
  bool hnewOK = false;
  double hs = hg, hnew = hg, yddnrm = 0;
  for (int count1 = 1; count1 <= MAX_ITERS; count1++) {
    bool hgOK = false;
    for (int count2 = 1; count2 <= MAX_ITERS; count2++) {
      const double hgs = hg * sign;
      const int retval = ydd_norm(m, hgs, &yddnrm);
      if (retval < 0) return PIHM_BDF_RHSFUNC_FAIL;
      if (retval == PIHM_BDF_SUCCESS) {
        hgOK = true;
        break;
      }
      hg *= POINT2;
    }
    if (!hgOK) {
      if (count1 <= 2) return PIHM_BDF_REPTD_RHSFUNC_ERR;
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
  m->h = h0;
  return PIHM_BDF_SUCCESS;
}

// ---------------------------------------------------------------------------
// Nordsieck history manipulation
// ---------------------------------------------------------------------------
void increase_bdf(Mem *m) {
  for (int i = 0; i <= m->qmax; i++) m->l[i] = ZERO;
  double alpha1, prod, xiold;
  m->l[2] = alpha1 = prod = xiold = ONE;
  double alpha0 = -ONE;
  double hsum = m->hscale;
  if (m->q > 1) {
    for (int j = 1; j < m->q; j++) {
      hsum += m->tau[j + 1];
      const double xi = hsum / m->hscale;
      prod *= xi;
      alpha0 -= ONE / (j + 1);
      alpha1 += ONE / xi;
      for (int i = j + 2; i >= 2; i--) m->l[i] = m->l[i] * xiold + m->l[i - 1];
      xiold = xi;
    }
  }
  const double A1 = (-alpha0 - alpha1) / prod;
  NVScale(A1, m->zn[m->indx_acor], m->zn[m->L]);
  for (int j = 2; j <= m->q; j++) NVLinearSum(m->l[j], m->zn[m->L], ONE, m->zn[j], m->zn[j]);
}

void decrease_bdf(Mem *m) {
  for (int i = 0; i <= m->qmax; i++) m->l[i] = ZERO;
  m->l[2] = ONE;
  double hsum = ZERO;
  for (int j = 1; j <= m->q - 2; j++) {
    hsum += m->tau[j];
    const double xi = hsum / m->hscale;
    for (int i = j + 2; i >= 2; i--) m->l[i] = m->l[i] * xi + m->l[i - 1];
  }
  for (int j = 2; j < m->q; j++) NVLinearSum(-m->l[j], m->zn[m->q], ONE, m->zn[j], m->zn[j]);
}

void adjust_order(Mem *m, int deltaq) {
  if (m->q == 2 && deltaq != 1) return;
  if (deltaq == 1) increase_bdf(m);
  else if (deltaq == -1) decrease_bdf(m);
}

void rescale(Mem *m) {
  double factor = m->eta;
  for (int j = 1; j <= m->q; j++) {
    NVScale(factor, m->zn[j], m->zn[j]);
    factor *= m->eta;
  }
  m->h = m->hscale * m->eta;
  m->next_h = m->h;
  m->hscale = m->h;
  m->nscon = 0;
}

void adjust_params(Mem *m) {
  if (m->qprime != m->q) {
    adjust_order(m, m->qprime - m->q);
    m->q = m->qprime;
    m->L = m->q + 1;
    m->qwait = m->L;
  }
  rescale(m);
}

void predict(Mem *m) {
  m->tn += m->h;
  if (m->tstopset) {
    if ((m->tn - m->tstop) * m->h > ZERO) m->tn = m->tstop;
  }
  for (int k = 1; k <= m->q; k++)
    for (int j = m->q; j >= k; j--) NVLinearSum(ONE, m->zn[j - 1], ONE, m->zn[j], m->zn[j - 1]);
}

void set_tq_bdf(Mem *m, double hsum, double alpha0, double alpha0_hat, double xi_inv, double xistar_inv) {
  const double A1 = ONE - alpha0_hat + alpha0;
  const double A2 = ONE + m->q * A1;
  m->tq[2] = std::fabs(A1 / (alpha0 * A2));
  m->tq[5] = std::fabs(A2 * xistar_inv / (m->l[m->q] * xi_inv));
  if (m->qwait == 1) {
    if (m->q > 1) {
      const double C = xistar_inv / m->l[m->q];
      const double A3 = alpha0 + ONE / m->q;
      const double A4 = alpha0_hat + xi_inv;
      const double Cpinv = (ONE - A4 + A3) / A3;
      m->tq[1] = std::fabs(C * Cpinv);
    } else {
      m->tq[1] = ONE;
    }
    hsum += m->tau[m->q];
    xi_inv = m->h / hsum;
    const double A5 = alpha0 - (ONE / (m->q + 1));
    const double A6 = alpha0_hat - xi_inv;
    const double Cppinv = (ONE - A6 + A5) / A2;
    m->tq[3] = std::fabs(Cppinv / (xi_inv * (m->q + 2) * A5));
  }
  m->tq[4] = m->nlscoef / m->tq[2];
}

void set_bdf(Mem *m) {
  double xi_inv, xistar_inv, alpha0, alpha0_hat, hsum;
  m->l[0] = m->l[1] = xi_inv = xistar_inv = ONE;
  for (int i = 2; i <= m->q; i++) m->l[i] = ZERO;
  alpha0 = alpha0_hat = -ONE;
  hsum = m->h;
  if (m->q > 1) {
    for (int j = 2; j < m->q; j++) {
      hsum += m->tau[j - 1];
      xi_inv = m->h / hsum;
      alpha0 -= ONE / j;
      for (int i = j; i >= 1; i--) m->l[i] += m->l[i - 1] * xi_inv;
    }
    alpha0 -= ONE / m->q;
    xistar_inv = -m->l[1] - alpha0;
    hsum += m->tau[m->q - 1];
    xi_inv = m->h / hsum;
    alpha0_hat = -m->l[1] - xi_inv;
    for (int i = m->q; i >= 1; i--) m->l[i] += m->l[i - 1] * xistar_inv;
  }
  set_tq_bdf(m, hsum, alpha0, alpha0_hat, xi_inv, xistar_inv);
}

void set_coefficients(Mem *m) {
  set_bdf(m);
  m->rl1 = ONE / m->l[1];
  m->gamma = m->h * m->rl1;
  if (m->nst == 0) m->gammap = m->gamma;
  m->gamrat = (m->nst > 0) ? m->gamma / m->gammap : ONE;
}

// ---------------------------------------------------------------------------
// GMRES (modified Gram-Schmidt, Givens QR, no restarts, no preconditioner)
// ---------------------------------------------------------------------------
int dq_atimes(Mem *m, N_Vector v, N_Vector z) {
  // CVSpilsDQJtimes: z = (f(t, y + sig v) - f(t, y)) / sig, then
  // CVSpilsAtimes: z = v - gamma z
  double sig = ONE / NVWrms(v, m->ewt);
  int retval = 0;
  for (int iter = 0; iter < MAX_ITERS; iter++) {
    NVLinearSum(sig, v, ONE, m->ycur, m->ytemp);
    retval = m->f(m->tn, m->ytemp, z, m->user_data);
    m->nfes++;
    if (retval == 0) break;
    if (retval < 0) return -1;
    sig *= PT25;
  }
  if (retval > 0) return +1;
  const double siginv = ONE / sig;
  NVLinearSum(siginv, z, -siginv, m->fcur, z);
  m->njtimes++;
  NVLinearSum(ONE, v, -m->gamma, z, z);
  return 0;
}

int modified_gs(Mem *m, int k, int p, double *new_vk_norm) {
  N_Vector *v = m->V;
  const double vk_norm = sun_sqrt(NVDot(v[k], v[k]));
  const int k_minus_1 = k - 1;
  const int i0 = (k - p > 0) ? k - p : 0;
  for (int i = i0; i < k; i++) {
    m->Hes[i][k_minus_1] = NVDot(v[i], v[k]);
    NVLinearSum(ONE, v[k], -m->Hes[i][k_minus_1], v[i], v[k]);
  }
  *new_vk_norm = sun_sqrt(NVDot(v[k], v[k]));
  double temp = GS_FACTOR * vk_norm;
  if ((temp + (*new_vk_norm)) != temp) return 0;
  double new_norm_2 = ZERO;
  for (int i = i0; i < k; i++) {
    const double new_product = NVDot(v[i], v[k]);
    temp = GS_FACTOR * m->Hes[i][k_minus_1];
    if ((temp + new_product) == temp) continue;
    m->Hes[i][k_minus_1] += new_product;
    NVLinearSum(ONE, v[k], -new_product, v[i], v[k]);
    new_norm_2 += new_product * new_product;
  }
  if (new_norm_2 != ZERO) {
    const double new_product = (*new_vk_norm) * (*new_vk_norm) - new_norm_2;
    *new_vk_norm = (new_product > ZERO) ? sun_sqrt(new_product) : ZERO;
  }
  return 0;
}

// QRfact with job != 0 (update by one column), sundials_iterative.c
int qr_fact_update(int n, double h[][MAXL_DEFAULT], double *q) {
  const int n_minus_1 = n - 1;
  int code = 0;
  for (int k = 0; k < n_minus_1; k++) {
    const int i = 2 * k;
    const double temp1 = h[k][n_minus_1], temp2 = h[k + 1][n_minus_1];
    const double c = q[i], s = q[i + 1];
    h[k][n_minus_1] = c * temp1 - s * temp2;
    h[k + 1][n_minus_1] = s * temp1 + c * temp2;
  }
  const double temp1 = h[n_minus_1][n_minus_1], temp2 = h[n][n_minus_1];
  double c, s;
  if (temp2 == ZERO) {
    c = ONE;
    s = ZERO;
  } else if (std::fabs(temp2) >= std::fabs(temp1)) {
    const double temp3 = temp1 / temp2;
    s = -ONE / sun_sqrt(ONE + temp3 * temp3);
    c = -s * temp3;
  } else {
    const double temp3 = temp2 / temp1;
    c = ONE / sun_sqrt(ONE + temp3 * temp3);
    s = -c * temp3;
  }
  const int q_ptr = 2 * n_minus_1;
  q[q_ptr] = c;
  q[q_ptr + 1] = s;
  if ((h[n_minus_1][n_minus_1] = c * temp1 - s * temp2) == ZERO) code = n;
  return code;
}

// QRfact with job == 0 (the first column: no earlier rotations)
int qr_fact_first(double h[][MAXL_DEFAULT], double *q) {
  const double temp1 = h[0][0], temp2 = h[1][0];
  double c, s;
  if (temp2 == ZERO) {
    c = ONE;
    s = ZERO;
  } else if (std::fabs(temp2) >= std::fabs(temp1)) {
    const double temp3 = temp1 / temp2;
    s = -ONE / sun_sqrt(ONE + temp3 * temp3);
    c = -s * temp3;
  } else {
    const double temp3 = temp2 / temp1;
    c = ONE / sun_sqrt(ONE + temp3 * temp3);
    s = -c * temp3;
  }
  q[0] = c;
  q[1] = s;
  return ((h[0][0] = c * temp1 - s * temp2) == ZERO) ? 1 : 0;
}

int qr_sol(int n, double h[][MAXL_DEFAULT], const double *q, double *b) {
  int code = 0;
  for (int k = 0; k < n; k++) {
    const int q_ptr = 2 * k;
    const double c = q[q_ptr], s = q[q_ptr + 1];
    const double temp1 = b[k], temp2 = b[k + 1];
    b[k] = c * temp1 - s * temp2;
    b[k + 1] = s * temp1 + c * temp2;
  }
  for (int k = n - 1; k >= 0; k--) {
    if (h[k][k] == ZERO) {
      code = k + 1;
      break;
    }
    b[k] /= h[k][k];
    for (int i = 0; i < k; i++) b[i] -= b[k] * h[i][k];
  }
  return code;
}

// SpgmrSolve with x = 0 initially, s1 = s2 = weight, no preconditioning and
// max_restarts = 0.  Solution returned in m->xsol.
int spgmr(Mem *m, N_Vector b, N_Vector weight, double delta, double *res_norm, int *nli) {
  const int l_max = m->maxl;
  N_Vector *V = m->V;
  int l_plus_1 = 0, krydim = 0;
  bool converged = false;
  *nli = 0;
  // the initial guess is x = 0 (lsolve zeroes it), so r0 = b; SpgmrSolve
  // tests N_VDotProd(x, x) == 0 to find that out, a reduction skipped here
  NVScale(ONE, b, m->vtemp);
  NVScale(ONE, m->vtemp, V[0]);
  NVScale(ONE, V[0], m->vtemp);
  V[0]->ops->nvprod(weight, m->vtemp, V[0]);
  double r_norm, beta, rho;
  *res_norm = r_norm = beta = sun_sqrt(NVDot(V[0], V[0]));
  if (r_norm <= delta) return SPGMR_SUCCESS;
  rho = beta;
  NVConst(ZERO, m->xcor);
  for (int i = 0; i <= l_max; i++)
    for (int j = 0; j < l_max; j++) m->Hes[i][j] = ZERO;
  double rotation_product = ONE;
  NVScale(ONE / r_norm, V[0], V[0]);
  for (int l = 0; l < l_max; l++) {
    (*nli)++;
    krydim = l_plus_1 = l + 1;
    NVDiv(V[l], weight, m->vtemp);
    int ier = dq_atimes(m, m->vtemp, V[l_plus_1]);
    if (ier != 0) return (ier < 0) ? SPGMR_ATIMES_FAIL_UNREC : SPGMR_ATIMES_FAIL_REC;
    NVScale(ONE, V[l_plus_1], m->vtemp);
    V[l_plus_1]->ops->nvprod(weight, m->vtemp, V[l_plus_1]);
    if (modified_gs(m, l_plus_1, l_max, &(m->Hes[l_plus_1][l])) != 0) return SPGMR_GS_FAIL;
    const int qr = (l == 0) ? qr_fact_first(m->Hes, m->givens) : qr_fact_update(krydim, m->Hes, m->givens);
    if (qr != 0) return SPGMR_QRFACT_FAIL;
    rotation_product *= m->givens[2 * l + 1];
    *res_norm = rho = std::fabs(rotation_product * r_norm);
    if (rho <= delta) {
      converged = true;
      break;
    }
    NVScale(ONE / m->Hes[l_plus_1][l], V[l_plus_1], V[l_plus_1]);
  }
  m->yg[0] = r_norm;
  for (int i = 1; i <= krydim; i++) m->yg[i] = ZERO;
  if (qr_sol(krydim, m->Hes, m->givens, m->yg) != 0) return SPGMR_QRSOL_FAIL;
  for (int k = 0; k < krydim; k++) NVLinearSum(m->yg[k], V[k], ONE, m->xcor, m->xcor);
  if (converged) {
    NVDiv(m->xcor, weight, m->xcor);
    NVScale(ONE, m->xcor, m->vtemp);
    NVLinearSum(ONE, m->xsol, ONE, m->vtemp, m->xsol);
    return SPGMR_SUCCESS;
  }
  if (rho < beta) {
    NVDiv(m->xcor, weight, m->xcor);
    NVScale(ONE, m->xcor, m->vtemp);
    NVLinearSum(ONE, m->xsol, ONE, m->vtemp, m->xsol);
    return SPGMR_RES_REDUCED;
  }
  return SPGMR_CONV_FAIL;
}

// CVSpgmrSolve, cvode_spgmr.c:366-420: solve (I - gamma J) x = b in place.
int lsolve(Mem *m, N_Vector b, N_Vector weight, N_Vector ynow, N_Vector fnow) {
  const double deltar = m->eplifac * m->tq[4];
  const double bnorm = NVWrms(b, weight);
  if (bnorm <= deltar) {
    if (m->mnewt > 0) NVConst(ZERO, b);
    return 0;
  }
  m->ycur = ynow;
  m->fcur = fnow;
  const double delta = deltar * m->sqrtN;
  NVConst(ZERO, m->xsol);
  double res_norm = 0;
  int nli_inc = 0;
  const int retval = spgmr(m, b, weight, delta, &res_norm, &nli_inc);
  NVScale(ONE, m->xsol, b);
  m->nli += nli_inc;
  if (retval != SPGMR_SUCCESS) m->ncfl++;
  switch (retval) {
    case SPGMR_SUCCESS: return 0;
    case SPGMR_RES_REDUCED: return (m->mnewt == 0) ? 0 : 1;
    case SPGMR_CONV_FAIL:
    case SPGMR_QRFACT_FAIL:
    case SPGMR_ATIMES_FAIL_REC: return 1;
    default: return -1;
  }
}

// ---------------------------------------------------------------------------
// Newton iteration (no linear-solver setup: PREC_NONE has none)
// ---------------------------------------------------------------------------
int newton_iteration(Mem *m) {
  int m_it = 0;
  double del = ZERO, delp = ZERO;
  m->mnewt = 0;
  for (;;) {
    NVLinearSum(m->rl1, m->zn[1], ONE, m->acor, m->tempv);
    NVLinearSum(m->gamma, m->ftemp, -ONE, m->tempv, m->tempv);
    N_Vector b = m->tempv;
    const int retval = lsolve(m, b, m->ewt, m->y, m->ftemp);
    m->nni++;
    if (retval < 0) return PIHM_BDF_LSOLVE_FAIL;
    if (retval > 0) return CONV_FAIL;
    del = NVWrms(b, m->ewt);
    NVLinearSum(ONE, m->acor, ONE, b, m->acor);
    NVLinearSum(ONE, m->zn[0], ONE, m->acor, m->y);
    if (m_it > 0) m->crate = sun_max(CRDOWN * m->crate, del / delp);
    const double dcon = del * sun_min(ONE, m->crate) / m->tq[4];
    if (dcon <= ONE) {
      m->acnrm = (m_it == 0) ? del : NVWrms(m->acor, m->ewt);
      return PIHM_BDF_SUCCESS;
    }
    m->mnewt = ++m_it;
    if ((m_it == m->maxcor) || ((m_it >= 2) && (del > RDIV * delp))) return CONV_FAIL;
    delp = del;
    const int rv = m->f(m->tn, m->y, m->ftemp, m->user_data);
    m->nfe++;
    if (rv < 0) return PIHM_BDF_RHSFUNC_FAIL;
    if (rv > 0) return RHSFUNC_RECVR;
  }
}

int nls_newton(Mem *m, int nflag) {
  (void)nflag;
  m->crate = ONE;  // no setup routine
  const int retval = m->f(m->tn, m->zn[0], m->ftemp, m->user_data);
  m->nfe++;
  if (retval < 0) return PIHM_BDF_RHSFUNC_FAIL;
  if (retval > 0) return RHSFUNC_RECVR;
  NVConst(ZERO, m->acor);
  NVScale(ONE, m->zn[0], m->y);
  return newton_iteration(m);
}

void restore(Mem *m, double saved_t) {
  m->tn = saved_t;
  for (int k = 1; k <= m->q; k++)
    for (int j = m->q; j >= k; j--) NVLinearSum(ONE, m->zn[j - 1], -ONE, m->zn[j], m->zn[j - 1]);
}

int handle_nflag(Mem *m, int *nflagPtr, double saved_t, int *ncfPtr) {
  const int nflag = *nflagPtr;
  if (nflag == PIHM_BDF_SUCCESS) return DO_ERROR_TEST;
  m->ncfn++;
  restore(m, saved_t);
  if (nflag == PIHM_BDF_LSOLVE_FAIL) return PIHM_BDF_LSOLVE_FAIL;
  if (nflag == PIHM_BDF_RHSFUNC_FAIL) return PIHM_BDF_RHSFUNC_FAIL;
  (*ncfPtr)++;
  m->etamax = ONE;
  if ((std::fabs(m->h) <= m->hmin * ONEPSM) || (*ncfPtr == m->maxncf)) {
    if (nflag == CONV_FAIL) return PIHM_BDF_CONV_FAILURE;
    if (nflag == RHSFUNC_RECVR) return PIHM_BDF_REPTD_RHSFUNC_ERR;
  }
  m->eta = sun_max(ETACF, m->hmin / std::fabs(m->h));
  *nflagPtr = PREV_CONV_FAIL;
  rescale(m);
  return PREDICT_AGAIN;
}

int do_error_test(Mem *m, int *nflagPtr, double saved_t, int *nefPtr, double *dsmPtr) {
  const double dsm = m->acnrm * m->tq[2];
  *dsmPtr = dsm;
  if (dsm <= ONE) return PIHM_BDF_SUCCESS;
  (*nefPtr)++;
  m->netf++;
  *nflagPtr = PREV_ERR_FAIL;
  restore(m, saved_t);
  if ((std::fabs(m->h) <= m->hmin * ONEPSM) || (*nefPtr == m->maxnef)) return PIHM_BDF_ERR_FAILURE;
  m->etamax = ONE;
  if (*nefPtr <= MXNEF1) {
    m->eta = ONE / (sun_powr(BIAS2 * dsm, ONE / m->L) + ADDON);
    m->eta = sun_max(ETAMIN, sun_max(m->eta, m->hmin / std::fabs(m->h)));
    if (*nefPtr >= SMALL_NEF) m->eta = sun_min(m->eta, ETAMXF);
    rescale(m);
    return TRY_AGAIN;
  }
  if (m->q > 1) {
    m->eta = sun_max(ETAMIN, m->hmin / std::fabs(m->h));
    adjust_order(m, -1);
    m->L = m->q;
    m->q--;
    m->qwait = m->L;
    rescale(m);
    return TRY_AGAIN;
  }
  m->eta = sun_max(ETAMIN, m->hmin / std::fabs(m->h));
  m->h *= m->eta;
  m->next_h = m->h;
  m->hscale = m->h;
  m->qwait = LONG_WAIT;
  m->nscon = 0;
  const int retval = m->f(m->tn, m->zn[0], m->tempv, m->user_data);
  m->nfe++;
  if (retval < 0) return PIHM_BDF_RHSFUNC_FAIL;
  if (retval > 0) return PIHM_BDF_UNREC_RHSFUNC_ERR;
  NVScale(m->h, m->tempv, m->zn[1]);
  return TRY_AGAIN;
}

void complete_step(Mem *m) {
  m->nst++;
  m->nscon++;
  m->hu = m->h;
  m->qu = m->q;
  for (int i = m->q; i >= 2; i--) m->tau[i] = m->tau[i - 1];
  if ((m->q == 1) && (m->nst > 1)) m->tau[2] = m->tau[1];
  m->tau[1] = m->h;
  for (int j = 0; j <= m->q; j++) NVLinearSum(m->l[j], m->acor, ONE, m->zn[j], m->zn[j]);
  m->qwait--;
  if ((m->qwait == 1) && (m->q != m->qmax)) {
    NVScale(ONE, m->acor, m->zn[m->qmax]);
    m->saved_tq5 = m->tq[5];
    m->indx_acor = m->qmax;
  }
}

void set_eta(Mem *m) {
  if (m->eta < THRESH) {
    m->eta = ONE;
    m->hprime = m->h;
  } else {
    m->eta = sun_min(m->eta, m->etamax);
    m->eta /= sun_max(ONE, std::fabs(m->h) * m->hmax_inv * m->eta);
    m->hprime = m->h * m->eta;
    if (m->qprime < m->q) m->nscon = 0;
  }
}

double compute_etaqm1(Mem *m) {
  m->etaqm1 = ZERO;
  if (m->q > 1) {
    const double ddn = NVWrms(m->zn[m->q], m->ewt) * m->tq[1];
    m->etaqm1 = ONE / (sun_powr(BIAS1 * ddn, ONE / m->q) + ADDON);
  }
  return m->etaqm1;
}

double compute_etaqp1(Mem *m) {
  m->etaqp1 = ZERO;
  if (m->q != m->qmax) {
    if (m->saved_tq5 == ZERO) return m->etaqp1;
    const double cquot = (m->tq[5] / m->saved_tq5) * sun_powi(m->h / m->tau[2], m->L);
    NVLinearSum(-cquot, m->zn[m->qmax], ONE, m->acor, m->tempv);
    const double dup = NVWrms(m->tempv, m->ewt) * m->tq[3];
    m->etaqp1 = ONE / (sun_powr(BIAS3 * dup, ONE / (m->L + 1)) + ADDON);
  }
  return m->etaqp1;
}

void choose_eta(Mem *m) {
  const double etam = sun_max(m->etaqm1, sun_max(m->etaq, m->etaqp1));
  if (etam < THRESH) {
    m->eta = ONE;
    m->qprime = m->q;
    return;
  }
  if (etam == m->etaq) {
    m->eta = m->etaq;
    m->qprime = m->q;
  } else if (etam == m->etaqm1) {
    m->eta = m->etaqm1;
    m->qprime = m->q - 1;
  } else {
    m->eta = m->etaqp1;
    m->qprime = m->q + 1;
    NVScale(ONE, m->acor, m->zn[m->qmax]);
  }
}

void prepare_next_step(Mem *m, double dsm) {
  if (m->etamax == ONE) {
    m->qwait = (m->qwait > 2) ? m->qwait : 2;
    m->qprime = m->q;
    m->hprime = m->h;
    m->eta = ONE;
    return;
  }
  m->etaq = ONE / (sun_powr(BIAS2 * dsm, ONE / m->L) + ADDON);
  if (m->qwait != 0) {
    m->eta = m->etaq;
    m->qprime = m->q;
    set_eta(m);
    return;
  }
  m->qwait = 2;
  m->etaqm1 = compute_etaqm1(m);
  m->etaqp1 = compute_etaqp1(m);
  choose_eta(m);
  set_eta(m);
}

// cvSLdet, cvode.c:3336-3600: stability-limit detection from the scaled
// derivative history ssdat.  Returns the detection flag (4..6 = violation).
int sl_det(Mem *m) {
  int kmin = 0, kflag = 0;
  double rat[5][4], rav[4], qkr[4], sigsq[4], smax[4], ssmax[4];
  double drr[4], rrc[4], sqmx[4], qjk[4][4], vrat[5], qc[6][4], qco[6][4];
  const double rrcut = 0.98, vrrtol = 1.0e-4, vrrt2 = 5.0e-4, sqtol = 1.0e-3, rrtol = 1.0e-2;
  double rr = ZERO, sqmin = ZERO;
  double (*ssdat)[4] = m->ssdat;
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
  const double qfac1 = FOURTH * (m->q * m->q - ONE);
  const double qfac2 = TWO / (m->q - ONE);
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

void bdf_stab(Mem *m) {
  if (m->q >= 3) {
    for (int k = 1; k <= 3; k++)
      for (int i = 5; i >= 2; i--) m->ssdat[i][k] = m->ssdat[i - 1][k];
    int factorial = 1;
    for (int i = 1; i <= m->q - 1; i++) factorial *= i;
    const double sq = factorial * m->q * (m->q + 1) * m->acnrm / sun_max(m->tq[5], TINY);
    const double sqm1 = factorial * m->q * NVWrms(m->zn[m->q], m->ewt);
    const double sqm2 = factorial * NVWrms(m->zn[m->q - 1], m->ewt);
    m->ssdat[1][1] = sqm2 * sqm2;
    m->ssdat[1][2] = sqm1 * sqm1;
    m->ssdat[1][3] = sq * sq;
  }
  if (m->qprime >= m->q) {
    if ((m->q >= 3) && (m->nscon >= m->q + 5)) {
      const int ldflag = sl_det(m);
      if (ldflag > 3) {
        m->qprime = m->q - 1;
        m->eta = m->etaqm1;
        m->eta = sun_min(m->eta, m->etamax);
        m->eta = m->eta / sun_max(ONE, std::fabs(m->h) * m->hmax_inv * m->eta);
        m->hprime = m->h * m->eta;
        m->nor = m->nor + 1;
      }
    }
  } else {
    m->nscon = 0;
  }
}

int step(Mem *m) {
  const double saved_t = m->tn;
  int ncf = 0, nef = 0;
  int nflag = FIRST_CALL;
  double dsm = 0;
  if ((m->nst > 0) && (m->hprime != m->h)) adjust_params(m);
  for (;;) {
    predict(m);
    set_coefficients(m);
    nflag = nls_newton(m, nflag);
    const int kflag = handle_nflag(m, &nflag, saved_t, &ncf);
    if (kflag == PREDICT_AGAIN) continue;
    if (kflag != DO_ERROR_TEST) return kflag;
    const int eflag = do_error_test(m, &nflag, saved_t, &nef, &dsm);
    if (eflag == TRY_AGAIN) continue;
    if (eflag != PIHM_BDF_SUCCESS) return eflag;
    break;
  }
  complete_step(m);
  prepare_next_step(m, dsm);
  if (m->sldeton) bdf_stab(m);
  m->etamax = (m->nst <= SMALL_NST) ? ETAMX2 : ETAMX3;
  NVScale(m->tq[2], m->acor, m->acor);
  return PIHM_BDF_SUCCESS;
}

int get_dky(Mem *m, double t, int k, N_Vector dky) {
  if (k < 0 || k > m->q) return PIHM_BDF_ILL_INPUT;
  double tfuzz = FUZZ_FACTOR * m->uround * (std::fabs(m->tn) + std::fabs(m->hu));
  if (m->hu < ZERO) tfuzz = -tfuzz;
  const double tp = m->tn - m->hu - tfuzz;
  const double tn1 = m->tn + tfuzz;
  if ((t - tp) * (t - tn1) > ZERO) return PIHM_BDF_ILL_INPUT;
  const double s = (t - m->tn) / m->h;
  for (int j = m->q; j >= k; j--) {
    double c = ONE;
    for (int i = j; i >= j - k + 1; i--) c *= i;
    if (j == m->q) NVScale(c, m->zn[m->q], dky);
    else NVLinearSum(c, m->zn[j], s, dky, dky);
  }
  if (k == 0) return PIHM_BDF_SUCCESS;
  NVScale(sun_powi(m->h, -k), dky, dky);
  return PIHM_BDF_SUCCESS;
}

int handle_failure(int flag) { return flag; }

}  // namespace

extern "C" {

pihm_bdf *pihm_bdf_create(void) { return new pihm_bdf(); }

int pihm_bdf_init(pihm_bdf *m, pihm_bdf_rhs_fn f, double t0, N_Vector y0) {
  if (!m || !f || !y0) return PIHM_BDF_ILL_INPUT;
  if (!m->malloc_done) {
    m->ewt = NVClone(y0);
    m->acor = NVClone(y0);
    m->tempv = NVClone(y0);
    m->ftemp = NVClone(y0);
    for (int j = 0; j <= m->qmax; j++) m->zn[j] = NVClone(y0);
    for (int i = 0; i <= m->maxl; i++) m->V[i] = NVClone(y0);
    m->xcor = NVClone(y0);
    m->vtemp = NVClone(y0);
    m->xsol = NVClone(y0);
    m->ytemp = NVClone(y0);
    for (int j = 0; j <= m->qmax; j++)
      if (!m->zn[j]) return PIHM_BDF_MEM_FAIL;
    if (!m->ewt || !m->acor || !m->tempv || !m->ftemp || !m->xcor || !m->vtemp || !m->xsol || !m->ytemp)
      return PIHM_BDF_MEM_FAIL;
    // sqrtN from a dot product of ones (CVSpgmr, cvode_spgmr.c:201-203)
    NVConst(ONE, m->ytemp);
    m->sqrtN = sun_sqrt(NVDot(m->ytemp, m->ytemp));
    m->malloc_done = true;
  }
  m->f = f;
  m->tn = t0;
  m->q = 1;
  m->L = 2;
  m->qwait = m->L;
  m->etamax = ETAMX1;
  m->qu = 0;
  m->hu = ZERO;
  m->tolsf = ONE;
  NVScale(ONE, y0, m->zn[0]);
  m->nst = m->nfe = m->ncfn = m->netf = m->nni = m->nhnil = m->nstlp = m->nscon = 0;
  m->nli = m->njtimes = m->nfes = m->ncfl = 0;
  m->h0u = ZERO;
  m->next_h = ZERO;
  m->next_q = 0;
  m->nor = 0;
  for (int i = 1; i <= 5; i++)
    for (int k = 1; k <= 3; k++) m->ssdat[i][k] = ZERO;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_reinit(pihm_bdf *m, double t0, N_Vector y0) {
  if (!m || !m->malloc_done) return PIHM_BDF_ILL_INPUT;
  return pihm_bdf_init(m, m->f, t0, y0);
}

int pihm_bdf_ss_tolerances(pihm_bdf *m, double reltol, double abstol) {
  if (!m || reltol < 0 || abstol < 0) return PIHM_BDF_ILL_INPUT;
  m->reltol = reltol;
  m->abstol = abstol;
  m->tol_set = true;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_set_user_data(pihm_bdf *m, void *user_data) {
  if (!m) return PIHM_BDF_ILL_INPUT;
  m->user_data = user_data;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_set_init_step(pihm_bdf *m, double hin) {
  if (!m) return PIHM_BDF_ILL_INPUT;
  m->hin = hin;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_set_max_step(pihm_bdf *m, double hmax) {
  if (!m || hmax < 0) return PIHM_BDF_ILL_INPUT;
  if (hmax == ZERO) {
    m->hmax_inv = ZERO;
    return PIHM_BDF_SUCCESS;
  }
  const double hmax_inv = ONE / hmax;
  if (hmax_inv * m->hmin > ONE) return PIHM_BDF_ILL_INPUT;
  m->hmax_inv = hmax_inv;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_set_max_num_steps(pihm_bdf *m, long mxsteps) {
  if (!m) return PIHM_BDF_ILL_INPUT;
  m->mxstep = (mxsteps == 0) ? 500 : mxsteps;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_set_stab_lim_det(pihm_bdf *m, int on) {
  if (!m) return PIHM_BDF_ILL_INPUT;
  m->sldeton = on != 0;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_set_stop_time(pihm_bdf *m, double tstop) {
  if (!m) return PIHM_BDF_ILL_INPUT;
  if (m->nst > 0 && (tstop - m->tn) * m->h < ZERO) return PIHM_BDF_ILL_INPUT;
  m->tstop = tstop;
  m->tstopset = true;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_solve(pihm_bdf *m, double tout, N_Vector yout, double *tret) {
  if (!m || !m->malloc_done || !yout || !tret) return PIHM_BDF_ILL_INPUT;
  if (!m->tol_set) return PIHM_BDF_ILL_INPUT;
  m->y = yout;
  m->toutc = tout;
  int istate = PIHM_BDF_SUCCESS;
  if (m->nst == 0) {
    m->tretlast = *tret = m->tn;
    if (ewt_set(m, m->zn[0], m->ewt) != 0) return PIHM_BDF_ILL_INPUT;
    const int retval = m->f(m->tn, m->zn[0], m->zn[1], m->user_data);
    m->nfe++;
    if (retval < 0) return PIHM_BDF_RHSFUNC_FAIL;
    if (retval > 0) return PIHM_BDF_FIRST_RHSFUNC_ERR;
    if (m->tstopset && (m->tstop - m->tn) * (tout - m->tn) <= ZERO) return PIHM_BDF_ILL_INPUT;
    m->h = m->hin;
    if (m->h != ZERO && (tout - m->tn) * m->h < ZERO) return PIHM_BDF_ILL_INPUT;
    if (m->h == ZERO) {
      double tout_hin = tout;
      if (m->tstopset && (tout - m->tn) * (tout - m->tstop) > ZERO) tout_hin = m->tstop;
      const int hflag = hin_estimate(m, tout_hin);
      if (hflag != PIHM_BDF_SUCCESS) return handle_failure(hflag);
    }
    const double rh = std::fabs(m->h) * m->hmax_inv;
    if (rh > ONE) m->h /= rh;
    if (std::fabs(m->h) < m->hmin) m->h *= m->hmin / std::fabs(m->h);
    if (m->tstopset) {
      if ((m->tn + m->h - m->tstop) * m->h > ZERO) m->h = (m->tstop - m->tn) * (ONE - FOUR * m->uround);
    }
    m->hscale = m->h;
    m->h0u = m->h;
    m->hprime = m->h;
    NVScale(m->h, m->zn[1], m->zn[1]);
  }
  if (m->nst > 0) {
    double troundoff = FUZZ_FACTOR * m->uround * (std::fabs(m->tn) + std::fabs(m->h));
    if ((m->tn - tout) * m->h >= ZERO) {
      m->tretlast = *tret = tout;
      if (get_dky(m, tout, 0, yout) != PIHM_BDF_SUCCESS) return PIHM_BDF_ILL_INPUT;
      return PIHM_BDF_SUCCESS;
    }
    if (m->tstopset) {
      if (std::fabs(m->tn - m->tstop) <= troundoff) {
        if (get_dky(m, m->tstop, 0, yout) != PIHM_BDF_SUCCESS) return PIHM_BDF_ILL_INPUT;
        m->tretlast = *tret = m->tstop;
        m->tstopset = false;
        return PIHM_BDF_TSTOP_RETURN;
      }
      if ((m->tn + m->hprime - m->tstop) * m->h > ZERO) {
        m->hprime = (m->tstop - m->tn) * (ONE - FOUR * m->uround);
        m->eta = m->hprime / m->h;
      }
    }
  }
  long nstloc = 0;
  for (;;) {
    m->next_h = m->h;
    m->next_q = m->q;
    if (m->nst > 0) {
      if (ewt_set(m, m->zn[0], m->ewt) != 0) {
        istate = PIHM_BDF_ILL_INPUT;
        m->tretlast = *tret = m->tn;
        NVScale(ONE, m->zn[0], yout);
        break;
      }
    }
    if ((m->mxstep > 0) && (nstloc >= m->mxstep)) {
      istate = PIHM_BDF_TOO_MUCH_WORK;
      m->tretlast = *tret = m->tn;
      NVScale(ONE, m->zn[0], yout);
      break;
    }
    const double nrm = NVWrms(m->zn[0], m->ewt);
    m->tolsf = m->uround * nrm;
    if (m->tolsf > ONE) {
      istate = PIHM_BDF_TOO_MUCH_ACC;
      m->tretlast = *tret = m->tn;
      NVScale(ONE, m->zn[0], yout);
      m->tolsf *= TWO;
      break;
    } else {
      m->tolsf = ONE;
    }
    if (m->tn + m->h == m->tn) m->nhnil++;
    const int kflag = step(m);
    if (kflag != PIHM_BDF_SUCCESS) {
      istate = handle_failure(kflag);
      m->tretlast = *tret = m->tn;
      NVScale(ONE, m->zn[0], yout);
      break;
    }
    nstloc++;
    if ((m->tn - tout) * m->h >= ZERO) {
      istate = PIHM_BDF_SUCCESS;
      m->tretlast = *tret = tout;
      (void)get_dky(m, tout, 0, yout);
      m->next_q = m->qprime;
      m->next_h = m->hprime;
      break;
    }
    if (m->tstopset) {
      const double troundoff = FUZZ_FACTOR * m->uround * (std::fabs(m->tn) + std::fabs(m->h));
      if (std::fabs(m->tn - m->tstop) <= troundoff) {
        (void)get_dky(m, m->tstop, 0, yout);
        m->tretlast = *tret = m->tstop;
        m->tstopset = false;
        istate = PIHM_BDF_TSTOP_RETURN;
        break;
      }
      if ((m->tn + m->hprime - m->tstop) * m->h > ZERO) {
        m->hprime = (m->tstop - m->tn) * (ONE - FOUR * m->uround);
        m->eta = m->hprime / m->h;
      }
    }
  }
  return istate;
}

int pihm_bdf_get_stats(const pihm_bdf *m, pihm_bdf_stats *s) {
  if (!m || !s) return PIHM_BDF_ILL_INPUT;
  s->nst = m->nst;
  s->nfe = m->nfe;
  s->nni = m->nni;
  s->ncfn = m->ncfn;
  s->netf = m->netf;
  s->nli = m->nli;
  s->nfes = m->nfes;
  s->njtimes = m->njtimes;
  s->ncfl = m->ncfl;
  s->nor = m->nor;
  s->qlast = m->qu;
  s->qcur = m->next_q;
  s->hlast = m->hu;
  s->hcur = m->next_h;
  s->tcur = m->tn;
  return PIHM_BDF_SUCCESS;
}

void pihm_bdf_free(pihm_bdf *m) {
  if (!m) return;
  if (m->malloc_done) {
    NVDestroy(m->ewt);
    NVDestroy(m->acor);
    NVDestroy(m->tempv);
    NVDestroy(m->ftemp);
    for (int j = 0; j <= m->qmax; j++) NVDestroy(m->zn[j]);
    for (int i = 0; i <= m->maxl; i++) NVDestroy(m->V[i]);
    NVDestroy(m->xcor);
    NVDestroy(m->vtemp);
    NVDestroy(m->xsol);
    NVDestroy(m->ytemp);
  }
  delete m;
}

}  // extern "C"
