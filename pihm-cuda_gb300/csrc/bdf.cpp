// The pihm_bdf C ABI (pihm_bdf.h): the BDF/Newton/GMRES integrator of
// bdf_core.h over any SUNDIALS 2.7 N_Vector, driven through the vector's own
// operations table -- the device N_Vector of this library on the GPU, a host
// serial vector in the tests -- with the right-hand side called through a
// CVRhsFn.  Every operation completes when it is issued, so each call into
// the integrator runs its coroutines straight through; the sequence of
// vector operations and right-hand-side evaluations is the one CVODE makes
// (and therefore so is the river-edge flux the PIHM right-hand side carries
// from one evaluation to the next).
#include <chrono>

#include "bdf_core.h"
#include "pihm_bdf.h"
#include "pihm_gpu.h"
#include "pihm_nvector.h"

namespace {

static_assert((int)pihm::bdf::COEF_HOST == PIHM_NV_COEF_HOST && (int)pihm::bdf::COEF_NEG == PIHM_NV_COEF_NEG &&
                  (int)pihm::bdf::COEF_INV == PIHM_NV_COEF_INV &&
                  (int)pihm::bdf::COEF_INV_INV == PIHM_NV_COEF_INV_INV &&
                  (int)pihm::bdf::COEF_NEG_INV_INV == PIHM_NV_COEF_NEG_INV_INV,
              "coefficient kinds");

// Host time spent inside the operations (pihm_bdf_set_op_timing): issuing
// element-wise operations, reductions until their value is back, right-hand
// side calls until they return, slot read-backs.
struct OpTimer {
  bool on = false;
  double ms[PIHM_BDF_OPT_COUNT] = {0};
  long long n[PIHM_BDF_OPT_COUNT] = {0};
};

struct Scope {
  OpTimer &t;
  int k;
  std::chrono::steady_clock::time_point a;
  Scope(OpTimer &t_, int k_) : t(t_), k(k_) {
    if (t.on) a = std::chrono::steady_clock::now();
  }
  ~Scope() {
    if (!t.on) return;
    t.ms[k] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
    t.n[k]++;
  }
};

struct NVectorOps {
  using Vec = N_Vector;
  pihm_bdf_rhs_fn f = nullptr;
  void *user_data = nullptr;
  OpTimer timer;
  // GMRES scalars kept with the vectors (pihm_bdf_set_deferred_scalars):
  // -1 automatic (device vectors of this library with its own right-hand
  // side), 0 off, 1 on for any vectors
  int deferred_setting = -1;
  // decided at the first GMRES iteration of a solve: 0 off, 1 host slots
  // (operations through the table, values kept here), 2 device slots
  int mode = -1;
  bool rhs_deferrable = false;  // the right-hand side's status joins the slot read-back
  bool rhs_pending = false;
  Vec slot_vec = nullptr;
  double host_slots[PIHM_NV_SLOTS] = {0};

  Vec clone(Vec w) { return w->ops->nvclone(w); }
  void destroy(Vec v) {
    if (v) v->ops->nvdestroy(v);
  }
  bool valid(Vec v) const { return v != nullptr; }

  pihm::ReadyVoid linear_sum(double a, Vec x, double b, Vec y, Vec z) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    z->ops->nvlinearsum(a, x, b, y, z);
    return {};
  }
  pihm::ReadyVoid const_(double c, Vec z) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    z->ops->nvconst(c, z);
    return {};
  }
  pihm::ReadyVoid scale(double c, Vec x, Vec z) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    z->ops->nvscale(c, x, z);
    return {};
  }
  pihm::ReadyVoid abs_(Vec x, Vec z) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    z->ops->nvabs(x, z);
    return {};
  }
  pihm::ReadyVoid inv(Vec x, Vec z) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    z->ops->nvinv(x, z);
    return {};
  }
  pihm::ReadyVoid div(Vec x, Vec y, Vec z) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    z->ops->nvdiv(x, y, z);
    return {};
  }
  pihm::ReadyVoid prod(Vec x, Vec y, Vec z) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    z->ops->nvprod(x, y, z);
    return {};
  }
  pihm::ReadyVoid addconst(Vec x, double b, Vec z) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    z->ops->nvaddconst(x, b, z);
    return {};
  }
  pihm::Ready<double> dot(Vec x, Vec y) {
    Scope sc(timer, PIHM_BDF_OPT_REDUCTION);
    return {x->ops->nvdotprod(x, y)};
  }
  pihm::Ready<double> maxnorm(Vec x) {
    Scope sc(timer, PIHM_BDF_OPT_REDUCTION);
    return {x->ops->nvmaxnorm(x)};
  }
  pihm::Ready<double> wrms(Vec x, Vec w) {
    Scope sc(timer, PIHM_BDF_OPT_REDUCTION);
    return {x->ops->nvwrmsnorm(x, w)};
  }
  pihm::Ready<double> vmin(Vec x) {
    Scope sc(timer, PIHM_BDF_OPT_REDUCTION);
    return {x->ops->nvmin(x)};
  }
  pihm::Ready<int> rhs(double t, Vec y, Vec ydot) {
    Scope sc(timer, PIHM_BDF_OPT_RHS);
    return {f(t, y, ydot, user_data)};
  }

  // ---- device-resident GMRES scalars (bdf_core.h atimes_gs_deferred) ----
  static bool is_device(Vec v) { return v && v->ops && v->ops->nvgetvectorid == N_VGetVectorID_PihmGpu; }

  bool deferred_scalars(Vec v) {
    if (mode < 0) {
      const bool own_rhs = f == pihm_gpu_ode && user_data &&
                           N_VGetStream_PihmGpu(v) == pihm_gpu_get_stream((const pihm_gpu_ctx *)user_data);
      if (deferred_setting == 0 || (deferred_setting < 0 && !(is_device(v) && own_rhs))) mode = 0;
      else mode = is_device(v) ? 2 : 1;
      rhs_deferrable = mode == 2 && own_rhs;
      slot_vec = v;
    }
    return mode > 0;
  }
  double host_coef_value(const pihm::bdf::Coef &c) const {
    switch (c.kind) {
      case pihm::bdf::COEF_NEG: return -host_slots[c.slot];
      case pihm::bdf::COEF_INV: return 1.0 / host_slots[c.slot];
      case pihm::bdf::COEF_INV_INV: return 1.0 / (1.0 / host_slots[c.slot]);
      case pihm::bdf::COEF_NEG_INV_INV: return -(1.0 / (1.0 / host_slots[c.slot]));
      default: return c.value;
    }
  }
  pihm::ReadyVoid dot_slot(Vec x, Vec y, int slot) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    if (mode == 2) N_VDotProdSlot_PihmGpu(x, y, slot);
    else host_slots[slot] = x->ops->nvdotprod(x, y);
    return {};
  }
  pihm::ReadyVoid wrms_slot(Vec x, Vec w, int slot) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    if (mode == 2) N_VWrmsNormSlot_PihmGpu(x, w, slot);
    else host_slots[slot] = x->ops->nvwrmsnorm(x, w);
    return {};
  }
  pihm::ReadyVoid linear_sum_coef(pihm::bdf::Coef a, Vec x, pihm::bdf::Coef b, Vec y, Vec z) {
    Scope sc(timer, PIHM_BDF_OPT_ELEMENTWISE);
    if (mode == 2) {
      const pihm_nv_coef ca = {a.kind, a.slot, a.value}, cb = {b.kind, b.slot, b.value};
      N_VLinearSumCoef_PihmGpu(&ca, x, &cb, y, z);
    } else {
      z->ops->nvlinearsum(host_coef_value(a), x, host_coef_value(b), y, z);
    }
    return {};
  }
  pihm::Ready<int> rhs_deferred(double t, Vec y, Vec ydot) {
    Scope sc(timer, PIHM_BDF_OPT_RHS);
    if (!rhs_deferrable) return {f(t, y, ydot, user_data)};
    const int rc = pihm_gpu_ode_launch(t, y, ydot, user_data);
    rhs_pending = rc == 0;
    return {rc};
  }
  // slots 0..count-1 to out; -1 when a deferred right-hand side produced a NaN
  pihm::Ready<int> fetch_slots(int count, double *out) {
    Scope sc(timer, PIHM_BDF_OPT_REDUCTION);
    if (mode != 2) {
      for (int i = 0; i < count; i++) out[i] = host_slots[i];
      return {0};
    }
    unsigned int word = 0;
    const bool pending = rhs_pending;
    rhs_pending = false;
    const unsigned int *dev_word = pending ? pihm_gpu_error_word((pihm_gpu_ctx *)user_data) : nullptr;
    if (N_VFetchSlots_PihmGpu(slot_vec, count, out, dev_word, &word) != 0) return {-1};
    if (word != 0) {
      (void)pihm_gpu_status((pihm_gpu_ctx *)user_data);  // reads and clears the word
      return {-1};
    }
    return {0};
  }
};

}  // namespace

struct pihm_bdf : pihm::bdf::BdfCore<NVectorOps> {};

extern "C" {

pihm_bdf *pihm_bdf_create(void) { return new pihm_bdf(); }

int pihm_bdf_init(pihm_bdf *m, pihm_bdf_rhs_fn f, double t0, N_Vector y0) {
  if (!m || !f || !y0) return PIHM_BDF_ILL_INPUT;
  m->ops.f = f;
  m->ops.mode = -1;
  return pihm::run_sync(m->init(t0, y0));
}

int pihm_bdf_reinit(pihm_bdf *m, double t0, N_Vector y0) {
  if (!m || !m->alloc_done || !y0) return PIHM_BDF_ILL_INPUT;
  return pihm::run_sync(m->init(t0, y0));
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
  m->ops.user_data = user_data;
  m->ops.mode = -1;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_set_op_timing(pihm_bdf *m, int on) {
  if (!m) return PIHM_BDF_ILL_INPUT;
  m->ops.timer = OpTimer();
  m->ops.timer.on = on != 0;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_get_op_times(const pihm_bdf *m, double *ms, int64_t *calls) {
  if (!m || !ms) return PIHM_BDF_ILL_INPUT;
  for (int k = 0; k < PIHM_BDF_OPT_COUNT; k++) {
    ms[k] = m->ops.timer.ms[k];
    if (calls) calls[k] = m->ops.timer.n[k];
  }
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_get_deferred_scalars(const pihm_bdf *m) {
  if (!m) return PIHM_BDF_ILL_INPUT;
  return m->ops.mode == 2 && m->ops.rhs_deferrable ? 3 : m->ops.mode;
}

int pihm_bdf_set_deferred_scalars(pihm_bdf *m, int setting) {
  if (!m || setting < -1 || setting > 1) return PIHM_BDF_ILL_INPUT;
  m->ops.deferred_setting = setting;
  m->ops.mode = -1;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_set_init_step(pihm_bdf *m, double hin) {
  if (!m) return PIHM_BDF_ILL_INPUT;
  m->hin = hin;
  return PIHM_BDF_SUCCESS;
}

int pihm_bdf_set_max_step(pihm_bdf *m, double hmax) {
  if (!m) return PIHM_BDF_ILL_INPUT;
  return m->set_max_step(hmax);
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
  return m->set_stop_time(tstop);
}

int pihm_bdf_solve(pihm_bdf *m, double tout, N_Vector yout, double *tret) {
  if (!m || !yout || !tret) return PIHM_BDF_ILL_INPUT;
  return pihm::run_sync(m->solve(tout, yout, tret));
}

int pihm_bdf_get_stats(const pihm_bdf *m, pihm_bdf_stats *s) {
  if (!m || !s) return PIHM_BDF_ILL_INPUT;
  const pihm::bdf::Stats st = m->stats();
  s->nst = st.nst;
  s->nfe = st.nfe;
  s->nni = st.nni;
  s->ncfn = st.ncfn;
  s->netf = st.netf;
  s->nli = st.nli;
  s->nfes = st.nfes;
  s->njtimes = st.njtimes;
  s->ncfl = st.ncfl;
  s->nor = st.nor;
  s->qlast = st.qlast;
  s->qcur = st.qcur;
  s->hlast = st.hlast;
  s->hcur = st.hcur;
  s->tcur = st.tcur;
  return PIHM_BDF_SUCCESS;
}

void pihm_bdf_free(pihm_bdf *m) {
  if (!m) return;
  m->release();
  delete m;
}

}  // extern "C"
