// The pihm_bdf C ABI (pihm_bdf.h): the BDF/Newton/GMRES integrator of
// bdf_core.h over any SUNDIALS 2.7 N_Vector, driven through the vector's own
// operations table -- the device N_Vector of this library on the GPU, a host
// serial vector in the tests -- with the right-hand side called through a
// CVRhsFn.  Every operation completes when it is issued, so each call into
// the integrator runs its coroutines straight through; the sequence of
// vector operations and right-hand-side evaluations is the one CVODE makes
// (and therefore so is the river-edge flux the PIHM right-hand side carries
// from one evaluation to the next).
#include "bdf_core.h"
#include "pihm_bdf.h"

namespace {

struct NVectorOps {
  using Vec = N_Vector;
  pihm_bdf_rhs_fn f = nullptr;
  void *user_data = nullptr;

  Vec clone(Vec w) { return w->ops->nvclone(w); }
  void destroy(Vec v) {
    if (v) v->ops->nvdestroy(v);
  }
  bool valid(Vec v) const { return v != nullptr; }

  pihm::ReadyVoid linear_sum(double a, Vec x, double b, Vec y, Vec z) {
    z->ops->nvlinearsum(a, x, b, y, z);
    return {};
  }
  pihm::ReadyVoid const_(double c, Vec z) {
    z->ops->nvconst(c, z);
    return {};
  }
  pihm::ReadyVoid scale(double c, Vec x, Vec z) {
    z->ops->nvscale(c, x, z);
    return {};
  }
  pihm::ReadyVoid abs_(Vec x, Vec z) {
    z->ops->nvabs(x, z);
    return {};
  }
  pihm::ReadyVoid inv(Vec x, Vec z) {
    z->ops->nvinv(x, z);
    return {};
  }
  pihm::ReadyVoid div(Vec x, Vec y, Vec z) {
    z->ops->nvdiv(x, y, z);
    return {};
  }
  pihm::ReadyVoid prod(Vec x, Vec y, Vec z) {
    z->ops->nvprod(x, y, z);
    return {};
  }
  pihm::ReadyVoid addconst(Vec x, double b, Vec z) {
    z->ops->nvaddconst(x, b, z);
    return {};
  }
  pihm::Ready<double> dot(Vec x, Vec y) { return {x->ops->nvdotprod(x, y)}; }
  pihm::Ready<double> maxnorm(Vec x) { return {x->ops->nvmaxnorm(x)}; }
  pihm::Ready<double> wrms(Vec x, Vec w) { return {x->ops->nvwrmsnorm(x, w)}; }
  pihm::Ready<double> vmin(Vec x) { return {x->ops->nvmin(x)}; }
  pihm::Ready<int> rhs(double t, Vec y, Vec ydot) { return {f(t, y, ydot, user_data)}; }
};

}  // namespace

struct pihm_bdf : pihm::bdf::BdfCore<NVectorOps> {};

extern "C" {

pihm_bdf *pihm_bdf_create(void) { return new pihm_bdf(); }

int pihm_bdf_init(pihm_bdf *m, pihm_bdf_rhs_fn f, double t0, N_Vector y0) {
  if (!m || !f || !y0) return PIHM_BDF_ILL_INPUT;
  m->ops.f = f;
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
