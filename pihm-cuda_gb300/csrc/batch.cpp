// The batch engine (include/pihm_batch.h).
//
// Every watershed runs the reference's model-step loop as a coroutine over the
// integrator of bdf_core.h.  Its vector operations are not executed when they
// are issued: element-wise ones are queued into the watershed's program for
// the current round, and a reduction or a right-hand-side evaluation ends the
// program and suspends the coroutine.  A round uploads all programs, runs them
// in one launch of the program kernel (batch_kernels.cu), evaluates the right
// hand side once over the arena for the watersheds that asked for it, reads
// back every reduction result and error word in one copy, and resumes the
// coroutines.  Watersheds therefore proceed independently -- each with its own
// step size, order, Newton and Krylov iterations, model step and stopping
// time -- while sharing every launch.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <coroutine>
#include <cstring>
#include <map>
#include <memory>
#include <thread>
#include <vector>

#include "batch_engine.h"
#include "pihm_deck.h"

using namespace pihm;
using namespace pihm::batch;
using pihm_nv::EwCall;

namespace pihm {
namespace batch {

bool BatchOps::Ew::await_ready() const noexcept { return (int)s->prog.size() < kMaxProgOps; }
void BatchOps::Ew::await_suspend(std::coroutine_handle<> h) const noexcept { s->waiting = h; }
void BatchOps::Red::await_suspend(std::coroutine_handle<> h) const noexcept { s->waiting = h; }
double BatchOps::Red::await_resume() const noexcept { return s->red_value; }
void BatchOps::Rhs::await_suspend(std::coroutine_handle<> h) const noexcept { s->waiting = h; }
int BatchOps::Rhs::await_resume() const noexcept { return s->rhs_rc; }

BatchOps::Ew BatchOps::push(int code, double a, double b, int x, int y, int z, double c, int i0, int i1) {
  Op o;
  std::memset(&o, 0, sizeof(o));
  o.code = (uint8_t)code;
  o.x = (uint8_t)x;
  o.y = (uint8_t)y;
  o.z = (uint8_t)z;
  o.i0 = i0;
  o.i1 = i1;
  o.a = a;
  o.b = b;
  o.c = c;
  s->prog.push_back(o);
  return Ew{s};
}

BatchOps::Red BatchOps::reduce(int red, int x, int y, bool wrms) {
  s->red = red;
  s->rx = (uint8_t)x;
  s->ry = (uint8_t)y;
  s->red_wrms = wrms;
  return Red{s};
}

BatchOps::Rhs BatchOps::rhs(double, int y, int ydot) {
  push(OP_STAGE_IN, 0.0, 0.0, y, y, y);
  s->rhs_req = true;
  s->rhs_out = (uint8_t)ydot;
  return Rhs{s};
}

// The reference's model-step loop for one watershed (src/pihm.c:7-187 with
// SolveCVode and AdjCVodeMaxStep, src/ode.c:555-661), as the single-watershed
// driver runs it: forcing, stop time, solve, post-step update, maximum-step
// adaptation, outlet record.
Task<int> model_run(Sys *s) {
  bdf::BdfCore<BatchOps> &c = s->core;
  BatchOps &o = c.ops;
  const pihm_step_control &ct = s->ctrl;
  const int Y = 0;
  co_await o.post_step(Y);  // ws0 <- y0
  int rc = co_await c.init(0.0, Y);
  if (rc != bdf::SUCCESS) co_return rc;
  c.reltol = ct.reltol;
  c.abstol = ct.abstol;
  c.tol_set = true;
  c.hin = ct.initstep;
  c.sldeton = true;
  double maxstep = ct.stepsize;
  if ((rc = c.set_max_step(maxstep)) != bdf::SUCCESS) co_return rc;
  c.mxstep = ct.mxstep ? ct.mxstep : (long)(ct.stepsize * 10.0);
  long nst0 = 0, ncfn0 = 0, nni0 = 0;
  double tret = 0.0;
  for (int k = 0; k < s->nsteps; k++) {
    // the step's forcing: the uniform series, or the deck's boundary values
    // and land-surface step, which the round that runs this program applies
    if (!s->land.alloc && !s->noah.alloc) co_await o.forcing(s->pcp[k], s->edir[k], s->ett[k]);
    if (s->has_bc || s->land.alloc || s->noah.alloc) s->pending_k = k;
    const double tout = (double)(k + 1) * ct.stepsize;
    if ((rc = c.set_stop_time(tout)) != bdf::SUCCESS) co_return rc;
    rc = co_await c.solve(tout, Y, &tret);
    if (rc < 0) co_return rc;
    co_await o.post_step(Y);
    if (s->noah.alloc) s->pending_post = true;  // Summary's _NOAH_ part and NoahHydrol
    // AdjCVodeMaxStep, src/ode.c:601-661
    const double nsteps_d = (double)(c.nst - nst0);
    const double nfails = (double)(c.ncfn - ncfn0) / nsteps_d;
    const double niters = (double)(c.nni - nni0) / nsteps_d;
    if (nfails > ct.nncfn || niters >= ct.nnimax) maxstep /= ct.decr;
    if (nfails == 0.0 && niters <= ct.nnimin) maxstep *= ct.incr;
    maxstep = maxstep < ct.stepsize ? maxstep : ct.stepsize;
    maxstep = maxstep > ct.stmin ? maxstep : ct.stmin;
    if ((rc = c.set_max_step(maxstep)) != bdf::SUCCESS) co_return rc;
    nst0 = c.nst;
    ncfn0 = c.ncfn;
    nni0 = c.nni;
    if (s->outlet >= 0) co_await o.record(k, s->outlet);
    s->steps_done = k + 1;
  }
  co_return bdf::SUCCESS;
}

// Counting mode of pihm_batch_create (pihm_batch_arena_bytes): allocations
// add their size here instead of allocating.
thread_local int64_t *t_count_bytes = nullptr;

template <class T>
T *dalloc(size_t n, std::vector<void *> &owned) {
  void *p = nullptr;
  if (n == 0) n = 1;
  if (t_count_bytes) {
    *t_count_bytes += (int64_t)((sizeof(T) * n + 511) & ~size_t(511));  // the allocator's granularity
    return (T *)(uintptr_t)4096;
  }
  if (cudaMalloc(&p, sizeof(T) * n) != cudaSuccess) return nullptr;
  owned.push_back(p);
  return (T *)p;
}

}  // namespace batch
}  // namespace pihm


namespace {

template <class T>
int h2d(T *dst, const T *src, size_t n, cudaStream_t st) {
  if (n == 0) return 0;
  return cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, st) == cudaSuccess ? 0 : -1;
}

// A watershed's uploads: on a device that can access pageable host memory,
// descriptors for one gather kernel that reads the host arrays directly
// (one launch instead of about a hundred staged copies); else staged copies.
// Either way every source must stay valid until flush() has synchronised.
struct Uploader {
  bool direct;
  cudaStream_t st;
  std::vector<CopyDesc> desc;
  uint64_t max_bytes = 0;
  int rc = 0;
  template <class T>
  void operator()(T *dst, const T *src, size_t n) {
    if (n == 0) return;
    if (direct) {
      desc.push_back({(const void *)src, (void *)dst, (uint64_t)(sizeof(T) * n)});
      max_bytes = std::max<uint64_t>(max_bytes, sizeof(T) * n);
    } else {
      rc |= h2d(dst, src, n, st);
    }
  }
  int flush() {
    if (direct && !desc.empty() && launch_gather_host(desc.data(), (int)desc.size(), max_bytes, st) != cudaSuccess)
      rc = -1;
    if (cudaStreamSynchronize(st) != cudaSuccess) rc = -1;
    return rc;
  }
};

// Translate a watershed image's indices to its arena ranges and upload it.
int place(pihm_batch *B, Sys *s, const Prepared &job) {
  const SystemImage &im = job.im;
  DevMesh &m = B->A.m;
  cudaStream_t st = B->st;
  Uploader up{B->host_pageable != 0, st, {}};
  const int ne = im.ne, nr = im.nr;
  const int64_t NE = B->ne_cap, NR = B->nr_cap;
  const int64_t eo = s->eoff, ro = s->roff, edo = s->edoff, bo = s->boff, uo = s->upoff;
  int rc = 0;
  for (int k = 0; k < EP_COUNT; k++) up((double *)(m.*kElemMember[k]) + eo, im.el[k].data(), ne);
  for (int k = 0; k < XP_COUNT; k++)
    for (int j = 0; j < 3; j++)
      up((double *)(m.*kEdgeMember[k]) + j * NE + eo, im.ed[k].data() + (size_t)j * ne, ne);
  std::vector<int32_t> t(3 * (size_t)ne);
  for (size_t q = 0; q < t.size(); q++) {
    const int32_t v = im.nb[q];
    t[q] = v >= 0 ? (int32_t)(v + eo) : (v == kBoundary ? v : (int32_t)(-1 - ((-1 - v) + ro)));
  }
  for (int j = 0; j < 3; j++) up((int32_t *)m.nb + j * NE + eo, t.data() + (size_t)j * ne, ne);
  std::vector<int32_t> t2(3 * (size_t)ne);
  for (size_t q = 0; q < t2.size(); q++) {
    const int32_t v = im.emap[q];
    t2[q] = v > 0 ? (int32_t)(v + edo) : (v < 0 ? (int32_t)(v - edo) : 0);
  }
  for (int j = 0; j < 3; j++) {
    up((int32_t *)m.emap + j * NE + eo, t2.data() + (size_t)j * ne, ne);
    up((int32_t *)m.bctype + j * NE + eo, im.bct.data() + (size_t)j * ne, ne);
  }
  std::vector<int32_t> ei(im.nedge), ek(im.nedge);
  for (int e = 0; e < im.nedge; e++) {
    ei[e] = (int32_t)(im.e_i[e] + eo);
    ek[e] = (int32_t)(im.e_k[e] + eo);
  }
  up((int32_t *)m.e_i + edo, ei.data(), im.nedge);
  up((int32_t *)m.e_k + edo, ek.data(), im.nedge);
  up((double *)m.e_invdist + edo, im.e_invdist.data(), im.nedge);
  up((double *)m.e_subk + edo, im.e_subk.data(), im.nedge);
  up((double *)m.e_ovlk + edo, im.e_ovlk.data(), im.nedge);
  std::vector<int32_t> bs(ne), be(im.nbank);
  for (int i = 0; i < ne; i++) bs[i] = im.bank_slot[i] >= 0 ? (int32_t)(im.bank_slot[i] + bo) : -1;
  for (int b = 0; b < im.nbank; b++) be[b] = (int32_t)(im.bank_elem[b] + eo);
  up((int32_t *)m.bank_slot + eo, bs.data(), ne);
  up((int32_t *)m.bank_elem + bo, be.data(), im.nbank);
  std::vector<int32_t> dn(nr), lf(nr), rt(nr), ub(nr), ue(nr), ui(im.up_idx.size());
  for (int r = 0; r < nr; r++) {
    dn[r] = im.down[r] > 0 ? (int32_t)(im.down[r] + ro) : im.down[r];
    lf[r] = (int32_t)(im.left[r] + eo);
    rt[r] = (int32_t)(im.right[r] + eo);
    ub[r] = (int32_t)(im.up_ptr[r] + uo);
    ue[r] = (int32_t)(im.up_ptr[r + 1] + uo);
  }
  for (size_t q = 0; q < ui.size(); q++) ui[q] = (int32_t)(im.up_idx[q] + ro);
  up((int32_t *)m.down + ro, dn.data(), nr);
  up((int32_t *)m.left + ro, lf.data(), nr);
  up((int32_t *)m.right + ro, rt.data(), nr);
  up((int32_t *)m.intrpl_ord + ro, im.ord.data(), nr);
  up((int32_t *)m.bctype_riv + ro, im.rbct.data(), nr);
  up((int32_t *)m.up_ptr + ro, ub.data(), nr);
  up((int32_t *)m.up_end + ro, ue.data(), nr);
  up((int32_t *)m.up_idx + uo, ui.data(), ui.size());
  for (int k = 0; k < RP_COUNT; k++) up((double *)(m.*kRiverMember[k]) + ro, im.rv[k].data(), nr);
  // boundary conditions (reference order in the job)
  std::vector<double> bc(3 * (size_t)ne, 0.0);
  if (!job.elem_bc.empty())
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < ne; i++) bc[(size_t)j * ne + i] = job.elem_bc[3 * (size_t)im.perm[i] + j];
  for (int j = 0; j < 3; j++) up((double *)m.elem_bc + j * NE + eo, bc.data() + (size_t)j * ne, ne);
  std::vector<double> rbc(nr, 0.0);
  if (!job.river_bc.empty()) std::copy(job.river_bc.begin(), job.river_bc.end(), rbc.begin());
  up((double *)m.river_bc + ro, rbc.data(), nr);
  // a fresh watershed carries no river-edge flux from an earlier evaluation
  for (int k = 0; k < NUM_RIVFLX; k++)
    if (nr && cudaMemsetAsync(m.rivflow + k * NR + ro, 0, sizeof(double) * nr, st) != cudaSuccess) rc = -1;
  for (int k = 0; k < 2; k++)
    if (nr && cudaMemsetAsync(m.carry_ovl + k * NR + ro, 0, sizeof(double) * nr, st) != cudaSuccess) rc = -1;
  // owner tables
  std::vector<int32_t> own(std::max<int64_t>({(int64_t)ne, (int64_t)nr, (int64_t)im.nedge, (int64_t)im.nbank, 1}),
                           s->slot);
  up((int32_t *)m.sys_elem + eo, own.data(), ne);
  up((int32_t *)m.sys_riv + ro, own.data(), nr);
  up((int32_t *)m.sys_edge + edo, own.data(), im.nedge);
  up((int32_t *)m.sys_bank + bo, own.data(), im.nbank);
  const double dt = job.ctrl.stepsize;
  up((double *)m.sys_dt + s->slot, &dt, 1);
  const double inv_dt = 1.0 / dt;
  up((double *)m.sys_inv_dt + s->slot, &inv_dt, 1);
  // initial state, internal order, into vector slot 0
  std::vector<double> y(s->neq);
  for (int p = 0; p < 3; p++)
    for (int i = 0; i < ne; i++) y[(size_t)p * ne + i] = job.y0[(size_t)p * ne + im.perm[i]];
  for (int64_t q = 3LL * ne; q < s->neq; q++) y[q] = job.y0[q];
  up(B->A.vec + s->soff, y.data(), s->neq);
  SysInfo info{};
  info.off = s->soff;
  info.neq = (int32_t)s->neq;
  info.ne = ne;
  info.nr = nr;
  info.eoff = (int32_t)eo;
  info.roff = (int32_t)ro;
  info.nblk = (int32_t)pihm_nv::red_grid_for(s->neq);
  info.rec_off = s->recoff;
  up(B->A.sysinfo + s->slot, &info, 1);
  rc |= up.flush();
  return rc ? PIHM_GPU_ERR_CUDA : PIHM_GPU_OK;
}

}  // namespace

namespace pihm {
namespace batch {

void free_ranges(pihm_batch *B, Sys *s) {
  DevMesh &m = B->A.m;
  if (s->noah.alloc) {
    cudaMemsetAsync(const_cast<int32_t *>(m.sys_noah) + s->slot, 0, sizeof(int32_t), B->st);
    if (--B->noah_resident == 0) m.noah = m.diag = 0;
    noah_release(s->noah);
  }
  // mark the items free so the masked kernels skip them whatever the slot's next owner
  if (s->ne) cudaMemsetAsync((int32_t *)m.sys_elem + s->eoff, 0xff, sizeof(int32_t) * s->ne, B->st);
  if (s->nr) cudaMemsetAsync((int32_t *)m.sys_riv + s->roff, 0xff, sizeof(int32_t) * s->nr, B->st);
  if (s->nedge) cudaMemsetAsync((int32_t *)m.sys_edge + s->edoff, 0xff, sizeof(int32_t) * s->nedge, B->st);
  if (s->nbank) cudaMemsetAsync((int32_t *)m.sys_bank + s->boff, 0xff, sizeof(int32_t) * s->nbank, B->st);
  cudaStreamSynchronize(B->st);
  B->ra_elem.release(s->eoff, s->ne);
  B->ra_riv.release(s->roff, s->nr);
  B->ra_edge.release(s->edoff, s->nedge);
  B->ra_bank.release(s->boff, s->nbank);
  B->ra_up.release(s->upoff, s->nup);
  B->ra_state.release(s->soff, s->neq);
  B->ra_rec.release(s->recoff, s->nrec);
  B->update_extents();
}

// Resume a watershed's coroutine and note how it stopped.
void resume(Sys *s) {
  std::coroutine_handle<> h = s->waiting;
  s->waiting = {};
  h.resume();
  if (s->task->done()) {
    s->solver_rc = s->task->result();
    s->state = (s->solver_rc < 0) ? S_FAILED : S_DONE;
  }
}


// Validate a job and build everything the arena needs from it on the host.
int prepare(const pihm_batch_job *job, int surf_mode, int riv_mode, int order, Prepared *p) {
  if (!job || !job->mesh || !job->y0 || !p || job->nsteps < 0) return PIHM_GPU_ERR_ARG;
  if (job->land && (!job->forcing || job->lsm_step <= 0 || job->land->nelem != job->mesh->nelem))
    return PIHM_GPU_ERR_ARG;
  if (job->noah && (job->land || !job->noah_state || !job->noah_forcing || job->noah_nforcing < 1 ||
                    !(job->noah_lsm_step > 0.0) || job->noah->nelem != job->mesh->nelem))
    return PIHM_GPU_ERR_ARG;
  if (job->nsteps > 0 && !job->land && !job->noah && (!job->pcpdrp || !job->edir || !job->ett))
    return PIHM_GPU_ERR_ARG;
  const pihm_step_control &c = job->ctrl;
  if (!(c.stepsize > 0.0) || c.reltol < 0 || c.abstol < 0 || !(c.decr > 0.0)) return PIHM_GPU_ERR_ARG;
  if (job->outlet >= job->mesh->nriver) return PIHM_GPU_ERR_ARG;
  const int brc = build_image(job->mesh, surf_mode, riv_mode, c.stepsize, order, &p->im);
  if (brc != PIHM_GPU_OK) return brc;
  const int ne = p->im.ne, nr = p->im.nr;
  const size_t neq = 3 * (size_t)ne + 2 * (size_t)nr;
  p->y0.assign(job->y0, job->y0 + neq);
  if (job->elem_bc) p->elem_bc.assign(job->elem_bc, job->elem_bc + 3 * (size_t)ne);
  if (job->river_bc) p->river_bc.assign(job->river_bc, job->river_bc + nr);
  if (!job->land && !job->noah) {
    p->pcp.assign(job->pcpdrp, job->pcpdrp + job->nsteps);
    p->edir.assign(job->edir, job->edir + job->nsteps);
    p->ett.assign(job->ett, job->ett + job->nsteps);
  }
  p->ctrl = c;
  p->nsteps = job->nsteps;
  p->outlet = job->outlet;
  // a deck's forcing
  p->deck = job->deck;
  if (job->deck) {
    for (int q = 0; q < 3 * ne && !p->has_bc; q++) p->has_bc = job->mesh->bc_type[q] != 0;
    for (int r = 0; r < nr && !p->has_bc; r++) p->has_bc = job->mesh->riverbc_type[r] != 0;
  }
  p->land = job->land;
  p->forcing = job->forcing;
  p->start = job->start;
  p->lsm_step = job->lsm_step;
  p->noah = job->noah;
  p->noah_state = job->noah_state;
  p->noah_forcing = job->noah_forcing;
  p->noah_nforcing = job->noah_nforcing;
  p->noah_lsm = job->noah_lsm_step;
  if (job->noah) {
    // every land-surface step of the run must have its forcing set
    const double t_last = (double)(job->nsteps > 0 ? job->nsteps - 1 : 0) * c.stepsize;
    if ((int64_t)(t_last / job->noah_lsm_step) >= job->noah_nforcing) return PIHM_GPU_ERR_ARG;
  }
  if (job->land) {
    p->cmc0.assign(ne, 0.0);
    p->sneqv0.assign(ne, 0.0);
    if (job->cmc0) p->cmc0.assign(job->cmc0, job->cmc0 + ne);
    if (job->sneqv0) p->sneqv0.assign(job->sneqv0, job->sneqv0 + ne);
  }
  return PIHM_GPU_OK;
}

// The deck's forcing of a watershed in the arena: the land-surface instance
// reading this watershed's mesh planes and writing its forcing planes, its
// initial storage, and the pinned staging of the boundary values.
int attach_deck(pihm_batch *B, Sys *s, const Prepared &p) {
  s->deck = p.deck;
  s->has_bc = p.has_bc;
  s->start = p.start;
  s->lsm_step = p.lsm_step;
  if (s->has_bc && cudaMallocHost(&s->bc_stage, sizeof(double) * (3 * (size_t)s->ne + s->nr)) != cudaSuccess) {
    s->bc_stage = nullptr;
    return PIHM_GPU_ERR_NOMEM;
  }
  if (p.noah) {
    DevMesh &m = B->A.m;
    const int64_t eo = s->eoff, NE = B->ne_cap;
    NoahTargets tg{m.d_sub + eo, m.d_et + eo, NE, const_cast<double *>(m.noah_etgw) + eo,
                   const_cast<double *>(m.noah_satn) + eo, const_cast<double *>(m.noah_fcr) + eo,
                   const_cast<double *>(m.edir) + eo, const_cast<double *>(m.ett) + eo,
                   const_cast<double *>(m.pcpdrp) + eo, const_cast<int32_t *>(m.noah_wtin) + eo};
    int rc = noah_build(p.noah, p.noah_state, p.im.perm.data(), s->ne, tg, B->st, &s->noah);
    if (rc != PIHM_GPU_OK) return rc;
    B->noah_resident++;  // free_ranges counts it back with the instance
    int64_t n = 0;
    rc = noah_launch_begin(s->noah, B->A.vec + s->soff, B->st, &n);  // ws0 of the first MassBalance
    if (rc != PIHM_GPU_OK) return rc;
    s->noah_forcing = p.noah_forcing;
    s->noah_nforcing = p.noah_nforcing;
    s->noah_lsm = p.noah_lsm;
    const int32_t one = 1;
    if (cudaMemcpyAsync(const_cast<int32_t *>(m.sys_noah) + s->slot, &one, sizeof(one), cudaMemcpyHostToDevice,
                        B->st) != cudaSuccess ||
        cudaStreamSynchronize(B->st) != cudaSuccess)
      return PIHM_GPU_ERR_CUDA;
    m.noah = 1;
    m.diag = 1;  // MassBalance reads each watershed's last evaluation's fluxes
  }
  if (!p.land) return PIHM_GPU_OK;
  DevMesh &m = B->A.m;
  const int64_t eo = s->eoff;
  LandTargets tg{m.depth + eo, m.porosity + eo, m.rzd + eo, m.d_rzd + eo, const_cast<double *>(m.pcpdrp) + eo,
                 const_cast<double *>(m.edir) + eo, const_cast<double *>(m.ett) + eo};
  int rc = land_build(p.land, p.forcing, p.im.perm.data(), s->ne, p.im.el[EP_ZMAX].data(), tg, &s->land);
  if (rc != PIHM_GPU_OK) return rc;
  // every land-surface step of the run must lie inside the series
  const int64_t step = (int64_t)p.ctrl.stepsize;
  const int64_t last = (int64_t)(p.nsteps > 0 ? p.nsteps - 1 : 0) * step;
  const int64_t t_end = p.start + last - last % p.lsm_step;
  if (p.start < s->land.t_lo || t_end > s->land.t_hi) return PIHM_GPU_ERR_ARG;
  return land_set_state(s->land, p.im.perm.data(), p.cmc0.data(), p.sneqv0.data(), B->st);
}

// ApplyBc at model time t into the arena (pinned staging, asynchronous; the
// round that applies it synchronises before the staging is reused).
int stage_bc(pihm_batch *B, Sys *s, int64_t t) {
  const int ne = s->ne, nr = s->nr;
  std::vector<double> e(3 * (size_t)ne), r((size_t)nr);
  if (pihm_deck_bc(s->deck, t, e.data(), r.data()) != PIHM_GPU_OK) return PIHM_GPU_ERR_ARG;
  double *h = s->bc_stage;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < ne; i++) h[(size_t)j * ne + i] = e[3 * (size_t)s->perm[i] + j];
  std::copy(r.begin(), r.end(), h + 3 * (size_t)ne);
  DevMesh &m = B->A.m;
  const int64_t NE = B->ne_cap;
  for (int j = 0; j < 3; j++)
    if (ne && cudaMemcpyAsync((double *)m.elem_bc + j * NE + s->eoff, h + (size_t)j * ne, sizeof(double) * ne,
                              cudaMemcpyHostToDevice, B->st) != cudaSuccess)
      return PIHM_GPU_ERR_CUDA;
  if (nr && cudaMemcpyAsync((double *)m.river_bc + s->roff, h + 3 * (size_t)ne, sizeof(double) * nr,
                            cudaMemcpyHostToDevice, B->st) != cudaSuccess)
    return PIHM_GPU_ERR_CUDA;
  return PIHM_GPU_OK;
}

// Reserve arena ranges for a prepared job, upload it and start its model
// loop.  PIHM_GPU_ERR_NOMEM when it does not fit now.
int admit(pihm_batch *B, const Prepared &p, int32_t *id) {
  const SystemImage &im = p.im;
  int slot = -1;
  for (int k = 0; k < B->max_sys; k++)
    if (!B->slots[k]) {
      slot = k;
      break;
    }
  if (slot < 0) return PIHM_GPU_ERR_NOMEM;
  auto s = std::make_unique<Sys>();
  s->slot = slot;
  s->ne = im.ne;
  s->nr = im.nr;
  s->nedge = im.nedge;
  s->nbank = im.nbank;
  s->nup = (int32_t)im.up_idx.size();
  s->neq = 3LL * im.ne + 2LL * im.nr;
  s->nrec = p.outlet >= 0 ? p.nsteps : 0;
  // admission: every range must fit now
  struct Want {
    RangeAlloc *ra;
    int64_t n, *off;
  } want[] = {{&B->ra_elem, s->ne, &s->eoff},   {&B->ra_riv, s->nr, &s->roff},
              {&B->ra_edge, s->nedge, &s->edoff}, {&B->ra_bank, s->nbank, &s->boff},
              {&B->ra_up, s->nup, &s->upoff},   {&B->ra_state, s->neq, &s->soff},
              {&B->ra_rec, s->nrec, &s->recoff}};
  int got = 0;
  for (; got < 7; got++) {
    const int64_t off = want[got].ra->alloc(want[got].n);
    if (off < 0) break;
    *want[got].off = off;
  }
  if (got < 7) {
    for (int k = 0; k < got; k++) want[k].ra->release(*want[k].off, want[k].n);
    return PIHM_GPU_ERR_NOMEM;
  }
  s->perm = im.perm;
  s->ctrl = p.ctrl;
  s->nsteps = p.nsteps;
  s->outlet = p.outlet;
  s->pcp = p.pcp;
  s->edir = p.edir;
  s->ett = p.ett;
  s->core.ops.s = s.get();
  Sys *sp = s.get();
  B->slots[slot] = std::move(s);
  int prc = place(B, sp, p);
  if (prc == PIHM_GPU_OK) prc = attach_deck(B, sp, p);
  if (prc != PIHM_GPU_OK) {
    free_ranges(B, sp);
    B->slots[slot].reset();
    return prc;
  }
  B->update_extents();
  sp->id = B->next_id++;
  B->by_id[sp->id] = sp;
  // start the model loop: it runs until its first device operation
  sp->task = std::make_unique<Task<int>>(model_run(sp));
  sp->state = S_RUNNING;
  sp->waiting = sp->task->handle();
  resume(sp);
  *id = sp->id;
  return PIHM_GPU_OK;
}


// One round: upload the programs, run them and the right-hand side, read
// the results back and resume the watersheds that were waiting.
int run_round(pihm_batch *B, bool *any) {
  const auto t_start = std::chrono::steady_clock::now();
  *any = false;
  std::vector<Sys *> part;
  RoundSys *rs = (RoundSys *)(B->h_up + B->up_round_off);
  Op *ops = (Op *)(B->h_up + B->up_ops_off);
  uint8_t *active = (uint8_t *)B->h_up;
  std::memset(active, 0, B->max_sys);
  int nops = 0, nblocks = 0;
  bool rhs = false;
  std::vector<Sys *> forcing;  // watersheds whose programs start a model step with a deck's forcing
  int64_t el_req = 0;          // elements of the watersheds evaluated this round
  // Right-hand-side gating: a watershed that waits for an evaluation is held
  // back while others still have reductions to run, until the waiting ones
  // hold at least rhs_gate of the waiting elements, so that evaluations are
  // launched over many watersheds at once.
  int64_t el_rhs = 0, el_other = 0;
  for (auto &up : B->slots) {
    const Sys *s = up.get();
    if (!s || !s->waiting) continue;
    (s->rhs_req ? el_rhs : el_other) += s->ne;
  }
  const bool hold_rhs = el_other > 0 && (double)el_rhs < B->rhs_gate * (double)(el_rhs + el_other);
  for (auto &up : B->slots) {
    Sys *s = up.get();
    if (!s) continue;
    const bool waiting = (bool)s->waiting;
    if (!waiting && s->prog.empty()) continue;
    if (waiting && s->rhs_req && hold_rhs) continue;
    RoundSys &r = rs[part.size()];
    r.sys = s->slot;
    r.prog_off = nops;
    r.prog_len = (int32_t)s->prog.size();
    r.red = waiting ? s->red : -1;
    r.rx = s->rx;
    r.ry = s->ry;
    r.pad0 = r.pad1 = 0;
    r.bstart = nblocks;
    if (s->pending_k >= 0 || s->pending_post) forcing.push_back(s);
    std::memcpy(ops + nops, s->prog.data(), sizeof(Op) * s->prog.size());
    nops += (int)s->prog.size();
    nblocks += (int)pihm_nv::red_grid_for(s->neq);
    if (waiting && s->rhs_req) {
      active[s->slot] = 1;
      rhs = true;
      el_req += s->ne;
    }
    part.push_back(s);
  }
  if (part.empty()) return 0;
  *any = true;
  cudaStream_t st = B->st;
  const size_t up1 = B->up_round_off + sizeof(RoundSys) * part.size();
  if (cudaMemcpyAsync(B->d_up, B->h_up, up1, cudaMemcpyHostToDevice, st) != cudaSuccess) return -1;
  if (nops && cudaMemcpyAsync(B->d_up + B->up_ops_off, B->h_up + B->up_ops_off, sizeof(Op) * nops,
                              cudaMemcpyHostToDevice, st) != cudaSuccess)
    return -1;
  int variant = B->prog_forced >= 0 ? B->prog_forced : B->prog_variant;
  const bool tune = B->prog_forced < 0 && B->tuning && nblocks >= pihm_batch::kTuneMinBlocks && B->tev[0];
  if (tune) {
    variant = B->tune_next;
    B->tune_next = (B->tune_next + 1) % kProgramVariants;
    cudaEventRecord(B->tev[0], st);
  }
  // a deck's boundary values for the model step (src/pihm.c:15-28), in
  // place before any evaluation of the step
  for (Sys *s : forcing)
    if (s->has_bc && stage_bc(B, s, s->start + (int64_t)s->pending_k * (int64_t)s->ctrl.stepsize) != PIHM_GPU_OK)
      return -1;
  if (B->profiling) cudaEventRecord(B->ev[0], st);
  if (launch_program(B->A, (int)part.size(), nblocks, variant, st) != cudaSuccess) return -1;
  B->launches++;
  if (B->profiling) cudaEventRecord(B->ev[1], st);
  if (tune) cudaEventRecord(B->tev[1], st);
  if (rhs && cudaMemsetAsync(B->err_sys, 0, sizeof(unsigned int) * B->max_sys, st) != cudaSuccess) return -1;
  // after the program, which ends the previous model step's state in vector
  // slot 0, and before the evaluation that starts the next step: Flux-PIHM's
  // post-step (Summary's _NOAH_ part and NoahHydrol, src/update.c:34-41,
  // src/noah/noah.c:57-160), then the land-surface step (src/pihm.c:30-66) or
  // Noah() (src/pihm.c:50-58); a Noah error word joins the watershed's
  // evaluation status
  for (Sys *s : forcing) {
    int64_t n = 0;
    if (s->pending_post) {
      if (noah_launch_post(s->noah, B->A.vec + s->soff, s->ctrl.stepsize, st, &n) != PIHM_GPU_OK) return -1;
      s->pending_post = false;
    }
    if (s->pending_k >= 0) {
      const int64_t t = s->start + (int64_t)s->pending_k * (int64_t)s->ctrl.stepsize;
      if (s->land.alloc && (t - s->start) % s->lsm_step == 0 &&
          land_launch(s->land, t, (double)s->lsm_step, B->A.vec + s->soff, st, &n) != PIHM_GPU_OK)
        return -1;
      if (s->noah.alloc) {
        const double tm = (double)s->pending_k * s->ctrl.stepsize;
        const double q = tm / s->noah_lsm;
        if (q == std::floor(q)) {
          if (noah_set_forcing(s->noah, s->noah_forcing + (int64_t)q, s->perm.data(), st) != PIHM_GPU_OK ||
              noah_launch_step(s->noah, s->noah_lsm, B->err_sys + s->slot, st, &n) != PIHM_GPU_OK)
            return -1;
        }
      }
      s->pending_k = -1;
    }
    B->launches += n;
  }
  const bool stune = rhs && B->shape_forced < 0 && B->shape_tuning && el_req >= pihm_batch::kShapeMinElems;
  const int shape = B->shape_forced >= 0 ? B->shape_forced : (stune ? B->shape_next : B->shape_best);
  if (rhs) {
    B->A.m.main_shape = shape;
    if (stune) cudaEventRecord(B->sev[0], st);
    if (launch_rhs(B->A.m, B->A.rhs_in, B->A.rhs_out, st, &B->launches, nullptr, &B->side) != cudaSuccess)
      return -1;
    if (stune) cudaEventRecord(B->sev[1], st);
    B->rhs_rounds++;
  }
  if (B->profiling) cudaEventRecord(B->ev[2], st);
  if (cudaMemcpyAsync(B->h_down, B->d_down, B->down_bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
  const auto t_wait = std::chrono::steady_clock::now();
  if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
  const auto t_done = std::chrono::steady_clock::now();
  B->wait_ms += std::chrono::duration<double, std::milli>(t_done - t_wait).count();
  B->host_ms += std::chrono::duration<double, std::milli>(t_wait - t_start).count();
  if (tune) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, B->tev[0], B->tev[1]);
    B->tune_ms_per_block[variant] += ms / nblocks;
    if (++B->tune_n[variant] >= pihm_batch::kTuneSamples) {
      bool all = true;
      for (int v = 0; v < kProgramVariants; v++) all = all && B->tune_n[v] >= pihm_batch::kTuneSamples;
      if (all) {
        int best = 0;
        for (int v = 1; v < kProgramVariants; v++)
          if (B->tune_ms_per_block[v] / B->tune_n[v] < B->tune_ms_per_block[best] / B->tune_n[best]) best = v;
        B->prog_variant = best;
        B->tuning = false;
      }
    }
  }
  if (stune) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, B->sev[0], B->sev[1]);
    B->shape_ms_per_elem[shape] += ms / (double)el_req;
    B->shape_next = (B->shape_next + 1) % pihm_batch::kShapes;
    if (++B->shape_n[shape] >= pihm_batch::kTuneSamples) {
      bool all = true;
      for (int v = 0; v < pihm_batch::kShapes; v++) all = all && B->shape_n[v] >= pihm_batch::kTuneSamples;
      if (all) {
        int best = 0;
        for (int v = 1; v < pihm_batch::kShapes; v++)
          if (B->shape_ms_per_elem[v] / B->shape_n[v] < B->shape_ms_per_elem[best] / B->shape_n[best]) best = v;
        B->shape_best = best;
        B->shape_tuning = false;
      }
    }
  }
  if (B->profiling) {
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, B->ev[0], B->ev[1]);
    cudaEventElapsedTime(&b, B->ev[1], B->ev[2]);
    B->program_ms += a;
    B->rhs_ms += b;
  }
  B->rounds++;
  const double *res = (const double *)B->h_down;
  const unsigned int *err = (const unsigned int *)(B->h_down + sizeof(double) * 2 * B->max_sys);
  for (Sys *s : part) {
    s->prog.clear();
    if (!s->waiting) continue;  // a finished watershed's last operations
    if (s->red >= 0) {
      const double v = res[2 * s->slot];
      s->red_value = s->red_wrms ? std::sqrt(v / (double)s->neq) : v;
      s->red = -1;
    }
    if (s->rhs_req) {
      s->rhs_rc = err[s->slot] ? -1 : 0;
      s->rhs_req = false;
      // the next program starts by delivering the evaluation
      Op o;
      std::memset(&o, 0, sizeof(o));
      o.code = OP_STAGE_OUT;
      o.x = o.y = o.z = s->rhs_out;
      s->prog.push_back(o);
    }
    resume(s);
  }
  return 0;
}

int read_result(pihm_batch *B, Sys *s, double *y, double *outlet, pihm_bdf_stats *stats) {
  if (y) {
    std::vector<double> yi(s->neq);
    if (cudaMemcpy(yi.data(), B->A.vec + s->soff, sizeof(double) * s->neq, cudaMemcpyDeviceToHost) != cudaSuccess)
      return PIHM_GPU_ERR_CUDA;
    const int ne = s->ne;
    for (int p = 0; p < 3; p++)
      for (int i = 0; i < ne; i++) y[(size_t)p * ne + s->perm[i]] = yi[(size_t)p * ne + i];
    for (int64_t q = 3LL * ne; q < s->neq; q++) y[q] = yi[q];
  }
  if (outlet && s->nrec > 0 &&
      cudaMemcpy(outlet, B->A.rec + s->recoff, sizeof(double) * s->nrec, cudaMemcpyDeviceToHost) != cudaSuccess)
    return PIHM_GPU_ERR_CUDA;
  if (stats) {
    const bdf::Stats st = s->core.stats();
    stats->nst = st.nst;
    stats->nfe = st.nfe;
    stats->nni = st.nni;
    stats->ncfn = st.ncfn;
    stats->netf = st.netf;
    stats->nli = st.nli;
    stats->nfes = st.nfes;
    stats->njtimes = st.njtimes;
    stats->ncfl = st.ncfl;
    stats->nor = st.nor;
    stats->qlast = st.qlast;
    stats->qcur = st.qcur;
    stats->hlast = st.hlast;
    stats->hcur = st.hcur;
    stats->tcur = st.tcur;
  }
  return PIHM_GPU_OK;
}

}  // namespace batch
}  // namespace pihm

extern "C" {

int pihm_batch_create(const pihm_batch_limits *lim, int surf_mode, int riv_mode, int order, pihm_batch **out) {
  if (!lim || !out) return PIHM_GPU_ERR_ARG;
  *out = nullptr;
  if (lim->max_elem <= 0 || lim->max_river < 0 || lim->max_edge < 0 || lim->max_systems <= 0 ||
      lim->max_record < 0 || lim->max_elem > INT32_MAX / 3 || lim->max_river > INT32_MAX / 3 ||
      lim->max_edge > INT32_MAX)
    return PIHM_GPU_ERR_ARG;
  if ((surf_mode != kKinematic && surf_mode != kDiffWave) || (riv_mode != kKinematic && riv_mode != kDiffWave))
    return PIHM_GPU_ERR_ARG;
  if (order != PIHM_GPU_ORDER_REFERENCE && order != PIHM_GPU_ORDER_RCM) return PIHM_GPU_ERR_ARG;
  auto B = std::make_unique<pihm_batch>();
  B->order = order;
  const int64_t NE = lim->max_elem, NR = std::max<int64_t>(lim->max_river, 1);
  const int64_t NED = std::max<int64_t>(lim->max_edge, 1), MS = lim->max_systems;
  B->ne_cap = NE;
  B->nr_cap = NR;
  B->ned_cap = NED;
  B->rec_cap = std::max<int64_t>(lim->max_record, 1);
  B->max_sys = (int)MS;
  const int64_t NEQ = 3 * NE + 2 * NR;
  B->ra_elem = RangeAlloc(NE);
  B->ra_riv = RangeAlloc(NR);
  B->ra_edge = RangeAlloc(NED);
  B->ra_bank = RangeAlloc(NE);
  B->ra_up = RangeAlloc(NR);
  B->ra_state = RangeAlloc(NEQ);
  B->ra_rec = RangeAlloc(B->rec_cap);
  B->slots.resize(MS);
  auto &o = B->owned;
  DevMesh &m = B->A.m;
  std::memset(&m, 0, sizeof(m));
  m.ne = (int32_t)NE;
  m.nr = (int32_t)NR;
  m.nedge = (int32_t)NED;
  m.nbank = (int32_t)NE;
  m.surf_mode = surf_mode;
  m.riv_mode = riv_mode;
  m.dt = 1.0;
  bool ok = true;
  auto D = [&](size_t n) {
    double *p = dalloc<double>(n, o);
    ok = ok && p;
    return p;
  };
  auto I = [&](size_t n) {
    int32_t *p = dalloc<int32_t>(n, o);
    ok = ok && p;
    return p;
  };
  for (int k = 0; k < EP_COUNT; k++) m.*kElemMember[k] = D(NE);
  for (int k = 0; k < XP_COUNT; k++) m.*kEdgeMember[k] = D(3 * NE);
  m.nb = I(3 * NE);
  m.bctype = I(3 * NE);
  m.emap = I(3 * NE);
  m.e_i = I(NED);
  m.e_k = I(NED);
  m.e_invdist = D(NED);
  m.e_subk = D(NED);
  m.e_ovlk = D(NED);
  m.bank_slot = I(NE);
  m.bank_elem = I(NE);
  m.down = I(NR);
  m.left = I(NR);
  m.right = I(NR);
  m.intrpl_ord = I(NR);
  m.bctype_riv = I(NR);
  for (int k = 0; k < RP_COUNT; k++) m.*kRiverMember[k] = D(NR);
  m.up_ptr = I(NR);
  m.up_end = I(NR);
  m.up_idx = I(NR);
  m.pcpdrp = D(NE);
  m.edir = D(NE);
  m.ett = D(NE);
  m.ws0_surf = D(NE);
  m.elem_bc = D(3 * NE);
  m.river_bc = D(NR);
  m.surfh = D(NE);
  m.head = D(NE);
  m.effk = D(NE);
  m.gradmag = D(NE);
  m.rivflow = D(NUM_RIVFLX * NR);
  m.carry_ovl = D(2 * NR);
  m.r_perim = D(NR);
  m.r_crossa = D(NR);
  m.eflux_ovl = D(NED);
  m.eflux_sub = D(NED);
  m.bank_part = D(8 * NE);
  m.err = dalloc<unsigned int>(1, o);
  int32_t *se = I(NE), *sr = I(NR), *sed = I(NED), *sb = I(NE);
  m.sys_elem = se;
  m.sys_riv = sr;
  m.sys_edge = sed;
  m.sys_bank = sb;
  m.sys_dt = D(MS);
  m.sys_inv_dt = D(MS);
  // Flux-PIHM watersheds: the right-hand side's Noah inputs, its diagnostics
  // (MassBalance reads the last evaluation's fluxes) and the per-watershed flag
  m.noah_etgw = D(NE);
  m.noah_satn = D(NE);
  m.noah_fcr = D(NE);
  m.noah_wtin = I(NE);
  m.d_ovl = D(3 * NE);
  m.d_sub = D(3 * NE);
  m.d_infil = D(NE);
  m.d_rechg = D(NE);
  m.d_et = D(5 * NE);
  int32_t *snoah = I(MS);
  m.sys_noah = snoah;
  DeviceArena &A = B->A;
  A.vec = D((size_t)kVecSlots * NEQ);
  A.neq_cap = NEQ;
  A.rhs_in = D(NEQ);
  A.rhs_out = D(NEQ);
  A.sysinfo = dalloc<SysInfo>(MS, o);
  A.partials = D(MS * 2 * pihm_nv::kMaxBlocks);
  A.tickets = dalloc<unsigned int>(MS, o);
  A.rec = D(B->rec_cap);
  A.max_sys = (int)MS;
  // upload block: active flags | round list | ops
  B->up_active_bytes = ((size_t)MS + 255) & ~size_t(255);
  B->up_round_off = B->up_active_bytes;
  B->up_ops_off = B->up_round_off + ((sizeof(RoundSys) * MS + 255) & ~size_t(255));
  const size_t up_bytes = B->up_ops_off + sizeof(Op) * MS * kMaxProgOps;
  B->d_up = (char *)dalloc<char>(up_bytes, o);
  // download block: results | error words
  B->down_bytes = sizeof(double) * 2 * MS + sizeof(unsigned int) * MS;
  B->d_down = (char *)dalloc<char>(B->down_bytes, o);
  if (t_count_bytes) return PIHM_GPU_OK;  // sizes counted, nothing allocated
  if (!ok || !m.err || !A.sysinfo || !A.tickets || !B->d_up || !B->d_down ||
      cudaMallocHost(&B->h_up, up_bytes) != cudaSuccess ||
      cudaMallocHost(&B->h_down, B->down_bytes) != cudaSuccess)
    return PIHM_GPU_ERR_NOMEM;
  m.active = (const uint8_t *)B->d_up;
  A.round = (RoundSys *)(B->d_up + B->up_round_off);
  A.ops = (Op *)(B->d_up + B->up_ops_off);
  A.results = (double *)B->d_down;
  B->err_sys = (unsigned int *)(B->d_down + sizeof(double) * 2 * MS);
  m.err_sys = B->err_sys;
  // everything starts free: owner -1, zero scratch
  bool z = cudaMemset(se, 0xff, sizeof(int32_t) * NE) == cudaSuccess &&
           cudaMemset(sr, 0xff, sizeof(int32_t) * NR) == cudaSuccess &&
           cudaMemset(sed, 0xff, sizeof(int32_t) * NED) == cudaSuccess &&
           cudaMemset(sb, 0xff, sizeof(int32_t) * NE) == cudaSuccess &&
           cudaMemset(A.tickets, 0, sizeof(unsigned int) * MS) == cudaSuccess &&
           cudaMemset(snoah, 0, sizeof(int32_t) * MS) == cudaSuccess &&
           cudaMemset(B->d_up, 0, up_bytes) == cudaSuccess &&
           cudaMemset(m.rivflow, 0, sizeof(double) * NUM_RIVFLX * NR) == cudaSuccess &&
           cudaMemset(m.carry_ovl, 0, sizeof(double) * 2 * NR) == cudaSuccess &&
           cudaMemset(A.rhs_in, 0, sizeof(double) * NEQ) == cudaSuccess &&
           cudaDeviceSynchronize() == cudaSuccess;
  if (!z) return PIHM_GPU_ERR_CUDA;
  if (pihm::create_rhs_streams(&B->side) != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  {
    int dev = 0, pageable = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess)
      B->host_pageable = pageable;
  }
  for (cudaEvent_t &e : B->tev)
    if (cudaEventCreate(&e) != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  for (cudaEvent_t &e : B->sev)
    if (cudaEventCreate(&e) != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  B->update_extents();
  *out = B.release();
  return PIHM_GPU_OK;
}

void pihm_batch_destroy(pihm_batch *b) { delete b; }

int pihm_batch_arena_bytes(const pihm_batch_limits *lim, int64_t *bytes) {
  if (!lim || !bytes) return PIHM_GPU_ERR_ARG;
  int64_t n = 0;
  t_count_bytes = &n;
  pihm_batch *b = nullptr;
  const int rc = pihm_batch_create(lim, 2, 2, PIHM_GPU_ORDER_RCM, &b);
  t_count_bytes = nullptr;
  if (rc != PIHM_GPU_OK) return rc;
  *bytes = n;
  return PIHM_GPU_OK;
}

int pihm_batch_limits_for_memory(int64_t bytes, double rivers_per_elem, double edges_per_elem,
                                 double records_per_elem, int32_t max_systems, pihm_batch_limits *out) {
  if (!out || bytes <= 0 || !(rivers_per_elem >= 0.0) || !(edges_per_elem >= 0.0) || !(records_per_elem >= 0.0) ||
      max_systems <= 0)
    return PIHM_GPU_ERR_ARG;
  auto limits = [&](int64_t ne) {
    pihm_batch_limits l{};
    l.max_elem = ne;
    l.max_river = (int64_t)(rivers_per_elem * (double)ne) + 1;
    l.max_edge = (int64_t)(edges_per_elem * (double)ne) + 16;
    l.max_record = (int64_t)(records_per_elem * (double)ne) + 1;
    l.max_systems = max_systems;
    return l;
  };
  // the largest element capacity whose arena fits (bytes grow with it)
  int64_t lo = 0, hi = INT32_MAX / 3;
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo + 1) / 2;
    const pihm_batch_limits l = limits(mid);
    int64_t need = 0;
    if (pihm_batch_arena_bytes(&l, &need) == PIHM_GPU_OK && need <= bytes) lo = mid;
    else hi = mid - 1;
  }
  if (lo < 1) return PIHM_GPU_ERR_NOMEM;
  *out = limits(lo);
  return PIHM_GPU_OK;
}

int pihm_batch_set_rhs_gate(pihm_batch *b, double gate) {
  if (!b || !(gate >= 0.0 && gate <= 1.0)) return PIHM_GPU_ERR_ARG;
  b->rhs_gate = gate;
  return PIHM_GPU_OK;
}

int pihm_batch_set_stream(pihm_batch *b, void *stream) {
  if (!b) return PIHM_GPU_ERR_ARG;
  b->st = (cudaStream_t)stream;
  return PIHM_GPU_OK;
}

int pihm_batch_add(pihm_batch *B, const pihm_batch_job *job, int32_t *id) {
  if (!B || !id) return PIHM_GPU_ERR_ARG;
  Prepared p;
  const int rc = prepare(job, B->A.m.surf_mode, B->A.m.riv_mode, B->order, &p);
  if (rc != PIHM_GPU_OK) return rc;
  return admit(B, p, id);
}

int pihm_batch_add_many(pihm_batch *B, const pihm_batch_job *jobs, int32_t n, int32_t threads, int32_t *ids,
                        int32_t *admitted) {
  if (!B || !jobs || !ids || n < 0) return PIHM_GPU_ERR_ARG;
  std::vector<Prepared> prep(n);
  std::vector<int> rcs(n, PIHM_GPU_OK);
  const int nt = std::max(1, std::min<int>(threads, n));
  std::atomic<int> next{0};
  auto work = [&] {
    for (int k; (k = next.fetch_add(1)) < n;)
      rcs[k] = prepare(&jobs[k], B->A.m.surf_mode, B->A.m.riv_mode, B->order, &prep[k]);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; t++) pool.emplace_back(work);
  work();
  for (auto &t : pool) t.join();
  int rc = PIHM_GPU_OK, count = 0;
  for (int k = 0; k < n; k++) {
    ids[k] = -1;
    if (rc != PIHM_GPU_OK) continue;
    if (rcs[k] != PIHM_GPU_OK) {
      rc = rcs[k];
      continue;
    }
    const int arc = admit(B, prep[k], &ids[k]);
    if (arc != PIHM_GPU_OK) {
      rc = arc;
      continue;
    }
    count++;
    prep[k] = Prepared();  // release the host image early
  }
  if (admitted) *admitted = count;
  return rc;
}

int pihm_batch_step(pihm_batch *B, int32_t max_rounds, int32_t *running) {
  if (!B) return PIHM_GPU_ERR_ARG;
  for (int32_t r = 0; max_rounds <= 0 || r < max_rounds; r++) {
    bool any = false;
    if (run_round(B, &any) != 0) return PIHM_GPU_ERR_CUDA;
    if (!any) break;
  }
  if (running) {
    int32_t n = 0;
    for (auto &kv : B->by_id)
      if (kv.second->state == S_RUNNING) n++;
    *running = n;
  }
  return PIHM_GPU_OK;
}

int pihm_batch_poll(const pihm_batch *B, int32_t id, int32_t *status, int32_t *solver_rc) {
  if (!B) return PIHM_GPU_ERR_ARG;
  auto it = B->by_id.find(id);
  if (it == B->by_id.end()) return PIHM_GPU_ERR_ARG;
  const Sys *s = it->second;
  const bool pending = !s->prog.empty();  // last operations not yet run
  if (status)
    *status = (s->state == S_RUNNING || pending) ? PIHM_BATCH_RUNNING
              : (s->state == S_DONE)             ? PIHM_BATCH_DONE
                                                 : PIHM_BATCH_FAILED;
  if (solver_rc) *solver_rc = s->solver_rc;
  return PIHM_GPU_OK;
}

int pihm_batch_result(pihm_batch *B, int32_t id, double *y, double *outlet, pihm_bdf_stats *stats,
                      int32_t *steps_done) {
  if (!B) return PIHM_GPU_ERR_ARG;
  auto it = B->by_id.find(id);
  if (it == B->by_id.end()) return PIHM_GPU_ERR_ARG;
  Sys *s = it->second;
  if (s->state == S_RUNNING || !s->prog.empty()) return PIHM_GPU_ERR_ARG;
  const int rc = read_result(B, s, y, outlet, stats);
  if (rc != PIHM_GPU_OK) return rc;
  if (steps_done) *steps_done = s->steps_done;
  return PIHM_GPU_OK;
}

int pihm_batch_release(pihm_batch *B, int32_t id) {
  if (!B) return PIHM_GPU_ERR_ARG;
  auto it = B->by_id.find(id);
  if (it == B->by_id.end()) return PIHM_GPU_ERR_ARG;
  Sys *s = it->second;
  if (s->state == S_RUNNING || !s->prog.empty()) return PIHM_GPU_ERR_ARG;
  free_ranges(B, s);
  const int slot = s->slot;
  B->by_id.erase(it);
  B->slots[slot].reset();
  return PIHM_GPU_OK;
}

int pihm_batch_get_info(const pihm_batch *B, pihm_batch_info *info) {
  if (!B || !info) return PIHM_GPU_ERR_ARG;
  info->rounds = B->rounds;
  info->rhs_rounds = B->rhs_rounds;
  info->launches = B->launches;
  info->elem_used = B->ra_elem.used();
  info->elem_hwm = B->ra_elem.hwm();
  info->resident = (int64_t)B->by_id.size();
  info->host_ms = B->host_ms;
  info->wait_ms = B->wait_ms;
  info->program_ms = B->program_ms;
  info->rhs_ms = B->rhs_ms;
  info->program_variant = B->prog_forced >= 0 ? B->prog_forced : B->prog_variant;
  info->tuning = B->prog_forced < 0 && B->tuning;
  info->rhs_shape = B->shape_forced >= 0 ? B->shape_forced : B->shape_best;
  info->rhs_tuning = B->shape_forced < 0 && B->shape_tuning;
  return PIHM_GPU_OK;
}

int pihm_batch_set_rhs_shape(pihm_batch *B, int32_t shape) {
  if (!B || shape < -1 || shape >= pihm_batch::kShapes) return PIHM_GPU_ERR_ARG;
  B->shape_forced = shape;
  return PIHM_GPU_OK;
}

int pihm_batch_set_program_variant(pihm_batch *B, int32_t variant) {
  if (!B || variant < -1 || variant >= kProgramVariants) return PIHM_GPU_ERR_ARG;
  B->prog_forced = variant;
  return PIHM_GPU_OK;
}

int pihm_batch_set_profiling(pihm_batch *B, int on) {
  if (!B) return PIHM_GPU_ERR_ARG;
  if (on && !B->ev[0])
    for (cudaEvent_t &e : B->ev)
      if (cudaEventCreate(&e) != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  B->profiling = on != 0;
  return PIHM_GPU_OK;
}

}  // extern "C"
