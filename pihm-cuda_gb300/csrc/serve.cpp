// Serving layer of the batch engine (pihm_serve_*, include/pihm_batch.h).
//
// Requests are queued with an arrival time.  Once a request has arrived, a
// pool of host threads prepares it (validation, renumbering, derived
// constants: the host image) while the GPU keeps integrating the resident
// watersheds.  The serving loop admits prepared requests in arrival order as
// soon as the arena has room for them (continuous batching: a request joins
// the rounds already in flight), runs rounds, and retires each watershed the
// moment it finishes -- its results are copied to the host and its arena
// ranges are freed for the next request.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>

#include "batch_engine.h"

using namespace pihm;
using namespace pihm::batch;

namespace {

enum ReqState { Q_WAITING = 0, Q_PREPARING, Q_READY, Q_RESIDENT, Q_DONE, Q_FAILED };

// A deep copy of a job, so the caller's arrays may go away after submit.
struct OwnedJob {
  pihm_gpu_mesh mesh{};
  std::vector<std::vector<int32_t>> ints;
  std::vector<std::vector<double>> dbls;
  std::vector<double> y0, elem_bc, river_bc, pcp, edir, ett, cmc0, sneqv0;
  pihm_batch_job job{};

  explicit OwnedJob(const pihm_batch_job &j) {
    const pihm_gpu_mesh &g = *j.mesh;
    const size_t ne = g.nelem, nr = g.nriver;
    mesh.nelem = g.nelem;
    mesh.nriver = g.nriver;
    auto I = [&](const int32_t *src, size_t n) {
      ints.emplace_back(src, src + n);
      return ints.back().data();
    };
    auto D = [&](const double *src, size_t n) {
      dbls.emplace_back(src, src + n);
      return dbls.back().data();
    };
    ints.reserve(7);
    dbls.reserve(40);
    mesh.nabr = I(g.nabr, 3 * ne);
    mesh.bc_type = I(g.bc_type, 3 * ne);
    mesh.area = D(g.area, ne);
    mesh.zmin = D(g.zmin, ne);
    mesh.zmax = D(g.zmax, ne);
    mesh.edge = D(g.edge, 3 * ne);
    mesh.nabrdist = D(g.nabrdist, 3 * ne);
    mesh.nabr_x = D(g.nabr_x, 3 * ne);
    mesh.nabr_y = D(g.nabr_y, 3 * ne);
    mesh.depth = D(g.depth, ne);
    mesh.ksath = D(g.ksath, ne);
    mesh.ksatv = D(g.ksatv, ne);
    mesh.kinfv = D(g.kinfv, ne);
    mesh.dinf = D(g.dinf, ne);
    mesh.alpha = D(g.alpha, ne);
    mesh.beta = D(g.beta, ne);
    mesh.porosity = D(g.porosity, ne);
    mesh.dmac = D(g.dmac, ne);
    mesh.kmach = D(g.kmach, ne);
    mesh.kmacv = D(g.kmacv, ne);
    mesh.areafv = D(g.areafv, ne);
    mesh.areafh = D(g.areafh, ne);
    mesh.rough = D(g.rough, ne);
    mesh.rzd = D(g.rzd, ne);
    mesh.down = I(g.down, nr);
    mesh.leftele = I(g.leftele, nr);
    mesh.rightele = I(g.rightele, nr);
    mesh.intrpl_ord = I(g.intrpl_ord, nr);
    mesh.riverbc_type = I(g.riverbc_type, nr);
    mesh.riv_area = D(g.riv_area, nr);
    mesh.riv_zmin = D(g.riv_zmin, nr);
    mesh.riv_zmax = D(g.riv_zmax, nr);
    mesh.riv_zbed = D(g.riv_zbed, nr);
    mesh.riv_node_zmax = D(g.riv_node_zmax, nr);
    mesh.riv_dist_left = D(g.riv_dist_left, nr);
    mesh.riv_dist_right = D(g.riv_dist_right, nr);
    mesh.riv_depth = D(g.riv_depth, nr);
    mesh.riv_coeff = D(g.riv_coeff, nr);
    mesh.riv_length = D(g.riv_length, nr);
    mesh.riv_width = D(g.riv_width, nr);
    mesh.riv_rough = D(g.riv_rough, nr);
    mesh.riv_cwr = D(g.riv_cwr, nr);
    mesh.riv_ksath = D(g.riv_ksath, nr);
    mesh.riv_ksatv = D(g.riv_ksatv, nr);
    mesh.riv_bedthick = D(g.riv_bedthick, nr);
    mesh.riv_porosity = D(g.riv_porosity, nr);
    y0.assign(j.y0, j.y0 + 3 * ne + 2 * nr);
    if (j.elem_bc) elem_bc.assign(j.elem_bc, j.elem_bc + 3 * ne);
    if (j.river_bc) river_bc.assign(j.river_bc, j.river_bc + nr);
    if (j.pcpdrp) pcp.assign(j.pcpdrp, j.pcpdrp + j.nsteps);
    if (j.edir) edir.assign(j.edir, j.edir + j.nsteps);
    if (j.ett) ett.assign(j.ett, j.ett + j.nsteps);
    if (j.cmc0) cmc0.assign(j.cmc0, j.cmc0 + ne);
    if (j.sneqv0) sneqv0.assign(j.sneqv0, j.sneqv0 + ne);
    job = j;  // the deck, land parameters and forcing series stay the caller's
    job.mesh = &mesh;
    job.y0 = y0.data();
    job.elem_bc = elem_bc.empty() ? nullptr : elem_bc.data();
    job.river_bc = river_bc.empty() ? nullptr : river_bc.data();
    job.pcpdrp = j.pcpdrp ? pcp.data() : nullptr;
    job.edir = j.edir ? edir.data() : nullptr;
    job.ett = j.ett ? ett.data() : nullptr;
    job.cmc0 = j.cmc0 ? cmc0.data() : nullptr;
    job.sneqv0 = j.sneqv0 ? sneqv0.data() : nullptr;
  }
};

struct Request {
  int32_t ticket = -1, id = -1, nelem = 0, state = Q_WAITING, solver_rc = 0, prep_rc = 0;
  double t_arrival = 0, t_admit = -1, t_done = -1;
  std::unique_ptr<OwnedJob> job;
  std::unique_ptr<Prepared> prep;
  std::vector<double> y, outlet;
  pihm_bdf_stats stats{};
};

}  // namespace

struct pihm_serve_state {
  std::vector<std::unique_ptr<Request>> reqs;  // by ticket
  std::mutex mu;
  std::condition_variable cv;
  std::deque<int32_t> todo;  // arrived, waiting for a worker
  bool stop = false;
  std::vector<std::thread> workers;
  int surf_mode = 2, riv_mode = 2, order = 1;

  ~pihm_serve_state() { stop_workers(); }

  void stop_workers() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv.notify_all();
    for (auto &t : workers) t.join();
    workers.clear();
    stop = false;
  }

  void worker() {
    for (;;) {
      int32_t tk;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || !todo.empty(); });
        if (stop) return;
        tk = todo.front();
        todo.pop_front();
      }
      Request &r = *reqs[tk];
      auto p = std::make_unique<Prepared>();
      const int rc = prepare(&r.job->job, surf_mode, riv_mode, order, p.get());
      {
        std::lock_guard<std::mutex> lk(mu);
        r.prep_rc = rc;
        if (rc == PIHM_GPU_OK) r.prep = std::move(p);
        r.job.reset();
        r.state = (rc == PIHM_GPU_OK) ? Q_READY : Q_FAILED;
      }
    }
  }
};

void pihm_serve_state_free(pihm_serve_state *s) { delete s; }

static pihm_serve_state *serve_state(pihm_batch *B) {
  if (!B->serve) {
    B->serve = new pihm_serve_state();
    B->serve->surf_mode = B->A.m.surf_mode;
    B->serve->riv_mode = B->A.m.riv_mode;
    B->serve->order = B->order;
  }
  return B->serve;
}

extern "C" {

int pihm_serve_submit(pihm_batch *B, const pihm_batch_job *job, double arrival_s, int32_t *ticket) {
  if (!B || !job || !job->mesh || !job->y0 || !ticket || job->nsteps < 0 ||
      (job->nsteps > 0 && !job->land && !job->noah && (!job->pcpdrp || !job->edir || !job->ett)) ||
      !(arrival_s >= 0.0))
    return PIHM_GPU_ERR_ARG;
  pihm_serve_state *S = serve_state(B);
  auto r = std::make_unique<Request>();
  r->ticket = (int32_t)S->reqs.size();
  r->t_arrival = arrival_s;
  r->nelem = job->mesh->nelem;
  r->job = std::make_unique<OwnedJob>(*job);
  *ticket = r->ticket;
  std::lock_guard<std::mutex> lk(S->mu);
  S->reqs.push_back(std::move(r));
  return PIHM_GPU_OK;
}

int pihm_serve_run(pihm_batch *B, int32_t workers) {
  if (!B) return PIHM_GPU_ERR_ARG;
  pihm_serve_state *S = serve_state(B);
  if (workers < 1) workers = 1;
  for (int k = 0; k < workers; k++) S->workers.emplace_back([S] { S->worker(); });
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  auto now = [&] { return std::chrono::duration<double>(clock::now() - t0).count(); };
  // arrival order
  std::vector<int32_t> order(S->reqs.size());
  for (size_t k = 0; k < order.size(); k++) order[k] = (int32_t)k;
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return S->reqs[a]->t_arrival < S->reqs[b]->t_arrival; });
  size_t next_arrival = 0;  // first request in `order` not yet handed to the workers
  size_t next_admit = 0;    // first request in `order` not yet admitted (FIFO)
  std::map<int32_t, int32_t> resident;  // batch id -> ticket
  int rc = PIHM_GPU_OK;
  while (rc == PIHM_GPU_OK) {
    const double t = now();
    // hand arrived requests to the preparation workers
    {
      std::lock_guard<std::mutex> lk(S->mu);
      bool any = false;
      while (next_arrival < order.size() && S->reqs[order[next_arrival]]->t_arrival <= t) {
        Request &r = *S->reqs[order[next_arrival++]];
        if (r.state == Q_WAITING) {
          r.state = Q_PREPARING;
          S->todo.push_back(r.ticket);
          any = true;
        }
      }
      if (any) S->cv.notify_all();
    }
    // admit prepared requests in arrival order while they fit
    while (next_admit < order.size()) {
      Request &r = *S->reqs[order[next_admit]];
      int st;
      {
        std::lock_guard<std::mutex> lk(S->mu);
        st = r.state;
      }
      if (st == Q_FAILED) {  // rejected by validation
        r.t_done = now();
        next_admit++;
        continue;
      }
      if (st != Q_READY) break;
      int32_t id = -1;
      const int arc = admit(B, *r.prep, &id);
      if (arc == PIHM_GPU_ERR_NOMEM && !resident.empty()) break;  // wait for room
      if (arc == PIHM_GPU_ERR_NOMEM) {  // larger than the whole arena: never fits
        r.state = Q_FAILED;
        r.prep_rc = arc;
        r.t_done = now();
        r.prep.reset();
        next_admit++;
        continue;
      }
      if (arc != PIHM_GPU_OK) {
        r.state = Q_FAILED;
        r.prep_rc = arc;
        r.t_done = now();
        r.prep.reset();
        next_admit++;
        continue;
      }
      r.id = id;
      r.state = Q_RESIDENT;
      r.t_admit = now();
      r.prep.reset();
      resident[id] = r.ticket;
      next_admit++;
    }
    // one round for everything resident
    bool ran = false;
    if (!resident.empty() && run_round(B, &ran) != 0) {
      rc = PIHM_GPU_ERR_CUDA;
      break;
    }
    // retire finished watersheds
    for (auto it = resident.begin(); it != resident.end();) {
      Sys *s = B->by_id[it->first];
      if (s->state == S_RUNNING || !s->prog.empty()) {
        ++it;
        continue;
      }
      Request &r = *S->reqs[it->second];
      r.y.assign(s->neq, 0.0);
      r.outlet.assign(s->nrec, 0.0);
      if (read_result(B, s, r.y.data(), r.outlet.data(), &r.stats) != PIHM_GPU_OK) rc = PIHM_GPU_ERR_CUDA;
      r.solver_rc = s->solver_rc;
      r.state = (s->state == S_DONE) ? Q_DONE : Q_FAILED;
      r.t_done = now();
      free_ranges(B, s);
      B->slots[s->slot].reset();
      B->by_id.erase(it->first);
      it = resident.erase(it);
    }
    if (next_admit >= order.size() && resident.empty()) break;  // all served
    if (resident.empty()) {
      // idle: wait for the next arrival or for a preparation to finish
      const double wait = (next_arrival < order.size())
                              ? std::max(0.0, S->reqs[order[next_arrival]]->t_arrival - now())
                              : 0.0005;
      std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.0005)));
    }
  }
  S->stop_workers();
  return rc;
}

int pihm_serve_record_get(const pihm_batch *B, int32_t ticket, pihm_serve_record *rec) {
  if (!B || !B->serve || !rec || ticket < 0 || ticket >= (int32_t)B->serve->reqs.size())
    return PIHM_GPU_ERR_ARG;
  const Request &r = *B->serve->reqs[ticket];
  rec->status = r.state == Q_DONE ? PIHM_BATCH_DONE : (r.state == Q_FAILED ? PIHM_BATCH_FAILED : PIHM_BATCH_RUNNING);
  rec->solver_rc = r.state == Q_FAILED && r.prep_rc != PIHM_GPU_OK ? r.prep_rc : r.solver_rc;
  rec->nelem = r.nelem;
  rec->t_arrival = r.t_arrival;
  rec->t_admit = r.t_admit;
  rec->t_done = r.t_done;
  return PIHM_GPU_OK;
}

int pihm_serve_result(const pihm_batch *B, int32_t ticket, double *y, double *outlet, pihm_bdf_stats *stats) {
  if (!B || !B->serve || ticket < 0 || ticket >= (int32_t)B->serve->reqs.size()) return PIHM_GPU_ERR_ARG;
  const Request &r = *B->serve->reqs[ticket];
  if (r.state != Q_DONE && r.state != Q_FAILED) return PIHM_GPU_ERR_ARG;
  if (y && !r.y.empty()) std::copy(r.y.begin(), r.y.end(), y);
  if (outlet && !r.outlet.empty()) std::copy(r.outlet.begin(), r.outlet.end(), outlet);
  if (stats) *stats = r.stats;
  return PIHM_GPU_OK;
}

}  // extern "C"
