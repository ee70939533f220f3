// Host side of the batch engine, shared by the batch ABI (batch.cpp) and the
// serving layer (serve.cpp): the arena's range allocators, the per-watershed
// record with its integrator coroutine and queued program, and the engine.
#pragma once

#include <coroutine>
#include <cstdint>
#include <map>
#include <memory>
#include <vector>

#include "batch_device.h"
#include "bdf_core.h"
#include "mesh_image.h"
#include "nv_select.h"
#include "pihm_batch.h"

namespace pihm {
namespace batch {

// First-fit allocator of index ranges in [0, cap).
class RangeAlloc {
 public:
  explicit RangeAlloc(int64_t cap = 0) : cap_(cap) {
    if (cap > 0) free_[0] = cap;
  }
  // start of a free range of n entries, or -1
  int64_t alloc(int64_t n) {
    if (n <= 0) return 0;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < n) continue;
      const int64_t start = it->first, len = it->second;
      free_.erase(it);
      if (len > n) free_[start + n] = len - n;
      used_ += n;
      return start;
    }
    return -1;
  }
  void release(int64_t start, int64_t n) {
    if (n <= 0) return;
    used_ -= n;
    auto next = free_.lower_bound(start);
    if (next != free_.end() && start + n == next->first) {
      n += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == start) {
        prev->second += n;
        return;
      }
    }
    free_[start] = n;
  }
  // one past the last allocated entry
  int64_t hwm() const {
    if (free_.empty()) return cap_;
    auto last = std::prev(free_.end());
    return (last->first + last->second == cap_) ? last->first : cap_;
  }
  int64_t used() const { return used_; }

 private:
  int64_t cap_;
  int64_t used_ = 0;
  std::map<int64_t, int64_t> free_;
};

struct Sys;

// The integrator's operations for one watershed of the batch: vectors are
// slot numbers; element-wise operations are queued; reductions and the right
// hand side suspend the calling coroutine until the round has run.
struct BatchOps {
  using Vec = int;
  Sys *s = nullptr;
  int next_slot = 1;  // slot 0 holds the model state y

  int clone(int) { return next_slot < kVecSlots ? next_slot++ : -1; }
  void destroy(int) {}
  bool valid(int v) const { return v >= 0; }

  struct Ew {
    Sys *s;
    bool await_ready() const noexcept;
    void await_suspend(std::coroutine_handle<> h) const noexcept;
    void await_resume() const noexcept {}
  };
  struct Red {
    Sys *s;
    bool await_ready() const noexcept { return false; }
    void await_suspend(std::coroutine_handle<> h) const noexcept;
    double await_resume() const noexcept;
  };
  struct Rhs {
    Sys *s;
    bool await_ready() const noexcept { return false; }
    void await_suspend(std::coroutine_handle<> h) const noexcept;
    int await_resume() const noexcept;
  };

  Ew push(int code, double a, double b, int x, int y, int z, double c = 0.0, int i0 = 0, int i1 = 0);
  Ew push(const pihm_nv::EwCall<int> &e) { return push(e.op, e.a, e.b, e.x, e.y, e.z); }
  Red reduce(int red, int x, int y, bool wrms);

  Ew linear_sum(double a, int x, double b, int y, int z) {
    return push(pihm_nv::select_linear_sum<int>(a, x, b, y, z));
  }
  Ew const_(double c, int z) { return push(pihm_nv::EW_CONST, c, 0.0, z, z, z); }
  Ew scale(double c, int x, int z) { return push(pihm_nv::select_scale<int>(c, x, z)); }
  Ew abs_(int x, int z) { return push(pihm_nv::EW_ABS, 0.0, 0.0, x, x, z); }
  Ew inv(int x, int z) { return push(pihm_nv::EW_INV, 0.0, 0.0, x, x, z); }
  Ew div(int x, int y, int z) { return push(pihm_nv::EW_DIV, 0.0, 0.0, x, y, z); }
  Ew prod(int x, int y, int z) { return push(pihm_nv::EW_PROD, 0.0, 0.0, x, y, z); }
  Ew addconst(int x, double b, int z) { return push(pihm_nv::EW_ADDCONST, 0.0, b, x, x, z); }
  Red dot(int x, int y) { return reduce(pihm_nv::R_DOT, x, y, false); }
  Red maxnorm(int x) { return reduce(pihm_nv::R_MAXABS, x, x, false); }
  Red wrms(int x, int w) { return reduce(pihm_nv::R_WSQ, x, w, true); }
  Red vmin(int x) { return reduce(pihm_nv::R_MIN, x, x, false); }
  Rhs rhs(double t, int y, int ydot);
  // model-step operations
  Ew forcing(double pcp, double edir, double ett) { return push(OP_FORCING, pcp, edir, 0, 0, 0, ett); }
  Ew post_step(int y) { return push(OP_WS0, 0.0, 0.0, y, y, y); }
  Ew record(int k, int seg) { return push(OP_RECORD, 0.0, 0.0, 0, 0, 0, 0.0, k, seg); }
};

enum SysState { S_NEW = 0, S_RUNNING, S_DONE, S_FAILED };

struct Sys {
  int32_t id = -1, slot = -1;
  // arena ranges
  int64_t eoff = 0, roff = 0, edoff = 0, boff = 0, upoff = 0, soff = 0, recoff = 0;
  int32_t ne = 0, nr = 0, nedge = 0, nbank = 0, nup = 0, nrec = 0;
  int64_t neq = 0;
  std::vector<int32_t> perm;
  // job
  pihm_step_control ctrl{};
  int32_t nsteps = 0, outlet = -1, steps_done = 0;
  std::vector<double> pcp, edir, ett;
  // integrator and its coroutine
  bdf::BdfCore<BatchOps> core;
  std::unique_ptr<Task<int>> task;
  std::coroutine_handle<> waiting{};
  int state = S_NEW, solver_rc = 0;
  // the program of the current round
  std::vector<Op> prog;
  int red = -1;
  uint8_t rx = 0, ry = 0;
  bool red_wrms = false, rhs_req = false, rhs_pending_out = false;
  uint8_t rhs_out = 0;
  double red_value = 0.0;
  int rhs_rc = 0;
  // an input deck's forcing (pihm_batch_job.deck / .land)
  const pihm_deck *deck = nullptr;  // ApplyBc every model step when has_bc
  bool has_bc = false;
  LandInstance land;                // the land-surface step; alloc null when absent
  int64_t start = 0, lsm_step = 0;
  int32_t pending_k = -1;           // model step whose forcing the next round applies
  double *bc_stage = nullptr;       // pinned [3 ne + nr], internal order
  // Flux-PIHM (pihm_batch_job.noah)
  NoahInstance noah;                // alloc null when absent
  const pihm_noah_forcing *noah_forcing = nullptr;
  int32_t noah_nforcing = 0;
  double noah_lsm = 0.0;
  bool pending_post = false;        // Summary's _NOAH_ part and NoahHydrol after the step just ended

  Sys() = default;
  Sys(const Sys &) = delete;
  ~Sys() {
    land_release(land);
    noah_release(noah);
    if (bc_stage) cudaFreeHost(bc_stage);
  }
};


// A job with everything the arena needs, built on the host (any thread).
struct Prepared {
  SystemImage im;
  std::vector<double> y0, elem_bc, river_bc, pcp, edir, ett;
  pihm_step_control ctrl{};
  int32_t nsteps = 0, outlet = -1;
  const pihm_deck *deck = nullptr;
  bool has_bc = false;
  const pihm_land_params *land = nullptr;
  const pihm_forcing_series *forcing = nullptr;
  std::vector<double> cmc0, sneqv0;
  int64_t start = 0, lsm_step = 0;
  const pihm_noah_params *noah = nullptr;
  const pihm_noah_state *noah_state = nullptr;
  const pihm_noah_forcing *noah_forcing = nullptr;
  int32_t noah_nforcing = 0;
  double noah_lsm = 0.0;
};

}  // namespace batch
}  // namespace pihm

struct pihm_serve_state;
void pihm_serve_state_free(pihm_serve_state *s);

struct pihm_batch {
  pihm::batch::DeviceArena A{};
  cudaStream_t st = nullptr;
  std::vector<void *> owned;
  int64_t ne_cap = 0, nr_cap = 0, ned_cap = 0, rec_cap = 0;
  int max_sys = 0;
  int order = PIHM_GPU_ORDER_RCM;
  pihm::batch::RangeAlloc ra_elem, ra_riv, ra_edge, ra_bank, ra_up, ra_state, ra_rec;
  std::vector<std::unique_ptr<pihm::batch::Sys>> slots;  // [max_sys]
  std::map<int32_t, pihm::batch::Sys *> by_id;
  int32_t next_id = 0;
  // per-round upload: active flags, then the round list, then the ops
  char *h_up = nullptr;
  char *d_up = nullptr;
  size_t up_active_bytes = 0, up_round_off = 0, up_ops_off = 0;
  // per-round download: results [max_sys][2], then error words [max_sys]
  char *h_down = nullptr;
  char *d_down = nullptr;
  size_t down_bytes = 0;
  unsigned int *err_sys = nullptr;
  // scheduling policy
  double rhs_gate = 1.0;
  // Tuner of the program kernel: while exploring, rounds of at least
  // kTuneMinBlocks blocks rotate through the variants and are timed with
  // events; after kTuneSamples rounds each, the fastest per block is kept.
  // Every variant gives the same bits, so tuning mid-run changes no result.
  static constexpr int kTuneSamples = 12, kTuneMinBlocks = 512;
  int prog_variant = 1, prog_forced = -1, tune_next = 0;
  bool tuning = true;
  double tune_ms_per_block[pihm::batch::kProgramVariants] = {0};
  int tune_n[pihm::batch::kProgramVariants] = {0};
  cudaEvent_t tev[2] = {nullptr, nullptr};
  // Tuner of k_elem_main's block shape (DevMesh::main_shape: 512 x 2,
  // 256 x 4, 128 x 8 per SM): evaluation rounds over at least
  // kShapeMinElems requesting elements rotate through the shapes and are
  // timed with events; after kTuneSamples rounds each, the fastest per
  // requesting element is kept.  Every shape gives the same bits.
  static constexpr int kShapes = 3;
  static constexpr int64_t kShapeMinElems = 20000;
  int shape_best = 1, shape_forced = -1, shape_next = 0;
  bool shape_tuning = true;
  double shape_ms_per_elem[kShapes] = {0};
  int shape_n[kShapes] = {0};
  cudaEvent_t sev[2] = {nullptr, nullptr};
  int noah_resident = 0;  // Flux-PIHM watersheds resident (the arena's noah and diagnostics switch on)
  pihm::RhsStreams side;  // river kernel beside the element kernels
  int host_pageable = 0;  // the device can access pageable host memory (uploads by one gather kernel)
  // counters and timing (host: building rounds and running the coroutines;
  // wait: blocked on the device; program/rhs: device time, when profiling)
  long long rounds = 0, rhs_rounds = 0, launches = 0;
  double host_ms = 0, wait_ms = 0, program_ms = 0, rhs_ms = 0;
  bool profiling = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};

  pihm_serve_state *serve = nullptr;  // serving layer (serve.cpp), created on first use

  ~pihm_batch() {
    pihm_serve_state_free(serve);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : tev)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : sev)
      if (e) cudaEventDestroy(e);
    if (side.fork) cudaEventDestroy(side.fork);
    if (side.join) cudaEventDestroy(side.join);
    if (side.side) cudaStreamDestroy(side.side);
    slots.clear();
    for (void *p : owned) cudaFree(p);
    if (h_up) cudaFreeHost(h_up);
    if (h_down) cudaFreeHost(h_down);
  }

  void update_extents() {
    A.m.ne_run = (int32_t)ra_elem.hwm();
    A.m.nr_run = (int32_t)ra_riv.hwm();
    A.m.nedge_run = (int32_t)ra_edge.hwm();
    A.m.nbank_run = (int32_t)ra_bank.hwm();
  }
};

namespace pihm {
namespace batch {

int prepare(const pihm_batch_job *job, int surf_mode, int riv_mode, int order, Prepared *p);
int admit(pihm_batch *B, const Prepared &p, int32_t *id);
int run_round(pihm_batch *B, bool *any);
void free_ranges(pihm_batch *B, Sys *s);
// A finished watershed's results (reference order) and counters.
int read_result(pihm_batch *B, Sys *s, double *y, double *outlet, pihm_bdf_stats *stats);

}  // namespace batch
}  // namespace pihm
