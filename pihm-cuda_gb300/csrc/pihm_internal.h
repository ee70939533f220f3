// Internal layout of the GB300 PIHM right-hand-side library.
//
// All element data live in internal (renumbered) order as structure-of-arrays
// FP64 planes; per-edge quantities are three planes [3][nelem] so that thread
// i reading edge j touches consecutive addresses.  River segments keep the
// reference order (they are ~3 % of the work and their upstream sums must run
// in reference order anyway).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pihm_gpu.h"
#include "pihm_land.h"
#include "pihm_noah.h"

namespace pihm {

// Physical and numerical constants of the reference model
// (src/include/pihm_const.h:64-156).
constexpr double kGrav = 9.80665;
constexpr double kPsiMin = -70.0;
constexpr double kDeprStg = 1E-4;
constexpr double kGradMin = 5E-8;
constexpr double kSatMin = 0.1;
constexpr double kRivGradMin = 0.05;
constexpr int kRectangle = 1, kTriangle = 2, kQuadratic = 3, kCubic = 4;
constexpr int kDirichlet = -1, kNeumann = -2, kZeroDpthGrad = -3, kCritDpth = -4;
constexpr int kKinematic = 1, kDiffWave = 2;
// river flux slots (src/include/pihm_const.h:127-137)
enum RivFlx {
  UP_CHANL2CHANL = 0, DOWN_CHANL2CHANL, LEFT_SURF2CHANL, RIGHT_SURF2CHANL,
  LEFT_AQUIF2CHANL, RIGHT_AQUIF2CHANL, CHANL_LKG, LEFT_AQUIF2AQUIF,
  RIGHT_AQUIF2AQUIF, DOWN_AQUIF2AQUIF, UP_AQUIF2AQUIF, NUM_RIVFLX
};

// Neighbour encoding inside the library: >= 0 internal element index,
// -1 - s for river segment s, kBoundary for the domain edge.
constexpr int32_t kBoundary = INT32_MIN;

// Device view of one watershed, passed by value to the kernels.
struct DevMesh {
  int32_t ne, nr, nbank;
  int surf_mode, riv_mode;
  double dt, inv_dt;  // model step (s), caps infiltration; its reciprocal

  // element static data [ne]
  const double *area, *zmin, *zmax;
  const double *depth, *ksath, *ksatv, *kinfv, *dinf, *alpha, *beta, *porosity,
      *dmac, *kmach, *kmacv, *areafv, *areafh, *rough, *rzd;
  // per edge [3][ne]
  const int32_t *nb;        // neighbour (encoded as above)
  const int32_t *bctype;    // boundary condition type (boundary edges)
  const double *edge, *nabrdist, *nabr_x, *nabr_y;
  const double *inv_den_x, *inv_den_y;  // [ne] reciprocals of the gradient's geometric denominators
  // element constants derived once at load: the reference evaluates these
  // sub-expressions inline with the same operation order (bit-identical),
  // except the reciprocals, which replace divisions (<= 1 ulp apart)
  const double *inv_area, *inv_por, *inv_alpha;
  const double *vg_m, *vg_e, *vg_ib;         // beta/(beta-1), (beta-1)/beta, 1/beta
  const double *kinf_mat, *kmac_a, *kv2_mac; // kinfv(1-areafh), kmacv areafh, AvgKv k2
  const double *d_dinf, *d_rzd, *d_dmac;     // depth-dinf, depth-rzd, depth-dmac
  const double *kh_k1;                       // EffKh k1 = kmach areafv + ksath (1-areafv)
  const double *inv_depth;                   // 1/depth (Recharge's denominators sum to depth)
  // interior edges: each pair of neighbouring elements is evaluated once by
  // its owner and read with a sign by the other side
  int32_t nedge;
  const int32_t *e_i, *e_k;                  // owner, neighbour (internal)
  const double *e_invdist, *e_subk, *e_ovlk;  // 1/dist, edge/(2 dist), edge/(dist avg_rough)
  const int32_t *emap;                       // [3][ne] +(e+1) owner, -(e+1) other, 0 none
  const int32_t *bank_slot;     // [ne] slot of an element with river edges
  const int32_t *bank_elem;     // [nbank]

  // river static data [nr], reference order
  const int32_t *down, *left, *right, *intrpl_ord, *bctype_riv;  // left/right internal
  const double *r_area, *r_zmin, *r_zmax, *r_zbed, *r_node_zmax, *r_dist_left,
      *r_dist_right, *r_depth, *r_coeff, *r_length, *r_width, *r_rough, *r_cwr,
      *r_ksath, *r_ksatv, *r_bedthick, *r_porosity;
  // derived at load: 1/(length/2), 1/((length + downstream length)/2) (0 at
  // an outlet), 1/dist_left, 1/dist_right, 1/bedthick, cwr 2 sqrt(2g) length/3
  const double *r_inv_half_len, *r_inv_dist_down, *r_inv_dist_left, *r_inv_dist_right,
      *r_inv_bedthick, *r_ovl_coef;
  // coefficient-only factors of the channel area and wetted perimeter, by
  // shape (k_riv_geom)
  const double *r_geo0, *r_geo1, *r_geo2, *r_geo3, *r_geo4;
  const int32_t *up_ptr, *up_idx;  // CSR of upstream segments, reference order
  const int32_t *up_end;           // [nr] end of each upstream list (up_ptr + 1 in a
                                   // single-watershed context)

  // inputs besides y
  const double *pcpdrp, *edir, *ett, *ws0_surf;  // [ne]
  const double *elem_bc;   // [3][ne]
  const double *river_bc;  // [nr]

  // scratch written and read inside one evaluation
  double *surfh, *head, *effk, *gradmag;  // [ne]
  double *eflux_ovl, *eflux_sub;          // [nedge]
  double *rivflow;                        // [11][nr]
  double *r_perim, *r_crossa;             // [nr] wetted perimeter and area at the stage
  double *carry_ovl;                      // [2][nr] river-edge overland flux (LEFT, RIGHT
                                          // SURF2CHANL of the last evaluation) that the
                                          // next evaluation's Infil reads
  double *bank_part;                      // [8][nbank]
  // diagnostics (optional)
  double *d_ovl, *d_sub, *d_infil, *d_rechg, *d_et;  // [3][ne],[3][ne],[ne],[ne],[5][ne]
  int diag;

  unsigned int *err;  // error word

  // Launch extents.  A single-watershed context evaluates every item
  // (ne_run = ne, ...); the batch engine's arena places watersheds in ranges of
  // planes sized ne, nr, nedge, nbank (the capacities, which stay the plane
  // strides) and evaluates items below the high-water marks.
  int32_t ne_run, nr_run, nedge_run, nbank_run;
  // k_elem_main's block shape (kMainShapes in rhs_kernels.cu): 0 = 512
  // threads x 2 blocks per SM, 1 = 256 x 4, 2 = 128 x 8 (64 registers each)
  int32_t main_shape;
  // Batch engine only (null otherwise): the watershed of each item (-1 for a
  // free arena slot), the watersheds evaluated by this call, their model steps
  // and their error words.
  const int32_t *sys_elem, *sys_riv, *sys_edge, *sys_bank;
  const uint8_t *active;
  const double *sys_dt, *sys_inv_dt;
  unsigned int *err_sys;
  // Batch engine: 1 for the watersheds that run Flux-PIHM (noah then marks
  // that some do); null otherwise
  const int32_t *sys_noah;

  // Flux-PIHM (_NOAH_) right-hand side, when noah != 0: per element, from
  // Noah's per-step outputs, the transpiration of the layers from the water
  // table down to the root depth (GwTransp's sum, noah/lsm_func.c:163-185)
  // and whether the water table is within the root zone, Infil's saturation
  // from the top layer's moisture (src/vert_flow.c:94-98, unclamped) and the
  // frozen-soil factor (src/vert_flow.c:16-19)
  int noah;
  const double *noah_etgw, *noah_satn, *noah_fcr;
  const int32_t *noah_wtin;

  // Land-surface model outputs the water balance reads when the model is
  // attached (include/pihm_land.h; null otherwise): precipitation, canopy
  // evaporation, canopy storage, snow water equivalent [ne]
  const double *land_prcp, *land_ec, *land_cmc, *land_sneqv;
};

// Device view of the land-surface model (include/pihm_land.h), internal
// element order.  Derived planes are the reference's own sub-expressions
// evaluated once on the host with the same operations (bit-identical):
// albedo = 0.5 (albedomin + albedomax), rs_ratio = rsmin / rsmax,
// topt_c = topt - 273.15, dsmc = smcref - smcwlt, and the surface pressure
// pres = 101.325e3 ((293 - 0.0065 zmax) / 293)^5.26 (src/is_sm_et.c:47-58,
// 134-137, 148-150).
struct LandDev {
  const int32_t *lc, *meteo, *lai_type;  // [ne], 1-based
  const double *albedo, *shdfac, *cmcfactr, *cfactr, *rgl, *rsmin, *rs_ratio, *rsmax, *topt_c, *smcmin,
      *smcwlt, *dsmc, *zlvl, *pres;
  const double *depth, *porosity, *rzd, *d_rzd;  // the mesh's planes (d_rzd = depth - rzd)
  double cal_edir, cal_ec, cal_ett;
  const int32_t *meteo_off, *meteo_len, *lai_off, *lai_len;  // first knot, knots per series
  const int64_t *meteo_time, *lai_time;
  const double *meteo_data, *lai_data;  // [knot][7], [knot]
  double *cmc, *sneqv;                  // state carried between steps
  double *prcp, *ec, *drip;             // outputs besides the forcing planes
  double *pcpdrp, *edir, *ett;          // the right-hand side's forcing planes
  // per step: each station's record and the values that depend on it alone
  // ([nmeteo][kStationVals], k_land_station) and each LAI series' value
  // [nlai]; per month: each element's log(z/z0) log(10 z/z0) [ne]
  double *station, *lai_value, *ra_num;
  int32_t nmeteo, nlai;
};

// Where a land-surface instance reads the mesh and writes the right-hand
// side's forcing: the element planes of one watershed (a context's own, or a
// watershed's range of the batch arena), internal order.
struct LandTargets {
  const double *depth, *porosity, *rzd, *d_rzd;
  double *pcpdrp, *edir, *ett;
};
// A land-surface model instance: its own allocation (parameters, series,
// state, outputs), the device view, the model times every series covers and
// the month whose aerodynamic term ra_num holds (-1: none yet).
struct LandInstance {
  void *alloc = nullptr;
  LandDev L{};
  int64_t t_lo = 0, t_hi = 0;
  int month = -1;
  int ne = 0;
};
// pihm_gpu_land_init's work for any targets: params and series in reference
// order, perm[internal] = reference element, zmax in internal order (host).
int land_build(const pihm_land_params *p, const pihm_forcing_series *s, const int32_t *perm, int ne,
               const double *zmax, const LandTargets &tg, LandInstance *out);
int land_set_state(LandInstance &li, const int32_t *perm, const double *cmc, const double *sneqv,
                   cudaStream_t st);
// The land-surface step at model time t over `stepsize` seconds, reading the
// state y_dev (the watershed's own layout); adds the kernels it launched.
int land_launch(LandInstance &li, int64_t t, double stepsize, const double *y_dev, cudaStream_t st,
                int64_t *launches);
void land_release(LandInstance &li);

// Where a Noah instance (noah.cu) reads the right-hand side's diagnostics of
// the last evaluation and writes the right-hand side's Flux-PIHM inputs: one
// watershed's elements, from its first element, with the planes' stride
// (a context's own planes, or a range of the batch arena).
struct NoahTargets {
  const double *d_sub, *d_et;  // [3][stride], [5][stride]
  int64_t stride;
  double *etgw, *satn, *fcr, *edir, *ett, *pcpdrp;
  int32_t *wtin;
};
struct NoahPlanes;
// A Noah instance: its own allocation (parameters, forcing, state, outputs
// in internal element order), the device view, and whether no model step has
// ended yet (the first post-step takes the previous state from y).
struct NoahInstance {
  void *alloc = nullptr;
  NoahPlanes *P = nullptr;
  NoahTargets tg{};
  int ne = 0;
  int first = 1;
};
// pihm_gpu_noah_init's work for any targets (perm[internal] = reference element)
int noah_build(const pihm_noah_params *p, const pihm_noah_state *s, const int32_t *perm, int ne,
               const NoahTargets &tg, cudaStream_t st, NoahInstance *out);
int noah_set_state(NoahInstance &n, const pihm_noah_state *s, const int32_t *perm, cudaStream_t st);
int noah_set_forcing(NoahInstance &n, const pihm_noah_forcing *f, const int32_t *perm, cudaStream_t st);
// Noah() over dt, then the right-hand side's inputs
int noah_launch_step(NoahInstance &n, double dt, unsigned int *err, cudaStream_t st, int64_t *launches);
// the state a run starts from (ws0 of MassBalance)
int noah_launch_begin(NoahInstance &n, const double *y0, cudaStream_t st, int64_t *launches);
// Summary's _NOAH_ part and NoahHydrol after a model step ending at y, then the inputs
int noah_launch_post(NoahInstance &n, const double *y, double dt, cudaStream_t st, int64_t *launches);
int noah_get(NoahInstance &n, int field, const int32_t *perm, cudaStream_t st, double *out);
void noah_release(NoahInstance &n);

// Optional per-kernel CUDA-event timing of the right-hand-side launches.
struct Profiler {
  static constexpr int kKernels = 8;
  struct Rec { int kernel; cudaEvent_t a, b; };
  Rec *recs = nullptr;
  int nrec = 0, cap = 0;
  cudaEvent_t *pool = nullptr;
  int npool = 0, used = 0;
  double ms[kKernels] = {0};
  long long calls[kKernels] = {0};
};

enum KernelId { K_PREP = 0, K_GRAD, K_MAIN, K_RIVER, K_FINISH, K_EDGE, K_PERMUTE };

// A second stream on which the river kernel of an evaluation runs beside the
// element kernels (it needs only k_elem_prep's outputs), joined before
// k_finish.  Null members: everything on one stream.
struct RhsStreams {
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};

// The river kernel's stream and events.  The stream has the highest
// priority the device offers, so that the few, long-running river blocks are
// dispatched ahead of the element kernels' many short ones and finish under
// them instead of after them.
inline cudaError_t create_rhs_streams(RhsStreams *s) {
  int least = 0, greatest = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->side, cudaStreamNonBlocking, greatest);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming);
  return e;
}

// y_ref, iperm (host-buffer evaluation of a single watershed): the state in
// reference order, read by k_elem_prep, which fills y (internal order) from it.
cudaError_t launch_rhs(const DevMesh &m, const double *y, double *ydot, cudaStream_t st,
                       long long *launches, Profiler *prof, const RhsStreams *side = nullptr,
                       const double *y_ref = nullptr, const int32_t *iperm = nullptr);

}  // namespace pihm

struct pihm_gpu_ctx {
  pihm::DevMesh m;
  int32_t ne, nr;
  int64_t neq;
  cudaStream_t stream;
  // device allocations
  void *d_static;  // one block for every static plane
  size_t static_bytes;
  void *d_dyn;     // inputs + scratch
  size_t dyn_bytes;
  double *d_stage_in, *d_stage_out;   // host-path staging [neq]
  // Copy path of the host-buffer evaluation: two staging pairs of its own,
  // so the next evaluation's state can arrive while this one's kernels run,
  // and one stream per copy direction, so a copy never waits behind a kernel
  // it does not depend on (created on the first copy-path evaluation).
  struct CopyPath {
    double *in[2] = {nullptr, nullptr}, *out[2] = {nullptr, nullptr};
    void *staging = nullptr;  // allocation holding both pairs
    cudaStream_t h2d = nullptr, d2h = nullptr;
    cudaEvent_t arrived[2] = {nullptr, nullptr}, done[2] = {nullptr, nullptr}, freed[2] = {nullptr, nullptr};
    int slot = 0;
    bool ready = false;
  } cp;
  int32_t *d_perm;                    // internal -> reference element index
  int32_t *d_iperm;                   // reference -> internal element index
  int host_pageable;                  // the device can access pageable host memory
  int host_path;                      // 0 direct where possible, 1 always copy
  int last_direct;                    // the last rhs_host accessed host memory directly
  int32_t *h_perm, *h_iperm;          // host copies (perm, inverse)
  int diag;
  int nan_check_deferred;  // 1: pihm_gpu_ode does not synchronise to read the error word
  long long launches;      // kernels launched by this context so far
  pihm::Profiler *prof;    // non-null while profiling is on
  void *d_noah;            // Flux-PIHM input planes, allocated on first use
  pihm::LandInstance land;  // land-surface model (pihm_gpu_land_init); alloc null when absent
  pihm::RhsStreams side;   // river kernel beside the element kernels
  pihm::NoahInstance noahlsm;   // Noah land-surface model (pihm_gpu_noah_init); alloc null when absent
};
