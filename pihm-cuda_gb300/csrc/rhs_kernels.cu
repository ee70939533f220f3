// FP64 right-hand-side kernels of the PIHM hydrologic model for sm_103a.
//
// One evaluation of f(t, y) (the reference ODE(), src/ode.c:4-399) runs as
// seven launches with no host synchronisation, the two river kernels on a
// second stream beside k_elem_grad/k_edge/k_elem_main (k_edge is listed at
// its definition: each interior edge is evaluated once and read with a sign
// by both elements).  GB300 issues ~2 FP64 lanes per clock per SM, so the
// FP64 pipe is the scarce one: the element rows' powers, divisions and
// square roots run in fixed point on the integer pipe (int_math.cuh; the
// divisions and roots IEEE-exact), comparisons and sign flips on the
// integer pipe too (fp64_cmp.h), divisions by static quantities are
// multiplications by reciprocals computed at load, sub-expressions the
// reference re-evaluates (EffKh per edge side, KrFunc/Psi in Infil and
// Recharge) are computed once, and each block ranks its elements by branch
// class so that a warp's lanes share their branches.
//
//   k_elem_prep   per element: clamp y (src/ode.c:25-49), SurfH
//                 (src/hydrol.c:100-134), surface head zmax + surfh and the
//                 macropore-weighted conductivity EffKh(gw)
//                 (src/lat_flow.c:248-277), each computed once per element
//                 instead of once per edge side as in the reference.
//   k_elem_grad   per element: FrictSlope/DhByDl water-surface gradient
//                 (src/lat_flow.c:130-185,239-246) reduced to its magnitude,
//                 with the purely geometric denominators precomputed.
//   k_elem_main   per element: edge fluxes (SubFlowElemToElem,
//                 OvlFlowElemToElem, BoundFluxElem, src/lat_flow.c:285-382),
//                 EtExtract (src/hydrol.c:33-97), Infil/Recharge/EffKinf/AvgKv
//                 (src/vert_flow.c:33-270) and the element rows of ydot
//                 (src/ode.c:111-209).  Elements with river edges hand their
//                 partial sums to k_finish, because their river-edge fluxes are
//                 written by the river kernel of the same evaluation.
//   k_riv_geom    per segment: channel area and wetted perimeter at the
//                 stage (src/river_flow.c:520-583), once per segment.
//   k_river       per segment: RiverFlow (src/river_flow.c:3-94) and
//                 RiverToElem (:113-183), ChanLeak, OutletFlux, BoundFluxRiver.
//   k_finish      per segment: upstream accumulation in reference order
//                 (src/river_flow.c:96-110, a CSR list instead of a serial
//                 loop) and the river rows of ydot (src/ode.c:228-300); per
//                 river-bank element: the rest of its element rows.
//
// Infil reads the river-edge overland flux of the previous evaluation
// (src/vert_flow.c:61 runs before src/river_flow.c:159-182 rewrites it); that
// value is the previous evaluation's LEFT/RIGHT_SURF2CHANL, which k_finish
// copies to carry_ovl, so k_elem_main can read it while this evaluation's
// k_river runs.
#include <cmath>

#include "fp64_math.cuh"
#include "pihm_internal.h"

namespace pihm {

#define RESTRICT __restrict__

// Comparisons go through fp64_cmp.h: the same results as the C operators,
// evaluated on the integer pipe instead of the FP64 pipe.
__device__ __forceinline__ double clamp0(double v) { return cmp::ge0(v) ? v : 0.0; }

// AvgH, src/lat_flow.c:217-237
__device__ __forceinline__ double avg_h_sub(double diff, double hsub, double hnabr) {
  if (cmp::gt0(diff)) return cmp::gt0(hsub) ? hsub : 0.0;
  return cmp::gt0(hnabr) ? hnabr : 0.0;
}

// AvgHsurf, src/lat_flow.c:187-215
__device__ __forceinline__ double avg_h_surf(double diff, double hsurf, double hnabr) {
  if (cmp::gt0(diff)) return cmp::gt_c(hsurf, kDeprStg) ? 1.0 * (hsurf - kDeprStg) : 0.0;
  return cmp::gt_c(hnabr, kDeprStg) ? 1.0 * (hnabr - kDeprStg) : 0.0;
}

// OverLandFlow, src/lat_flow.c:279-283
__device__ __forceinline__ double overland_flow(double avg_h, double grad_h, double avg_sf,
                                                double crossa, double avg_rough) {
  return crossa * pow_manning(avg_h, kManningSurf) * grad_h /
         (sqrt(avg_sf) * avg_rough);
}

// KrFunc (src/soil.c:8-13) and Psi (src/vert_flow.c:272-278) of one
// saturation in [SATMIN, 1], in the reference's own operations:
//   KrFunc = sqrt(satn) (1 - (1 - satn^m)^e) (1 - (1 - satn^m)^e),
//   Psi    = -((1 / satn)^m - 1)^ib / alpha,
// m = beta/(beta - 1), e = (beta - 1)/beta, ib = 1/beta formed at load as
// the reference forms them.  Recharge's head gradient 0.5 deficit + Psi and
// Infil's surfh + zmax - (Psi + zmax - 0.5 dinf) cancel by up to four
// orders of magnitude near equilibrium, so Psi has to carry the reference's
// roundings: each power is correctly rounded but for a rare last bit
// (pow_any), and 1/satn and the division by alpha are IEEE divisions as in
// the reference.  The powers run on the integer pipe.
// sq returns sqrt(satn), which EffKinf's macropore branch needs too.
// satn^m and (1/satn)^m share satn's logarithm: the second is the power of
// the rounded reciprocal fl(1/satn), whose logarithm follows from satn's and
// the exact residual of the division (im::log2k_recip), within the same
// 0.502 ulp as a power of its own.
__device__ __forceinline__ void kr_psi(double satn, double vm, double vg_e, double vg_ib, double alpha,
                                       double &satkfunc, double &psi, double &sq) {
  sq = sqrt_any(satn);
  const double q = div_any(1.0, satn);
  double pm, qm;  // satn^m, (1/satn)^m
  int k, kq;
  int64_t w, wq;
  im::TVal t1, t3;
  if (im::log2k(satn, k, w) && im::mul_t(vm, k, w, t1) && im::log2k_recip(satn, q, k, w, kq, wq) &&
      im::mul_t(vm, kq, wq, t3)) {
    pm = im::exp2k(t1);
    qm = im::exp2k(t3);
  } else {
    pm = pow_any(satn, vm);
    qm = pow_any(q, vm);
  }
  const double t = 1.0 - pow_any(1.0 - pm, vg_e);
  satkfunc = sq * t * t;
  psi = cmp::neg_if(div_any(pow_any(qm - 1.0, vg_ib), alpha), true);
}

// Batch engine: whether the watershed of item idx sits out this evaluation
// (a free arena slot, or a watershed that did not ask for one).  Always false
// in a single-watershed context.
__device__ __forceinline__ bool skip_item(const DevMesh &m, const int32_t *sys_of, int idx, int *sy) {
  *sy = 0;
  if (!m.active) return false;
  const int s = sys_of[idx];
  *sy = s;
  return s < 0 || !m.active[s];
}

__device__ __forceinline__ void report_err(const DevMesh &m, int sy) {
  atomicOr(m.err_sys ? &m.err_sys[sy] : m.err, 1u);
}

// Slot of the calling thread in a block's shared-memory work queue when take
// is true (one shared atomic per warp); every thread of the warp calls it.
// Queued work is evaluated densely after a barrier, so a few lanes that need
// an expensive branch do not hold a whole warp on the FP64 pipe.
__device__ __forceinline__ int queue_slot(int *count, bool take) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned mask = __ballot_sync(0xffffffffu, take);
  int base = 0;
  if (lane == 0 && mask) base = atomicAdd(count, __popc(mask));
  base = __shfl_sync(0xffffffffu, base, 0);
  return base + __popc(mask & ((1u << lane) - 1u));
}

// ---------------------------------------------------------------------------
// k_elem_prep.  Thin surface films (SurfH's square root, about half the
// elements) and water tables inside the macropore zone (EffKh's division,
// about a third) are spread over every warp, so both are queued and
// evaluated densely.
// ---------------------------------------------------------------------------
constexpr int kPrepBlock = 256;

//
// kFromRef: the host-buffer evaluation, where the state arrives in reference
// order in memory the device reads over the host link.  Thread r then takes
// reference element r (the link read is contiguous), stores its three values
// at the element's internal position in y_int and prepares that element; the
// threads past the elements copy the river values.  This replaces a separate
// reordering pass, and the preparation runs under the transfer.
template <bool kFromRef>
__global__ void __launch_bounds__(kPrepBlock) k_elem_prep(DevMesh m, const double *RESTRICT y,
                                                          const double *RESTRICT y_ref, double *RESTRICT y_int,
                                                          const int32_t *RESTRICT iperm) {
  __shared__ int qs_i[kPrepBlock], qd_i[kPrepBlock];
  __shared__ double qs_x[kPrepBlock], qd_num[kPrepBlock], qd_den[kPrepBlock];
  __shared__ int qs_n, qd_n;
  if (threadIdx.x == 0) {
    qs_n = 0;
    qd_n = 0;
  }
  __syncthreads();
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  int i = t0;
  double y_surf = 0.0, y_gw = 0.0;
  bool elem;
  int sy = 0;
  if (kFromRef) {
    const int ne = m.ne;
    elem = t0 < ne;
    if (elem) {
      i = iperm[t0];
      y_surf = y_ref[t0];
      const double u = y_ref[ne + t0];
      y_gw = y_ref[2 * ne + t0];
      y_int[i] = y_surf;
      y_int[ne + i] = u;
      y_int[2 * ne + i] = y_gw;
    } else if (t0 < ne + 2 * m.nr) {
      y_int[2 * ne + t0] = y_ref[2 * ne + t0];  // stage and river gw, same order
    }
  } else {
    elem = i < m.ne_run && !skip_item(m, m.sys_elem, i, &sy);
    if (elem) {
      y_surf = y[i];
      y_gw = y[2 * m.ne + i];
    }
  }
  bool thin = false, mix = false;
  double sx = 0.0, num = 0.0, den = 0.0;
  if (elem) {
    // SurfH, src/hydrol.c:100-134
    const double surfeqv = clamp0(y_surf);
    if (cmp::lt0(surfeqv)) {
      m.surfh[i] = 0.0;
      m.head[i] = 0.0 + m.zmax[i];
    } else if (cmp::le_c(surfeqv, 0.5 * kDeprStg)) {
      thin = true;
      sx = 2.0 * kDeprStg * surfeqv;
    } else {
      const double sh = kDeprStg + (surfeqv - 0.5 * kDeprStg);
      m.surfh[i] = sh;
      m.head[i] = sh + m.zmax[i];
    }
    // EffKh, src/lat_flow.c:248-277, with k1 = kmach*areafv + ksath*(1-areafv)
    // and depth - dmac formed at load (the reference evaluates both inline
    // with the same operations)
    double gw = clamp0(y_gw);
    gw = cmp::gt0(gw) ? gw : 0.0;
    const double d_dmac = m.d_dmac[i];
    if (cmp::gt_v(gw, d_dmac)) {
      const double d1 = cmp::gt_v(gw, m.depth[i]) ? m.dmac[i] : gw - d_dmac;
      num = m.kh_k1[i] * d1 + m.ksath[i] * d_dmac;
      den = d1 + d_dmac;
      mix = true;
    } else {
      m.effk[i] = m.ksath[i];
    }
  }
  const int ss = queue_slot(&qs_n, thin);
  if (thin) {
    qs_i[ss] = i;
    qs_x[ss] = sx;
  }
  const int sd = queue_slot(&qd_n, mix);
  if (mix) {
    qd_i[sd] = i;
    qd_num[sd] = num;
    qd_den[sd] = den;
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t < qs_n) {
    const int e = qs_i[t];
    const double sh = sqrt_any(qs_x[t]);
    m.surfh[e] = sh;
    m.head[e] = sh + m.zmax[e];
  }
  if (t < qd_n) m.effk[qd_i[t]] = div_any(qd_num[t], qd_den[t]);
}

// ---------------------------------------------------------------------------
// k_elem_grad
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_elem_grad(DevMesh m, const double *RESTRICT y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int sy;
  if (i >= m.ne_run || skip_item(m, m.sys_elem, i, &sy)) return;
  const int ne = m.ne;
  double h[3];
  const double hself = m.head[i];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int32_t nb = m.nb[j * ne + i];
    if (nb >= 0) {
      h[j] = m.head[nb];
    } else if (nb != kBoundary) {
      const int s = -1 - nb;
      const double stage = clamp0(y[3 * ne + s]);
      h[j] = cmp::gt_v(stage, m.r_depth[s]) ? m.r_zbed[s] + stage : m.r_zmax[s];
    } else {
      h[j] = (m.bctype[j * ne + i] == 0) ? hself : m.elem_bc[j * ne + i];
    }
  }
  const double y0 = m.nabr_y[i], y1 = m.nabr_y[ne + i], y2 = m.nabr_y[2 * ne + i];
  const double x0 = m.nabr_x[i], x1 = m.nabr_x[ne + i], x2 = m.nabr_x[2 * ne + i];
  // DhByDl(nabr_y, nabr_x, h) and DhByDl(nabr_x, nabr_y, h)
  const double dhdx = -1.0 * (y2 * (h[1] - h[0]) + y1 * (h[0] - h[2]) + y0 * (h[2] - h[1])) * m.inv_den_x[i];
  const double dhdy = -1.0 * (x2 * (h[1] - h[0]) + x1 * (h[0] - h[2]) + x0 * (h[2] - h[1])) * m.inv_den_y[i];
  m.gradmag[i] = sqrt_any(dhdx * dhdx + dhdy * dhdy);
}

// ---------------------------------------------------------------------------
// k_edge: one thread per interior edge.  SubFlowElemToElem and
// OvlFlowElemToElem (src/lat_flow.c:285-338) are antisymmetric in IEEE
// arithmetic under the diffusion wave (negated head difference, commutative
// averages, the same distance and edge length on both sides, which the host
// checks bit for bit), so the owner evaluates each edge once and the
// neighbour reads the negated value.  Kinematic overland flow is not
// antisymmetric (avg_sf depends on the sign of the gradient): there every
// element side is its own one-sided edge.
//
// The Manning flux costs about 35 FP64 operations and only edges whose
// upwind element holds water above the depression storage have one (about
// half of them, spread over nearly every warp).  So each thread computes its
// Darcy flux and the Manning flux's inputs, the edges with water are queued
// in shared memory (warp-aggregated slots), and after one barrier the block
// evaluates the queue densely: ceil(n/32) warps instead of all eight carry
// the powers.  Each flux depends on its edge alone, so which thread computes
// it changes no bit.
// ---------------------------------------------------------------------------
constexpr int kEdgeBlock = 256;

__global__ void __launch_bounds__(kEdgeBlock) k_edge(DevMesh m, const double *RESTRICT y) {
  __shared__ int q_e[kEdgeBlock];
  __shared__ double q_h[kEdgeBlock], q_d[kEdgeBlock], q_sf[kEdgeBlock];
  __shared__ int q_n;
  if (threadIdx.x == 0) q_n = 0;
  __syncthreads();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  int sy;
  bool wet = false;
  double avg_h = 0.0, diff_h = 0.0, avg_sf = 0.0;
  if (e < m.nedge_run && !skip_item(m, m.sys_edge, e, &sy)) {
    const int ne = m.ne;
    const int i = m.e_i[e], k = m.e_k[e];
    // Darcy flux between the two groundwater columns,
    // avg_ksat grad_h avg_h edge = (effk_i + effk_k) diff_h avg_h edge/(2 dist)
    const double gw_i = clamp0(y[2 * ne + i]), gw_k = clamp0(y[2 * ne + k]);
    diff_h = (gw_i + m.zmin[i]) - (gw_k + m.zmin[k]);
    avg_h = avg_h_sub(diff_h, gw_i, gw_k);
    m.eflux_sub[e] = (m.effk[i] + m.effk[k]) * diff_h * avg_h * m.e_subk[e];
    // Manning overland flux, crossa h^p grad_h / (sqrt(avg_sf) avg_rough) =
    // avg_h h^p diff_h / sqrt(avg_sf) edge/(dist avg_rough)
    const double s_i = m.surfh[i], s_k = m.surfh[k];
    if (m.surf_mode == kKinematic) {
      diff_h = m.zmax[i] - m.zmax[k];
      avg_h = avg_h_surf(diff_h, s_i, s_k);
      const double grad_h = diff_h * m.e_invdist[e];
      avg_sf = cmp::gt0(grad_h) ? grad_h : kGradMin;
    } else {
      diff_h = m.head[i] - m.head[k];
      avg_h = avg_h_surf(diff_h, s_i, s_k);
      avg_sf = 0.5 * (m.gradmag[i] + m.gradmag[k]);
      avg_sf = cmp::gt_c(avg_sf, kGradMin) ? avg_sf : kGradMin;
    }
    // avg_h == 0 gives crossa == 0: the flux is zero
    wet = cmp::gt0(avg_h);
    if (!wet) m.eflux_ovl[e] = 0.0;
  }
  const int slot = queue_slot(&q_n, wet);
  if (wet) {
    q_e[slot] = e;
    q_h[slot] = avg_h;
    q_d[slot] = diff_h;
    q_sf[slot] = avg_sf;
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t < q_n) {
    const int qe = q_e[t];
    const double h = q_h[t];
    m.eflux_ovl[qe] = h * pow_manning(h, kManningSurf) * q_d[t] * rsqrt(q_sf[t]) *
                      m.e_ovlk[qe];
  }
}

// ---------------------------------------------------------------------------
// k_elem_main
// ---------------------------------------------------------------------------
// Block shapes: the same 64-register budget (1,024 resident threads per
// SM) cut into 512 x 2, 256 x 4 or 128 x 8 blocks.  With the elements
// ranked by branch class per block, 256 x 4 is fastest on large meshes (92
// against 102 and 97 us per 400k elements): larger blocks group more
// elements of a class but gather their loads from a wider window.  On a
// small mesh or a sparsely occupied batch arena the smaller blocks spread
// the work over more SMs.  The batch engine tunes the shape per arena.
//
// Branch classes: a block first sorts its elements by the branches the
// element rows take -- water table within the infiltration depth (no
// Psi/KrFunc, Recharge = Infil), ponded surface (EffKinf's second case),
// unsaturated zone deeper than the macropores (AvgKv's first case) -- so
// that a warp's lanes mostly take the same ones, and each thread then
// evaluates the element at its rank.  The classes only group; every element
// is evaluated by the same code whatever its class, so the results do not
// depend on the grouping.  Items that sit out (past the end, or a batch
// watershed without an evaluation) sort last and leave as whole warps.
constexpr int kElemClasses = 8;

__device__ __forceinline__ int elem_class(const DevMesh &m, const double *RESTRICT y, int i) {
  const int ne = m.ne;
  const double gw = clamp0(y[2 * ne + i]);
  const int ponded = cmp::gt_c(m.surfh[i], kDeprStg) ? 1 : 0;
  if (cmp::gt_v(gw, m.d_dinf[i])) return 4 + ponded;
  return 2 * ponded + (cmp::lt_v(gw, m.d_dmac[i]) ? 1 : 0);
}

template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) k_elem_main(DevMesh m, const double *RESTRICT y,
                                                    double *RESTRICT ydot) {
  // a stable ranking: class-major, then warp, then lane, so each class keeps
  // the block's element order and a warp's elements lie close together
  constexpr int kWarps = BLOCK / 32, kSlots = kElemClasses * kWarps;
  __shared__ int s_off[kSlots];  // [class][warp]: count, then exclusive offset
  __shared__ unsigned short s_order[BLOCK];
  {
    const int i0 = blockIdx.x * BLOCK + threadIdx.x;
    int sy0;
    const int cls = (i0 >= m.ne_run || skip_item(m, m.sys_elem, i0, &sy0)) ? kElemClasses - 1
                                                                          : elem_class(m, y, i0);
    for (int k = threadIdx.x; k < kSlots; k += BLOCK) s_off[k] = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const int warp = threadIdx.x >> 5;
    const unsigned peers = __match_any_sync(0xffffffffu, cls);
    if ((int)lane == __ffs(peers) - 1) s_off[cls * kWarps + warp] = __popc(peers);
    __syncthreads();
    if (warp == 0) {
      // exclusive scan of the kSlots counts: each lane sums its run of
      // consecutive slots, the lanes scan their sums, then write back
      constexpr int kRun = (kSlots + 31) / 32;
      int run[kRun], sum = 0;
#pragma unroll
      for (int r = 0; r < kRun; r++) {
        const int k = (int)lane * kRun + r;
        run[r] = k < kSlots ? s_off[k] : 0;
        sum += run[r];
      }
      int incl = sum;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, d);
        if ((int)lane >= d) incl += v;
      }
      int off = incl - sum;
#pragma unroll
      for (int r = 0; r < kRun; r++) {
        const int k = (int)lane * kRun + r;
        if (k < kSlots) s_off[k] = off;
        off += run[r];
      }
    }
    __syncthreads();
    s_order[s_off[cls * kWarps + warp] + __popc(peers & ((1u << lane) - 1u))] = (unsigned short)threadIdx.x;
    __syncthreads();
  }
  const int i = blockIdx.x * BLOCK + s_order[threadIdx.x];
  int sy;
  if (i >= m.ne_run || skip_item(m, m.sys_elem, i, &sy)) return;
  const int ne = m.ne;
  const double gw = clamp0(y[2 * ne + i]);
  const double unsat = clamp0(y[ne + i]);
  const double surfh = m.surfh[i];
  const double zmin = m.zmin[i];
  const double inv_area = m.inv_area[i];
  const double gwhead = gw + zmin;

  double ovl[3], sub[3];
  bool riv[3];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int32_t code = m.emap[j * ne + i];
    riv[j] = false;
    if (code != 0) {
      // the edge's flux with the sign seen from this element (a negative
      // code: the flux was computed from the neighbour's side)
      const int e = (code > 0 ? code : -code) - 1;
      ovl[j] = cmp::neg_if(m.eflux_ovl[e], code < 0);
      sub[j] = cmp::neg_if(m.eflux_sub[e], code < 0);
    } else {
      const int32_t nb = m.nb[j * ne + i];
      if (nb != kBoundary) {
        // river edge: Infil sees the previous evaluation's value
        const int s = -1 - nb;
        ovl[j] = -m.carry_ovl[(m.left[s] == i ? 0 : 1) * m.nr + s];
        sub[j] = 0.0;
        riv[j] = true;
      } else {
        // BoundFluxElem, src/lat_flow.c:340-382
        const int bct = m.bctype[j * ne + i];
        ovl[j] = 0.0;
        if (bct == 0) {
          sub[j] = 0.0;
        } else if (bct > 0) {
          const double bc = m.elem_bc[j * ne + i];
          const double diff_h = gwhead - bc;
          const double avg_h = avg_h_sub(diff_h, gw, bc - zmin);
          const double grad_h = diff_h / m.nabrdist[j * ne + i];
          sub[j] = m.effk[i] * grad_h * avg_h * m.edge[j * ne + i];
        } else {
          sub[j] = -m.elem_bc[j * ne + i];
        }
      }
    }
  }

  // EtExtract, src/hydrol.c:33-97
  const double depth = m.depth[i];
  const double d_dinf = m.d_dinf[i];
  const double edir = m.edir[i], ett = m.ett[i];
  double edir_surf = 0.0, edir_unsat = 0.0, edir_gw = 0.0, ett_unsat = 0.0, ett_gw = 0.0;
  const bool gw_in_dinf = cmp::gt_v(gw, d_dinf);
  const bool noah = m.noah && (!m.sys_noah || m.sys_noah[sy]);
  if (noah) {
    // Flux-PIHM (src/hydrol.c:43-55,79-83): no ponded-water source, and the
    // transpiration split by GwTransp (noah/lsm_func.c:163-185) over the
    // Noah layers from the water table down to the root depth
    if (gw_in_dinf) edir_gw = edir;
    else edir_unsat = edir;
    double gwet = 0.0;
    if (cmp::gt0(ett) && m.noah_wtin[i]) {
      gwet = div_any(m.noah_etgw[i], ett);
      gwet = cmp::gt_c(gwet, 1.0) ? 1.0 : gwet;
      gwet = cmp::lt0(gwet) ? 0.0 : gwet;
    }
    ett_unsat = (1.0 - gwet) * ett;
    ett_gw = gwet * ett;
  } else {
    if (cmp::ge_c(surfh, kDeprStg)) edir_surf = edir;
    else if (gw_in_dinf) edir_gw = edir;
    else edir_unsat = edir;
    if (cmp::gt_v(gw, m.d_rzd[i])) ett_gw = ett;
    else ett_unsat = ett;
  }

  // Infil, src/vert_flow.c:33-130, and Recharge, :132-170, sharing KrFunc and
  // Psi of the same saturation
  const double kinf_mat = m.kinf_mat[i], kmac_a = m.kmac_a[i], areafh = m.areafh[i];
  const double kinfv = m.kinfv[i], ksatv = m.ksatv[i], dmac = m.dmac[i];
  const double pcpdrp = m.pcpdrp[i];
  const double zmax = m.zmax[i];
  const double dinf = m.dinf[i];
  double satn = 1.0, satkfunc = 1.0, psi_u = 0.0, sq = 1.0;
  if (!gw_in_dinf) {
    const double deficit = depth - gw;
    satn = div_any(unsat, deficit);
    satn = cmp::gt_c(satn, 1.0) ? 1.0 : satn;
    satn = cmp::lt_c(satn, kSatMin) ? kSatMin : satn;
    kr_psi(satn, m.vg_m[i], m.vg_e[i], m.vg_ib[i], m.alpha[i], satkfunc, psi_u, sq);
  }
  // Infil's saturation: the same one, except in Flux-PIHM, where it is
  // Noah's top-layer moisture (src/vert_flow.c:94-98) and Recharge keeps
  // the column's
  double satn_i = satn, satkfunc_i = satkfunc, psi_i = psi_u, sq_i = sq;
  if (noah && !gw_in_dinf) {
    double s = m.noah_satn[i];
    s = cmp::gt_c(s, 1.0) ? 1.0 : s;
    s = cmp::lt_c(s, kSatMin) ? kSatMin : s;
    satn_i = s;
    kr_psi(s, m.vg_m[i], m.vg_e[i], m.vg_ib[i], m.alpha[i], satkfunc_i, psi_i, sq_i);
  }
  // KrFunc(beta, 1) == 1 exactly: pow(1 - pow(1, m), e) == pow(0, e) == 0
  double infil;
  if (cmp::gt_v(unsat + gw, depth)) {
    infil = 0.0;
  } else {
    double applrate = 0.0;
#pragma unroll
    for (int j = 0; j < 3; j++) applrate += -ovl[j] * inv_area;
    applrate = cmp::gt0(applrate) ? applrate : 0.0;
    applrate += pcpdrp;
    double wetfrac = surfh * (1.0 / kDeprStg);
    wetfrac = cmp::gt0(wetfrac) ? wetfrac : 0.0;
    wetfrac = cmp::lt_c(wetfrac, 1.0) ? wetfrac : 1.0;
    // the head below the infiltration front: the water table when it lies
    // within dinf of the surface, else the unsaturated zone's; both
    // reference branches divide (surfh + zmax - head) by the same
    // denominator, so one division serves a warp whose lanes take both
    double h_u = gwhead;
    double esatn = 1.0;
    if (!gw_in_dinf) {
      const double psi_c = cmp::gt_nc(psi_i, kPsiMin) ? psi_i : kPsiMin;
      h_u = psi_c + zmax - 0.5 * dinf;
      esatn = satn_i;
    }
    double dh_by_dz = div_any(surfh + zmax - h_u, 0.5 * (surfh + dinf));
    dh_by_dz = (cmp::le0(surfh) && cmp::gt0(dh_by_dz)) ? 0.0 : dh_by_dz;
    // EffKinf, src/vert_flow.c:211-270
    double kinf;
    if (cmp::eq0(areafh)) {
      kinf = kinfv * satkfunc_i;
    } else if (cmp::gt_c(surfh, kDeprStg)) {
      kinf = kinf_mat * satkfunc_i + kmac_a;
    } else if (cmp::le_v(applrate, dh_by_dz * kinfv * satkfunc_i)) {
      kinf = kinfv * satkfunc_i;
    } else if (cmp::lt_v(applrate, dh_by_dz * (kmac_a + kinf_mat * satkfunc_i))) {
      // KrFunc(2, satn): pow(satn, 2) and pow(., 0.5) are a product and
      // sqrt; sqrt(esatn) is kr_psi's (1 when esatn is 1)
      const double t2 = 1.0 - sqrt_any(1.0 - esatn * esatn);
      kinf = kinf_mat * satkfunc_i + kmac_a * (sq_i * t2 * t2);
    } else {
      kinf = kinf_mat * satkfunc_i + kmac_a;
    }
    infil = kinf * dh_by_dz;
    if (!gw_in_dinf) infil = cmp::gt0(infil) ? infil : 0.0;
    const double ws0 = m.ws0_surf[i];
    const double inv_dt = m.sys_inv_dt ? m.sys_inv_dt[sy] : m.inv_dt;
    const double infil_max = applrate + (cmp::gt0(ws0) ? ws0 * inv_dt : 0.0);
    infil = cmp::gt_v(infil, infil_max) ? infil_max : infil;
    infil *= wetfrac;
  }
  if (noah) infil *= m.noah_fcr[i];  // frozen top soil, src/vert_flow.c:16-19
  double rechg;
  if (gw_in_dinf) {
    rechg = infil;
  } else {
    const double deficit = depth - gw;
    // the denominators of Recharge add up to depth: (deficit + gw) and the
    // AvgKv weights d1 + d2 + d3 (to an ulp); multiply by 1/depth instead
    const double inv_depth = m.inv_depth[i];
    const double dh_by_dz = (0.5 * deficit + psi_u) * (2.0 * inv_depth);
    // AvgKv, src/vert_flow.c:172-209, arithmetic mean (_ARITH_ is defined at
    // src/include/pihm_func.h:4)
    double k1, k2, k3, d1, d2, d3;
    if (cmp::gt_v(deficit, dmac)) {
      k1 = satkfunc * ksatv;
      d1 = dmac;
      k2 = satkfunc * ksatv;
      d2 = deficit - dmac;
      k3 = ksatv;
      d3 = gw;
    } else {
      k1 = satkfunc * ksatv;
      d1 = deficit;
      k2 = m.kv2_mac[i];
      d2 = dmac - deficit;
      k3 = ksatv;
      d3 = gw - (dmac - deficit);
    }
    const double kavg = (k1 * d1 + k2 * d2 + k3 * d3) * inv_depth;
    rechg = kavg * dh_by_dz;
    rechg = (cmp::gt0(rechg) && cmp::le0(unsat)) ? 0.0 : rechg;
    rechg = (cmp::lt0(rechg) && cmp::le0(gw)) ? 0.0 : rechg;
  }

  if (m.diag) {
#pragma unroll
    for (int j = 0; j < 3; j++) {
      if (!riv[j]) {
        m.d_ovl[j * ne + i] = ovl[j];
        m.d_sub[j * ne + i] = sub[j];
      }
    }
    m.d_infil[i] = infil;
    m.d_rechg[i] = rechg;
    m.d_et[i] = edir_surf;
    m.d_et[ne + i] = edir_unsat;
    m.d_et[2 * ne + i] = edir_gw;
    m.d_et[3 * ne + i] = ett_unsat;
    m.d_et[4 * ne + i] = ett_gw;
  }

  // element rows of ydot, src/ode.c:111-209
  const double inv_por = m.inv_por[i];
  const double base_surf = pcpdrp - infil - edir_surf;
  const double base_gw = rechg - edir_gw - ett_gw;
  const double du = (infil - rechg - edir_unsat - ett_unsat) * inv_por;
  ydot[ne + i] = du;
  unsigned int bad = cmp::isnan_(du);
  if (riv[0] || riv[1] || riv[2]) {
    const int b = m.bank_slot[i];
    const int nbk = m.nbank;
    double *bp = m.bank_part;
    bp[b] = base_surf;
    bp[nbk + b] = base_gw;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      bp[(2 + j) * nbk + b] = ovl[j];
      bp[(5 + j) * nbk + b] = sub[j];
    }
  } else {
    double ds = base_surf, dg = base_gw;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      ds -= ovl[j] * inv_area;
      dg -= sub[j] * inv_area;
    }
    dg *= inv_por;
    ydot[i] = ds;
    ydot[2 * ne + i] = dg;
    bad |= cmp::isnan_(ds) | cmp::isnan_(dg);
  }
  if (bad) report_err(m, sy);
}

// ---------------------------------------------------------------------------
// k_riv_geom: wetted perimeter and cross-section area of every segment at its
// stage (RivPerim / RivCsArea, src/river_flow.c:520-583), once per segment
// and evaluation (k_river needs them for the segment and for its downstream
// neighbour), with the coefficient-only factors formed at load (r_geo*, in
// the order the shape's formula uses them):
//   rectangle  area d c,           perimeter 2 d + c
//   triangle   area d^2 / c,       perimeter 2 d sqrt(1 + c^2) / c
//   quadratic  area 4 d^1.5 / (3 sqrt c),
//              perimeter sqrt(d (1 + 4 c d) / c) + ln(2 sqrt(c d) + sqrt(1 + 4 c d)) / (2 c)
//   cubic      area 3 d^(4/3) / (2 c^(1/3)),
//              perimeter 2 (sqrt(d (1 + 9 c^(2/3) d)) / 3
//                           + ln(3 c^(1/3) sqrt(d) + sqrt(1 + 9 c^(2/3) d)) / (9 c^(1/3)))
// The reference's pow(x, 0.5) is sqrt(x).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double log_of(double x) {
  double sh, lo;
  return log_dd_fast(x, sh, lo) ? sh + lo : log(x);
}

__global__ void __launch_bounds__(128) k_riv_geom(DevMesh m, const double *RESTRICT y) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  int sy;
  if (s >= m.nr_run || skip_item(m, m.sys_riv, s, &sy)) return;
  double d = y[3 * m.ne + s];
  d = cmp::gt0(d) ? d : 0.0;
  const double g0 = m.r_geo0[s];
  double area = 0.0, perim = 0.0;
  switch (m.intrpl_ord[s]) {
    case kRectangle:
      area = d * g0;
      perim = 2.0 * d + g0;
      break;
    case kTriangle:
      area = d * d * g0;
      perim = d * m.r_geo1[s];
      break;
    case kQuadratic: {
      const double sd = sqrt(d), w = 1.0 + m.r_geo1[s] * d;
      area = g0 * d * sd;
      perim = sqrt(d * w * m.r_geo2[s]) + log_of(m.r_geo4[s] * sd + sqrt(w)) * m.r_geo3[s];
      break;
    }
    case kCubic: {
      const double sd = sqrt(d), w = 1.0 + m.r_geo1[s] * d;
      area = g0 * pow_fast(d, 4.0 / 3.0);
      perim = 2.0 * (sqrt(d * w) * (1.0 / 3.0) + log_of(m.r_geo2[s] * sd + sqrt(w)) * m.r_geo3[s]);
      break;
    }
  }
  m.r_perim[s] = perim;
  m.r_crossa[s] = area;
}

// ---------------------------------------------------------------------------
// k_river
// ---------------------------------------------------------------------------
struct RivState {
  double stage, gw, zbed, zmin, zmax, length, width, rough;
};

__device__ __forceinline__ RivState load_riv(const DevMesh &m, const double *y, int s) {
  RivState r;
  r.stage = clamp0(y[3 * m.ne + s]);
  r.gw = clamp0(y[3 * m.ne + m.nr + s]);
  r.zbed = m.r_zbed[s];
  r.zmin = m.r_zmin[s];
  r.zmax = m.r_zmax[s];
  r.length = m.r_length[s];
  r.width = m.r_width[s];
  r.rough = m.r_rough[s];
  return r;
}

// OvlFlowElemToRiver, src/river_flow.c:185-255, with the weir coefficient
// cwr 2 sqrt(2 g) length / 3 formed at load (coef)
__device__ __forceinline__ double ovl_elem_to_river(double e_zmax, double e_surfh, const RivState &r,
                                                    double coef) {
  const double zbank = cmp::gt_v(r.zmax, e_zmax) ? r.zmax : e_zmax;
  const double elem_h = e_zmax + e_surfh;
  const double rivseg_h = r.zbed + r.stage;
  if (cmp::gt_v(rivseg_h, elem_h)) {
    if (cmp::gt_v(elem_h, zbank)) return coef * sqrt(rivseg_h - elem_h) * (rivseg_h - zbank);
    if (cmp::lt_v(zbank, rivseg_h)) return coef * sqrt(rivseg_h - zbank) * (rivseg_h - zbank);
    return 0.0;
  }
  if (cmp::gt_c(e_surfh, kDeprStg)) {
    if (cmp::gt_v(rivseg_h, zbank)) return -coef * sqrt(elem_h - rivseg_h) * (elem_h - zbank);
    if (cmp::lt_v(zbank, elem_h)) return -coef * sqrt(elem_h - zbank) * (elem_h - zbank);
    return 0.0;
  }
  return 0.0;
}

// ChanFlowElemToRiver, src/river_flow.c:429-460
__device__ __forceinline__ double chan_elem_to_river(double e_gw, double e_zmin, double effk,
                                                     const RivState &r, double r_ksath,
                                                     double inv_distance) {
  const double diff_h = (r.stage + r.zbed) - (e_gw + e_zmin);
  double avg_h;
  if (cmp::gt_v(e_zmin, r.zbed)) avg_h = e_gw;
  else if (cmp::gt_v(e_zmin + e_gw, r.zbed)) avg_h = e_zmin + e_gw - r.zbed;
  else avg_h = 0.0;
  avg_h = avg_h_sub(diff_h, r.stage, avg_h);
  const double grad_h = diff_h * inv_distance;
  const double avg_ksat = 0.5 * (effk + r_ksath);
  return r.length * avg_ksat * grad_h * avg_h;
}

// SubFlowElemToRiver, src/river_flow.c:462-498 (arithmetic mean)
__device__ __forceinline__ double sub_elem_to_river(double e_gw, double e_zmin, double effk,
                                                    const RivState &r, double effk_riv,
                                                    double inv_distance) {
  const double diff_h = (r.gw + r.zmin) - (e_gw + e_zmin);
  double avg_h;
  if (cmp::gt_v(e_zmin, r.zbed)) avg_h = 0.0;
  else if (cmp::gt_v(e_zmin + e_gw, r.zbed)) avg_h = r.zbed - e_zmin;
  else avg_h = e_gw;
  avg_h = avg_h_sub(diff_h, r.gw, avg_h);
  const double avg_ksat = 0.5 * (effk + effk_riv);
  const double grad_h = diff_h * inv_distance;
  return r.length * avg_ksat * grad_h * avg_h;
}

__global__ void __launch_bounds__(128) k_river(DevMesh m, const double *RESTRICT y) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  int sy;
  if (s >= m.nr_run || skip_item(m, m.sys_riv, s, &sy)) return;
  const int nr = m.nr, ne = m.ne;
  const RivState r = load_riv(m, y, s);
  const int down = m.down[s];
  double f[NUM_RIVFLX];
  f[UP_CHANL2CHANL] = 0.0;
  f[UP_AQUIF2AQUIF] = 0.0;
  const int L = m.left[s], R = m.right[s];
  const double effk_l = m.effk[L], effk_r = m.effk[R];
  if (down > 0) {
    const int bct = m.bctype_riv[s];
    if (bct != 0) {
      // BoundFluxRiver, src/river_flow.c:392-427
      double flux = 0.0;
      const double bc = m.river_bc[s];
      if (bct > 0) {
        const double total_h = r.stage + r.zbed;
        const double grad_h = (total_h - bc) * m.r_inv_half_len[s];
        const double avg_perim = m.r_perim[s];
        const double crossa = m.r_crossa[s];
        const double avg_h = cmp::eq0(avg_perim) ? 0.0 : (crossa / avg_perim);
        flux = overland_flow(avg_h, grad_h, grad_h, crossa, r.rough);
      } else {
        flux = -bc;
      }
      f[UP_CHANL2CHANL] += flux;
    }
    const int d = down - 1;
    const RivState dn = load_riv(m, y, d);
    const double inv_dist_down = m.r_inv_dist_down[s];
    // ChanFlowRiverToRiver, src/river_flow.c:257-300
    {
      const double total_h = r.stage + r.zbed;
      const double perim = m.r_perim[s];
      const double total_h_down = dn.stage + dn.zbed;
      const double perim_down = m.r_perim[d];
      const double avg_perim = (perim + perim_down) / 2.0;
      const double avg_rough = (r.rough + dn.rough) / 2.0;
      const double diff_h = (m.riv_mode == kKinematic) ? (r.zbed - dn.zbed) : (total_h - total_h_down);
      const double grad_h = diff_h * inv_dist_down;
      const double avg_sf = cmp::gt0(grad_h) ? grad_h : kRivGradMin;
      const double crossa = m.r_crossa[s];
      const double crossa_down = m.r_crossa[d];
      const double avg_crossa = 0.5 * (crossa + crossa_down);
      const double avg_h = cmp::eq0(avg_perim) ? 0.0 : (avg_crossa / avg_perim);
      f[DOWN_CHANL2CHANL] = overland_flow(avg_h, grad_h, avg_sf, crossa, avg_rough);
    }
    // SubFlowRiverToRiver, src/river_flow.c:302-331 (arithmetic mean)
    {
      const double effk = 0.5 * (effk_l + effk_r);
      const double effk_nabr = 0.5 * (m.effk[m.left[d]] + m.effk[m.right[d]]);
      const double total_h = r.gw + r.zmin;
      const double total_h_down = dn.gw + dn.zmin;
      const double avg_wid = (r.width + dn.width) / 2.0;
      const double diff_h = total_h - total_h_down;
      const double avg_h = avg_h_sub(diff_h, r.gw, dn.gw);
      const double grad_h = diff_h * inv_dist_down;
      const double avg_ksat = 0.5 * (effk + effk_nabr);
      f[DOWN_AQUIF2AQUIF] = avg_ksat * grad_h * avg_h * avg_wid;
    }
  } else {
    // OutletFlux, src/river_flow.c:333-390
    const double depth = m.r_depth[s];
    const double bc = m.river_bc[s];
    double q = 0.0;
    if (down == kDirichlet) {
      const double total_h = r.stage + r.zbed;
      const double grad_h = (total_h - bc) * m.r_inv_half_len[s];
      const double avg_perim = m.r_perim[s];
      const double crossa = m.r_crossa[s];
      const double avg_h = cmp::eq0(avg_perim) ? 0.0 : (crossa / avg_perim);
      q = overland_flow(avg_h, grad_h, grad_h, crossa, r.rough);
    } else if (down == kNeumann) {
      q = -bc;
    } else if (down == kZeroDpthGrad) {
      const double grad_h = (r.zbed - (m.r_node_zmax[s] - depth)) * m.r_inv_half_len[s];
      const double avg_perim = m.r_perim[s];
      const double crossa = m.r_crossa[s];
      q = sqrt(grad_h) * crossa *
          (cmp::gt0(avg_perim) ? pow_manning(crossa / avg_perim, kManningRiv) : 0.0) /
          r.rough;
    } else {  // kCritDpth (other values are rejected at load)
      const double crossa = m.r_crossa[s];
      q = crossa * sqrt(kGrav * r.stage);
    }
    f[DOWN_CHANL2CHANL] = q;
    f[DOWN_AQUIF2AQUIF] = 0.0;
  }
  // RiverToElem, src/river_flow.c:113-183
  const double coef = m.r_ovl_coef[s];
  const double gw_l = clamp0(y[2 * ne + L]), gw_r = clamp0(y[2 * ne + R]);
  const double zmin_l = m.zmin[L], zmin_r = m.zmin[R];
  f[LEFT_SURF2CHANL] = ovl_elem_to_river(m.zmax[L], m.surfh[L], r, coef);
  f[RIGHT_SURF2CHANL] = ovl_elem_to_river(m.zmax[R], m.surfh[R], r, coef);
  const double r_ksath = m.r_ksath[s];
  const double inv_dl = m.r_inv_dist_left[s], inv_dr = m.r_inv_dist_right[s];
  f[LEFT_AQUIF2CHANL] = chan_elem_to_river(gw_l, zmin_l, effk_l, r, r_ksath, inv_dl);
  f[RIGHT_AQUIF2CHANL] = chan_elem_to_river(gw_r, zmin_r, effk_r, r, r_ksath, inv_dr);
  const double effk_avg = 0.5 * (effk_l + effk_r);
  f[LEFT_AQUIF2AQUIF] = sub_elem_to_river(gw_l, zmin_l, effk_l, r, effk_avg, inv_dl);
  f[RIGHT_AQUIF2AQUIF] = sub_elem_to_river(gw_r, zmin_r, effk_r, r, effk_avg, inv_dr);
  // ChanLeak, src/river_flow.c:500-518
  {
    double diff_h;
    if (cmp::gt0(r.zbed - (r.gw + r.zmin))) diff_h = r.stage;
    else diff_h = r.stage + r.zbed - (r.gw + r.zmin);
    const double grad_h = diff_h * m.r_inv_bedthick[s];
    f[CHANL_LKG] = m.r_ksatv[s] * r.width * r.length * grad_h;
  }
#pragma unroll
  for (int k = 0; k < NUM_RIVFLX; k++) m.rivflow[k * nr + s] = f[k];
}

// ---------------------------------------------------------------------------
// k_finish
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_finish(DevMesh m, double *RESTRICT ydot) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nr = m.nr, ne = m.ne;
  const double *F = m.rivflow;
  int sy;
  if (t < m.nr_run) {
    const int s = t;
    if (skip_item(m, m.sys_riv, s, &sy)) return;
    double up_c = F[UP_CHANL2CHANL * nr + s];
    double up_a = 0.0;
    for (int k = m.up_ptr[s]; k < m.up_end[s]; k++) {
      const int u = m.up_idx[k];
      up_c -= F[DOWN_CHANL2CHANL * nr + u];
      up_a -= F[DOWN_AQUIF2AQUIF * nr + u];
    }
    const double area = m.r_area[s];
    double ds = 0.0;
    ds -= up_c / area;
#pragma unroll
    for (int j = 1; j <= 6; j++) ds -= F[j * nr + s] / area;
    double dg = -F[LEFT_AQUIF2AQUIF * nr + s] - F[RIGHT_AQUIF2AQUIF * nr + s] -
                F[DOWN_AQUIF2AQUIF * nr + s] - up_a + F[CHANL_LKG * nr + s];
    dg /= m.r_porosity[s] * area;
    ydot[3 * ne + s] = ds;
    ydot[3 * ne + nr + s] = dg;
    if (m.diag) {
      m.rivflow[UP_CHANL2CHANL * nr + s] = up_c;
      m.rivflow[UP_AQUIF2AQUIF * nr + s] = up_a;
    }
    if (cmp::isnan_(ds) | cmp::isnan_(dg)) report_err(m, sy);
    // the next evaluation's Infil reads this evaluation's river-edge
    // overland flux (src/vert_flow.c:61 before src/river_flow.c:159-182)
    m.carry_ovl[s] = F[LEFT_SURF2CHANL * nr + s];
    m.carry_ovl[nr + s] = F[RIGHT_SURF2CHANL * nr + s];
    return;
  }
  const int b = t - m.nr_run;
  if (b >= m.nbank_run || skip_item(m, m.sys_bank, b, &sy)) return;
  const int i = m.bank_elem[b];
  const int nbk = m.nbank;
  const double *bp = m.bank_part;
  double ds = bp[b], dg = bp[nbk + b];
  const double inv_area = m.inv_area[i];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int32_t nb = m.nb[j * ne + i];
    double o, u;
    if (nb < 0 && nb != kBoundary) {
      const int s = -1 - nb;
      if (m.left[s] == i) {
        o = -F[LEFT_SURF2CHANL * nr + s];
        u = -(F[LEFT_AQUIF2CHANL * nr + s] + F[LEFT_AQUIF2AQUIF * nr + s]);
      } else {
        o = -F[RIGHT_SURF2CHANL * nr + s];
        u = -(F[RIGHT_AQUIF2CHANL * nr + s] + F[RIGHT_AQUIF2AQUIF * nr + s]);
      }
      if (m.diag) {
        m.d_ovl[j * ne + i] = o;
        m.d_sub[j * ne + i] = u;
      }
    } else {
      o = bp[(2 + j) * nbk + b];
      u = bp[(5 + j) * nbk + b];
    }
    ds -= o * inv_area;
    dg -= u * inv_area;
  }
  dg *= m.inv_por[i];
  ydot[i] = ds;
  ydot[2 * ne + i] = dg;
  if (cmp::isnan_(ds) | cmp::isnan_(dg)) report_err(m, sy);
}

// ---------------------------------------------------------------------------
// state reordering between reference and internal order
// ---------------------------------------------------------------------------
__global__ void k_permute(const double *RESTRICT src, double *RESTRICT dst, const int32_t *RESTRICT perm,
                          int ne, int nr, int to_internal) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n_el = 3LL * ne;
  if (t < n_el) {
    const int blk = (int)(t / ne);
    const int i = (int)(t - (long long)blk * ne);
    const long long ref = (long long)blk * ne + perm[i];
    if (to_internal) dst[t] = src[ref];
    else dst[ref] = src[t];
  } else if (t < n_el + 2LL * nr) {
    dst[t] = src[t];
  }
}

// The same reordering walked in reference order (iperm: reference ->
// internal element index): the reference-order side is read or written
// contiguously, which is the side in host memory when the host-buffer
// evaluation accesses it directly.
__global__ void k_permute_ref(const double *RESTRICT src, double *RESTRICT dst,
                              const int32_t *RESTRICT iperm, int ne, int nr, int to_internal) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n_el = 3LL * ne;
  if (t < n_el) {
    const int blk = (int)(t / ne);
    const int r = (int)(t - (long long)blk * ne);
    const long long in = (long long)blk * ne + iperm[r];
    if (to_internal) dst[in] = src[t];
    else dst[t] = src[in];
  } else if (t < n_el + 2LL * nr) {
    dst[t] = src[t];
  }
}

}  // namespace pihm

// ---------------------------------------------------------------------------
// launch helpers used by the host side
// ---------------------------------------------------------------------------
namespace pihm {

static inline unsigned blocks_for(long long n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

// Take two events from the profiler's pool (grown on demand).
static bool prof_begin(Profiler *p, int kernel, cudaStream_t st) {
  if (!p) return false;
  if (p->used + 2 > p->npool) {
    int n = p->npool ? 2 * p->npool : 256;
    cudaEvent_t *np_ = (cudaEvent_t *)realloc(p->pool, sizeof(cudaEvent_t) * n);
    if (!np_) return false;
    p->pool = np_;
    for (int k = p->npool; k < n; k++) cudaEventCreate(&p->pool[k]);
    p->npool = n;
  }
  if (p->nrec + 1 > p->cap) {
    int n = p->cap ? 2 * p->cap : 128;
    Profiler::Rec *nr_ = (Profiler::Rec *)realloc(p->recs, sizeof(Profiler::Rec) * n);
    if (!nr_) return false;
    p->recs = nr_;
    p->cap = n;
  }
  Profiler::Rec &r = p->recs[p->nrec++];
  r.kernel = kernel;
  r.a = p->pool[p->used++];
  r.b = p->pool[p->used++];
  cudaEventRecord(r.a, st);
  return true;
}
static void prof_end(Profiler *p, bool on, cudaStream_t st) {
  if (on) cudaEventRecord(p->recs[p->nrec - 1].b, st);
}

cudaError_t launch_rhs(const DevMesh &m, const double *y, double *ydot, cudaStream_t st,
                       long long *launches, Profiler *prof, const RhsStreams *side, const double *y_ref,
                       const int32_t *iperm) {
  bool on;
  // the river kernel reads only k_elem_prep's outputs, the state and static
  // data, so with a side stream it runs beside grad/edge/main (per-kernel
  // timing keeps one stream)
  const bool fork = side && side->side && !prof && m.ne_run > 0 && m.nr_run > 0;
  if (m.ne_run > 0) {
    on = prof_begin(prof, K_PREP, st);
    if (y_ref)  // y is the internal-order buffer the kernel fills
      k_elem_prep<true><<<blocks_for((long long)m.ne + 2LL * m.nr, kPrepBlock), kPrepBlock, 0, st>>>(
          m, nullptr, y_ref, const_cast<double *>(y), iperm);
    else
      k_elem_prep<false><<<blocks_for(m.ne_run, kPrepBlock), kPrepBlock, 0, st>>>(m, y, nullptr, nullptr, nullptr);
    prof_end(prof, on, st);
    ++*launches;
    if (fork) {
      if (cudaEventRecord(side->fork, st) != cudaSuccess) return cudaErrorUnknown;
      if (cudaStreamWaitEvent(side->side, side->fork, 0) != cudaSuccess) return cudaErrorUnknown;
      k_riv_geom<<<blocks_for(m.nr_run, 128), 128, 0, side->side>>>(m, y);
      k_river<<<blocks_for(m.nr_run, 128), 128, 0, side->side>>>(m, y);
      *launches += 2;
      if (cudaEventRecord(side->join, side->side) != cudaSuccess) return cudaErrorUnknown;
    }
    if (m.surf_mode == kDiffWave) {
      on = prof_begin(prof, K_GRAD, st);
      k_elem_grad<<<blocks_for(m.ne_run, 256), 256, 0, st>>>(m, y);
      prof_end(prof, on, st);
      ++*launches;
    }
    if (m.nedge_run > 0) {
      on = prof_begin(prof, K_EDGE, st);
      k_edge<<<blocks_for(m.nedge_run, kEdgeBlock), kEdgeBlock, 0, st>>>(m, y);
      prof_end(prof, on, st);
      ++*launches;
    }
    on = prof_begin(prof, K_MAIN, st);
    switch (m.main_shape) {
      case 1: k_elem_main<256, 4><<<blocks_for(m.ne_run, 256), 256, 0, st>>>(m, y, ydot); break;
      case 2: k_elem_main<128, 8><<<blocks_for(m.ne_run, 128), 128, 0, st>>>(m, y, ydot); break;
      default: k_elem_main<512, 2><<<blocks_for(m.ne_run, 512), 512, 0, st>>>(m, y, ydot); break;
    }
    prof_end(prof, on, st);
    ++*launches;
  }
  if (fork) {
    if (cudaStreamWaitEvent(st, side->join, 0) != cudaSuccess) return cudaErrorUnknown;
  } else if (m.nr_run > 0) {
    on = prof_begin(prof, K_RIVER, st);  // both river kernels
    k_riv_geom<<<blocks_for(m.nr_run, 128), 128, 0, st>>>(m, y);
    k_river<<<blocks_for(m.nr_run, 128), 128, 0, st>>>(m, y);
    prof_end(prof, on, st);
    *launches += 2;
  }
  if (m.nr_run + m.nbank_run > 0) {
    on = prof_begin(prof, K_FINISH, st);
    k_finish<<<blocks_for((long long)m.nr_run + m.nbank_run, 128), 128, 0, st>>>(m, ydot);
    prof_end(prof, on, st);
    ++*launches;
  }
  return cudaGetLastError();
}

cudaError_t launch_permute(const double *src, double *dst, const int32_t *perm, int ne, int nr,
                           int to_internal, cudaStream_t st) {
  const long long n = 3LL * ne + 2LL * nr;
  if (n == 0) return cudaSuccess;
  k_permute<<<blocks_for(n, 256), 256, 0, st>>>(src, dst, perm, ne, nr, to_internal);
  return cudaGetLastError();
}

cudaError_t launch_permute_ref(const double *src, double *dst, const int32_t *iperm, int ne, int nr,
                               int to_internal, cudaStream_t st) {
  const long long n = 3LL * ne + 2LL * nr;
  if (n == 0) return cudaSuccess;
  k_permute_ref<<<blocks_for(n, 256), 256, 0, st>>>(src, dst, iperm, ne, nr, to_internal);
  return cudaGetLastError();
}

}  // namespace pihm
