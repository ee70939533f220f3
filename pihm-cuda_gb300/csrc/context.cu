// Host side of the C ABI: validation, locality renumbering, device images,
// inputs and the host-buffer entry points (include/pihm_gpu.h).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <queue>
#include <vector>

#include <type_traits>

#include "mesh_image.h"
#include "pihm_internal.h"

namespace pihm {
cudaError_t launch_permute(const double *src, double *dst, const int32_t *perm, int ne, int nr,
                           int to_internal, cudaStream_t st);
cudaError_t launch_permute_ref(const double *src, double *dst, const int32_t *iperm, int ne, int nr,
                               int to_internal, cudaStream_t st);
}  // namespace pihm

using namespace pihm;

namespace {

// An address through which kernels may read or write the host range
// [p, p + bytes), or nullptr: any host address on a device with
// pageable-memory access, else pinned or registered memory, whose first and
// last bytes must map to one contiguous device range.
const void *host_view(const pihm_gpu_ctx *c, const void *p, size_t bytes) {
  if (c->host_pageable) return p;
  cudaPointerAttributes a{}, b{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  const char *last = (const char *)p + bytes - 1;
  if (cudaPointerGetAttributes(&b, last) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (b.type != cudaMemoryTypeHost || !b.devicePointer) return nullptr;
  if ((const char *)b.devicePointer - (const char *)a.devicePointer != (ptrdiff_t)(bytes - 1)) return nullptr;
  return a.devicePointer;
}

template <class T>
T *carve(char *&p, size_t n) {
  T *r = reinterpret_cast<T *>(p);
  size_t bytes = (n * sizeof(T) + 255) & ~size_t(255);
  p += bytes;
  return r;
}
template <class T>
size_t carve_size(size_t n) {
  return (n * sizeof(T) + 255) & ~size_t(255);
}

int cuda_fail(cudaError_t e) { return e == cudaSuccess ? PIHM_GPU_OK : PIHM_GPU_ERR_CUDA; }

}  // namespace

extern "C" {

int pihm_gpu_create(const pihm_gpu_mesh *g, int surf_mode, int riv_mode, double stepsize, int order,
                    pihm_gpu_ctx **out) {
  if (!g || !out) return PIHM_GPU_ERR_ARG;
  *out = nullptr;
  SystemImage im;
  const int brc = build_image(g, surf_mode, riv_mode, stepsize, order, &im);
  if (brc != PIHM_GPU_OK) return brc;
  const int ne = im.ne, nr = im.nr, nbank = im.nbank, nedge = im.nedge;

  pihm_gpu_ctx *c = new pihm_gpu_ctx();
  std::memset(&c->m, 0, sizeof(c->m));
  c->ne = ne;
  c->nr = nr;
  c->neq = 3LL * ne + 2LL * nr;
  c->stream = nullptr;
  c->diag = 0;
  c->launches = 0;
  c->nan_check_deferred = 0;
  c->prof = nullptr;
  c->d_noah = nullptr;
  c->host_path = 0;
  c->last_direct = 0;
  {
    int dev = 0, pageable = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess)
      c->host_pageable = pageable;
    else
      c->host_pageable = 0;
  }
  c->h_perm = (int32_t *)std::malloc(sizeof(int32_t) * ne);
  c->h_iperm = (int32_t *)std::malloc(sizeof(int32_t) * ne);
  std::memcpy(c->h_perm, im.perm.data(), sizeof(int32_t) * ne);
  std::memcpy(c->h_iperm, im.iperm.data(), sizeof(int32_t) * ne);

  // ---- one host block holding every static plane, uploaded at once ----
  const size_t NE = ne, NR = nr > 0 ? nr : 1, NB = nbank > 0 ? nbank : 1;
  const size_t NED = nedge > 0 ? nedge : 1;
  const size_t NUP = im.up_idx.empty() ? 1 : im.up_idx.size();
  size_t sbytes = 0;
  sbytes += EP_COUNT * carve_size<double>(NE) + XP_COUNT * carve_size<double>(3 * NE);
  sbytes += 3 * carve_size<int32_t>(3 * NE);                   // nb, bctype, emap
  sbytes += 2 * carve_size<int32_t>(NED) + 3 * carve_size<double>(NED);  // edge list
  sbytes += carve_size<int32_t>(NE) + carve_size<int32_t>(NB); // bank_slot, bank_elem
  sbytes += 5 * carve_size<int32_t>(NR) + RP_COUNT * carve_size<double>(NR);
  sbytes += carve_size<int32_t>(NR + 1) + carve_size<int32_t>(NUP);
  sbytes += 2 * carve_size<int32_t>(NE);                       // perm, iperm
  std::vector<char> host(sbytes, 0);
  char *hp = host.data();
  if (cudaMalloc(&c->d_static, sbytes) != cudaSuccess) {
    pihm_gpu_destroy(c);
    return PIHM_GPU_ERR_NOMEM;
  }
  c->static_bytes = sbytes;
  char *base = host.data();
  char *dbase = (char *)c->d_static;
  // carve n items on the host, copy src in, return the device address
  auto put = [&](const auto *src, size_t n, size_t cap) {
    using T = std::remove_cv_t<std::remove_pointer_t<decltype(src)>>;
    T *h = carve<T>(hp, cap);
    if (n) std::memcpy(h, src, sizeof(T) * n);
    return (T *)(dbase + ((char *)h - base));
  };
  DevMesh &m = c->m;
  m.ne = ne;
  m.nr = nr;
  m.nbank = nbank;
  m.surf_mode = surf_mode;
  m.riv_mode = riv_mode;
  m.dt = stepsize;
  m.inv_dt = 1.0 / stepsize;
  for (int k = 0; k < EP_COUNT; k++) m.*kElemMember[k] = put(im.el[k].data(), NE, NE);
  for (int k = 0; k < XP_COUNT; k++) m.*kEdgeMember[k] = put(im.ed[k].data(), 3 * NE, 3 * NE);
  m.nb = put(im.nb.data(), 3 * NE, 3 * NE);
  m.bctype = put(im.bct.data(), 3 * NE, 3 * NE);
  m.emap = put(im.emap.data(), 3 * NE, 3 * NE);
  m.e_i = put(im.e_i.data(), nedge, NED);
  m.e_k = put(im.e_k.data(), nedge, NED);
  m.e_invdist = put(im.e_invdist.data(), nedge, NED);
  m.e_subk = put(im.e_subk.data(), nedge, NED);
  m.e_ovlk = put(im.e_ovlk.data(), nedge, NED);
  m.bank_slot = put(im.bank_slot.data(), NE, NE);
  m.bank_elem = put(im.bank_elem.data(), nbank, NB);
  m.down = put(im.down.data(), nr, NR);
  m.left = put(im.left.data(), nr, NR);
  m.right = put(im.right.data(), nr, NR);
  m.intrpl_ord = put(im.ord.data(), nr, NR);
  m.bctype_riv = put(im.rbct.data(), nr, NR);
  for (int k = 0; k < RP_COUNT; k++) m.*kRiverMember[k] = put(im.rv[k].data(), nr, NR);
  m.up_ptr = put(im.up_ptr.data(), nr + 1, NR + 1);
  m.up_idx = put(im.up_idx.data(), im.up_idx.size(), NUP);
  c->d_perm = put(im.perm.data(), NE, NE);
  c->d_iperm = put(im.iperm.data(), NE, NE);
  if (cudaMemcpy(c->d_static, host.data(), sbytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    pihm_gpu_destroy(c);
    return PIHM_GPU_ERR_CUDA;
  }
  m.up_end = m.up_ptr + 1;
  m.nedge = nedge;
  m.ne_run = ne;
  m.nr_run = nr;
  m.nedge_run = nedge;
  m.nbank_run = nbank;
  m.main_shape = 1;  // k_elem_main at 256 x 4 per SM

  // dynamic block: inputs, scratch, diagnostics, staging, error word
  size_t dbytes = 0;
  dbytes += 4 * carve_size<double>(NE);       // pcpdrp, edir, ett, ws0
  dbytes += carve_size<double>(3 * NE);       // elem_bc
  dbytes += carve_size<double>(NR);           // river_bc
  dbytes += 4 * carve_size<double>(NE);       // surfh, head, effk, gradmag
  dbytes += carve_size<double>(11 * NR);      // rivflow
  dbytes += carve_size<double>(2 * NR);       // carried river-edge overland flux
  dbytes += 2 * carve_size<double>(NR);       // channel perimeter and area
  dbytes += 2 * carve_size<double>(NED);      // edge fluxes
  dbytes += carve_size<double>(8 * NB);       // bank_part
  dbytes += 2 * carve_size<double>(3 * NE) + 2 * carve_size<double>(NE) + carve_size<double>(5 * NE);
  dbytes += 2 * carve_size<double>(c->neq);   // staging
  dbytes += carve_size<unsigned int>(1);
  if (cudaMalloc(&c->d_dyn, dbytes) != cudaSuccess) {
    pihm_gpu_destroy(c);
    return PIHM_GPU_ERR_NOMEM;
  }
  c->dyn_bytes = dbytes;
  if (cudaMemset(c->d_dyn, 0, dbytes) != cudaSuccess) {
    pihm_gpu_destroy(c);
    return PIHM_GPU_ERR_CUDA;
  }
  char *dp = (char *)c->d_dyn;
  m.pcpdrp = carve<double>(dp, NE); m.edir = carve<double>(dp, NE); m.ett = carve<double>(dp, NE);
  m.ws0_surf = carve<double>(dp, NE);
  m.elem_bc = carve<double>(dp, 3 * NE);
  m.river_bc = carve<double>(dp, NR);
  m.surfh = carve<double>(dp, NE); m.head = carve<double>(dp, NE); m.effk = carve<double>(dp, NE);
  m.gradmag = carve<double>(dp, NE);
  m.rivflow = carve<double>(dp, 11 * NR);
  m.carry_ovl = carve<double>(dp, 2 * NR);
  m.r_perim = carve<double>(dp, NR); m.r_crossa = carve<double>(dp, NR);
  m.eflux_ovl = carve<double>(dp, NED); m.eflux_sub = carve<double>(dp, NED);
  m.bank_part = carve<double>(dp, 8 * NB);
  m.d_ovl = carve<double>(dp, 3 * NE); m.d_sub = carve<double>(dp, 3 * NE);
  m.d_infil = carve<double>(dp, NE); m.d_rechg = carve<double>(dp, NE); m.d_et = carve<double>(dp, 5 * NE);
  c->d_stage_in = carve<double>(dp, c->neq);
  c->d_stage_out = carve<double>(dp, c->neq);
  m.err = carve<unsigned int>(dp, 1);
  m.diag = 0;
  if (pihm::create_rhs_streams(&c->side) != cudaSuccess) {
    pihm_gpu_destroy(c);
    return PIHM_GPU_ERR_CUDA;
  }
  *out = c;
  return PIHM_GPU_OK;
}

static void free_profiler(Profiler *p) {
  if (!p) return;
  for (int k = 0; k < p->npool; k++) cudaEventDestroy(p->pool[k]);
  free(p->pool);
  free(p->recs);
  delete p;
}

static void copy_path_release(pihm_gpu_ctx *c);

void pihm_gpu_destroy(pihm_gpu_ctx *c) {
  if (!c) return;
  copy_path_release(c);
  free_profiler(c->prof);
  if (c->d_static) cudaFree(c->d_static);
  if (c->d_dyn) cudaFree(c->d_dyn);
  if (c->d_noah) cudaFree(c->d_noah);
  pihm::land_release(c->land);
  pihm::noah_release(c->noahlsm);
  if (c->side.fork) cudaEventDestroy(c->side.fork);
  if (c->side.join) cudaEventDestroy(c->side.join);
  if (c->side.side) cudaStreamDestroy(c->side.side);
  std::free(c->h_perm);
  std::free(c->h_iperm);
  delete c;
}

int pihm_gpu_set_stream(pihm_gpu_ctx *c, void *stream) {
  if (!c) return PIHM_GPU_ERR_ARG;
  c->stream = (cudaStream_t)stream;
  return PIHM_GPU_OK;
}

void *pihm_gpu_get_stream(const pihm_gpu_ctx *c) { return c ? (void *)c->stream : nullptr; }

int pihm_gpu_set_kernel_shape(pihm_gpu_ctx *c, int shape) {
  if (!c || shape < 0 || shape > 2) return PIHM_GPU_ERR_ARG;
  c->m.main_shape = shape;
  return PIHM_GPU_OK;
}

int pihm_gpu_sizes(const pihm_gpu_ctx *c, int32_t *ne, int32_t *nr, int64_t *neq) {
  if (!c) return PIHM_GPU_ERR_ARG;
  if (ne) *ne = c->ne;
  if (nr) *nr = c->nr;
  if (neq) *neq = c->neq;
  return PIHM_GPU_OK;
}

int pihm_gpu_get_permutation(const pihm_gpu_ctx *c, int32_t *elem_perm, int32_t *river_perm) {
  if (!c) return PIHM_GPU_ERR_ARG;
  if (elem_perm) std::memcpy(elem_perm, c->h_perm, sizeof(int32_t) * c->ne);
  if (river_perm)
    for (int s = 0; s < c->nr; s++) river_perm[s] = s;
  return PIHM_GPU_OK;
}

// Copy a host array in reference order into an internal-order device plane.
static int upload_elem(pihm_gpu_ctx *c, const double *src, double *dst, int planes, int stride_in) {
  std::vector<double> tmp((size_t)planes * c->ne);
  for (int j = 0; j < planes; j++)
    for (int i = 0; i < c->ne; i++) tmp[(size_t)j * c->ne + i] = src[(size_t)stride_in * c->h_perm[i] + j];
  return cuda_fail(cudaMemcpyAsync(dst, tmp.data(), sizeof(double) * tmp.size(), cudaMemcpyHostToDevice,
                                   c->stream)) ?: cuda_fail(cudaStreamSynchronize(c->stream));
}

int pihm_gpu_set_forcing(pihm_gpu_ctx *c, const double *pcpdrp, const double *edir, const double *ett) {
  if (!c) return PIHM_GPU_ERR_ARG;
  int rc = PIHM_GPU_OK;
  if (pcpdrp && (rc = upload_elem(c, pcpdrp, (double *)c->m.pcpdrp, 1, 1))) return rc;
  if (edir && (rc = upload_elem(c, edir, (double *)c->m.edir, 1, 1))) return rc;
  if (ett && (rc = upload_elem(c, ett, (double *)c->m.ett, 1, 1))) return rc;
  return rc;
}

int pihm_gpu_set_bc(pihm_gpu_ctx *c, const double *elem_bc, const double *river_bc) {
  if (!c) return PIHM_GPU_ERR_ARG;
  int rc = PIHM_GPU_OK;
  if (elem_bc && (rc = upload_elem(c, elem_bc, (double *)c->m.elem_bc, 3, 3))) return rc;
  if (river_bc && c->nr)
    rc = cuda_fail(cudaMemcpyAsync((double *)c->m.river_bc, river_bc, sizeof(double) * c->nr,
                                   cudaMemcpyHostToDevice, c->stream)) ?:
         cuda_fail(cudaStreamSynchronize(c->stream));
  return rc;
}

int pihm_gpu_set_noah(pihm_gpu_ctx *c, const double *et, int nlayers, const int32_t *nwtbl,
                      const int32_t *nroot, const double *sh2o0, const double *smcmin, const double *smcmax,
                      const double *fcr) {
  if (!c || !nwtbl || !nroot || !sh2o0 || !smcmin || !smcmax || !fcr || nlayers < 0 || nlayers > 11 ||
      (nlayers > 0 && !et))
    return PIHM_GPU_ERR_ARG;
  const int ne = c->ne;
  const size_t NE = ne;
  for (int r = 0; r < ne; r++)
    if (nroot[r] > nlayers) return PIHM_GPU_ERR_ARG;
  if (!c->d_noah) {
    const size_t bytes = 3 * carve_size<double>(NE) + carve_size<int32_t>(NE);
    if (cudaMalloc(&c->d_noah, bytes) != cudaSuccess) {
      c->d_noah = nullptr;
      return PIHM_GPU_ERR_NOMEM;
    }
    char *p = (char *)c->d_noah;
    c->m.noah_etgw = carve<double>(p, NE);
    c->m.noah_satn = carve<double>(p, NE);
    c->m.noah_fcr = carve<double>(p, NE);
    c->m.noah_wtin = carve<int32_t>(p, NE);
  }
  // per element, internal order: GwTransp's layer sum in its order
  // (noah/lsm_func.c:171-177), Infil's top-layer saturation
  // (src/vert_flow.c:94-98), the frozen-soil factor
  std::vector<double> etgw(NE), satn(NE), f(NE);
  std::vector<int32_t> wtin(NE);
  for (int i = 0; i < ne; i++) {
    const int r = c->h_perm[i];
    double g = 0.0;
    const int top = nwtbl[r], nr = nroot[r];
    wtin[i] = top <= nr;
    if (top <= nr)
      for (int j = (top <= 0 ? 0 : top - 1); j < nr; j++) g += et[(size_t)nlayers * r + j];
    etgw[i] = g;
    satn[i] = (sh2o0[r] - smcmin[r]) / (smcmax[r] - smcmin[r]);
    f[i] = fcr[r];
  }
  const int rc = cuda_fail(cudaMemcpyAsync((void *)c->m.noah_etgw, etgw.data(), sizeof(double) * NE,
                                           cudaMemcpyHostToDevice, c->stream)) ?:
                 cuda_fail(cudaMemcpyAsync((void *)c->m.noah_satn, satn.data(), sizeof(double) * NE,
                                           cudaMemcpyHostToDevice, c->stream)) ?:
                 cuda_fail(cudaMemcpyAsync((void *)c->m.noah_fcr, f.data(), sizeof(double) * NE,
                                           cudaMemcpyHostToDevice, c->stream)) ?:
                 cuda_fail(cudaMemcpyAsync((void *)c->m.noah_wtin, wtin.data(), sizeof(int32_t) * NE,
                                           cudaMemcpyHostToDevice, c->stream)) ?:
                 cuda_fail(cudaStreamSynchronize(c->stream));
  if (rc == PIHM_GPU_OK) c->m.noah = 1;
  return rc;
}

int pihm_gpu_set_ws0_surf(pihm_gpu_ctx *c, const double *ws0) {
  if (!c || !ws0) return PIHM_GPU_ERR_ARG;
  return upload_elem(c, ws0, (double *)c->m.ws0_surf, 1, 1);
}

int pihm_gpu_set_river_edge_ovlflow(pihm_gpu_ctx *c, const double *ovl) {
  if (!c || !ovl) return PIHM_GPU_ERR_ARG;
  if (!c->nr) return PIHM_GPU_OK;
  // the carried value of element e's river edge is -rivflow[LEFT/RIGHT_SURF2CHANL]
  // of that river (src/river_flow.c:159-182); rebuild the carry (and those
  // two slots)
  std::vector<double> slots(2 * (size_t)c->nr, 0.0);
  const int ne = c->ne;
  std::vector<int32_t> left(c->nr), right(c->nr);
  cudaMemcpy(left.data(), c->m.left, sizeof(int32_t) * c->nr, cudaMemcpyDeviceToHost);
  cudaMemcpy(right.data(), c->m.right, sizeof(int32_t) * c->nr, cudaMemcpyDeviceToHost);
  std::vector<int32_t> nb(3 * (size_t)ne);
  cudaMemcpy(nb.data(), c->m.nb, sizeof(int32_t) * 3 * ne, cudaMemcpyDeviceToHost);
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < 3; j++) {
      int32_t v = nb[(size_t)j * ne + i];
      if (v < 0 && v != kBoundary) {
        int s = -1 - v;
        double val = -ovl[3 * (size_t)c->h_perm[i] + j];
        if (left[s] == i) slots[s] = val;
        else slots[c->nr + s] = val;
      }
    }
  double *F = c->m.rivflow;
  return cuda_fail(cudaMemcpyAsync(c->m.carry_ovl, slots.data(), sizeof(double) * 2 * c->nr,
                                   cudaMemcpyHostToDevice, c->stream)) ?:
         cuda_fail(cudaMemcpyAsync(F + LEFT_SURF2CHANL * (size_t)c->nr, slots.data(),
                                   sizeof(double) * c->nr, cudaMemcpyHostToDevice, c->stream)) ?:
         cuda_fail(cudaMemcpyAsync(F + RIGHT_SURF2CHANL * (size_t)c->nr, slots.data() + c->nr,
                                   sizeof(double) * c->nr, cudaMemcpyHostToDevice, c->stream)) ?:
         cuda_fail(cudaStreamSynchronize(c->stream));
}

int pihm_gpu_rhs(pihm_gpu_ctx *c, double t, const double *y, double *ydot) {
  (void)t;
  if (!c || !y || !ydot) return PIHM_GPU_ERR_ARG;
  c->m.diag = c->diag;
  return cuda_fail(launch_rhs(c->m, y, ydot, c->stream, &c->launches, c->prof, &c->side));
}

int pihm_gpu_status(pihm_gpu_ctx *c) {
  if (!c) return PIHM_GPU_ERR_ARG;
  unsigned int err = 0;
  if (cudaMemcpyAsync(&err, c->m.err, sizeof(err), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
    return PIHM_GPU_ERR_CUDA;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  if (err) {
    cudaMemsetAsync(c->m.err, 0, sizeof(unsigned int), c->stream);
    cudaStreamSynchronize(c->stream);
    return PIHM_GPU_ERR_NAN;
  }
  return PIHM_GPU_OK;
}

// The copy path's staging pairs, streams and events, on first use.
static bool copy_path_init(pihm_gpu_ctx *c) {
  auto &cp = c->cp;
  if (cp.ready) return true;
  const size_t bytes = sizeof(double) * c->neq;
  const size_t one = (bytes + 255) & ~size_t(255);
  // staging of its own: the direct path's kernels use d_stage_in/out on the
  // context's stream, which this path's copy streams are not ordered after
  if (cudaMalloc(&cp.staging, 4 * one) != cudaSuccess) {
    cp.staging = nullptr;
    return false;
  }
  for (int k = 0; k < 2; k++) {
    cp.in[k] = (double *)((char *)cp.staging + (2 * k) * one);
    cp.out[k] = (double *)((char *)cp.staging + (2 * k + 1) * one);
  }
  bool ok = cudaStreamCreateWithFlags(&cp.h2d, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&cp.d2h, cudaStreamNonBlocking) == cudaSuccess;
  for (int k = 0; k < 2 && ok; k++)
    ok = cudaEventCreateWithFlags(&cp.arrived[k], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&cp.done[k], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&cp.freed[k], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    copy_path_release(c);
    return false;
  }
  cp.ready = true;
  return true;
}

static void copy_path_release(pihm_gpu_ctx *c) {
  auto &cp = c->cp;
  if (cp.h2d) cudaStreamSynchronize(cp.h2d);
  if (cp.d2h) cudaStreamSynchronize(cp.d2h);
  for (int k = 0; k < 2; k++)
    for (cudaEvent_t e : {cp.arrived[k], cp.done[k], cp.freed[k]})
      if (e) cudaEventDestroy(e);
  if (cp.h2d) cudaStreamDestroy(cp.h2d);
  if (cp.d2h) cudaStreamDestroy(cp.d2h);
  if (cp.staging) cudaFree(cp.staging);
  cp = pihm_gpu_ctx::CopyPath{};
}

// The host-buffer evaluation queued on the context's stream.
static int rhs_host_enqueue(pihm_gpu_ctx *c, const double *y_host, double *ydot_host) {
  const size_t bytes = sizeof(double) * c->neq;
  // direct: k_elem_prep reads y from and the reordering kernel writes ydot to
  // host memory over the host link, in reference order (contiguous on the
  // host side)
  const double *y_dev = c->host_path == 0 ? (const double *)host_view(c, y_host, bytes) : nullptr;
  double *yd_dev = y_dev ? (double *)host_view(c, ydot_host, bytes) : nullptr;
  c->last_direct = yd_dev != nullptr;
  if (yd_dev) {
    // k_elem_prep reads the state from host memory in reference order and
    // fills y_int itself
    double *y_int = c->d_stage_out, *ydot_int = c->d_stage_in;
    c->m.diag = c->diag;
    cudaError_t e = launch_rhs(c->m, y_int, ydot_int, c->stream, &c->launches, c->prof, &c->side, y_dev,
                               c->d_iperm);
    if (e == cudaSuccess) {
      e = launch_permute_ref(ydot_int, yd_dev, c->d_iperm, c->ne, c->nr, 0, c->stream);
      c->launches++;
    }
    return e == cudaSuccess ? PIHM_GPU_OK : PIHM_GPU_ERR_CUDA;
  }
  // copy, then k_elem_prep reorders while preparing (the right-hand side
  // writes ydot over the reference-order copy once it has been read).  The
  // staging pairs alternate: the state of the evaluation after this one
  // arrives on the h2d stream while this one's kernels run, and this one's
  // derivative leaves on the d2h stream while the next one's kernels run.
  // A pair is refilled only after the derivative it held two evaluations
  // ago has left (freed), and the kernels start only after their state has
  // arrived.
  if (!copy_path_init(c)) return PIHM_GPU_ERR_NOMEM;
  auto &cp = c->cp;
  const int s = cp.slot;
  cp.slot ^= 1;
  double *in = cp.in[s], *out = cp.out[s];
  cudaError_t e = cudaStreamWaitEvent(cp.h2d, cp.freed[s], 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(in, y_host, bytes, cudaMemcpyHostToDevice, cp.h2d);
  if (e == cudaSuccess) e = cudaEventRecord(cp.arrived[s], cp.h2d);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, cp.arrived[s], 0);
  if (e == cudaSuccess) {
    c->m.diag = c->diag;
    e = launch_rhs(c->m, out, in, c->stream, &c->launches, c->prof, &c->side, in, c->d_iperm);
  }
  if (e == cudaSuccess) {
    e = launch_permute(in, out, c->d_perm, c->ne, c->nr, 0, c->stream);
    c->launches++;
  }
  if (e == cudaSuccess) e = cudaEventRecord(cp.done[s], c->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cp.d2h, cp.done[s], 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ydot_host, out, bytes, cudaMemcpyDeviceToHost, cp.d2h);
  if (e == cudaSuccess) e = cudaEventRecord(cp.freed[s], cp.d2h);
  return e == cudaSuccess ? PIHM_GPU_OK : PIHM_GPU_ERR_CUDA;
}

// Everything a host-buffer evaluation queued: the derivatives' copies out
// (after their kernels), then the error word on the context's stream.
static int host_wait(pihm_gpu_ctx *c) {
  if (c->cp.ready && cudaStreamSynchronize(c->cp.d2h) != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  return pihm_gpu_status(c);
}

int pihm_gpu_rhs_host(pihm_gpu_ctx *c, double t, const double *y_host, double *ydot_host) {
  (void)t;
  if (!c || !y_host || !ydot_host) return PIHM_GPU_ERR_ARG;
  const int rc = rhs_host_enqueue(c, y_host, ydot_host);
  return rc != PIHM_GPU_OK ? rc : host_wait(c);
}

int pihm_gpu_rhs_host_async(pihm_gpu_ctx *c, double t, const double *y_host, double *ydot_host) {
  (void)t;
  if (!c || !y_host || !ydot_host) return PIHM_GPU_ERR_ARG;
  return rhs_host_enqueue(c, y_host, ydot_host);
}

int pihm_gpu_wait(pihm_gpu_ctx *c) { return c ? host_wait(c) : PIHM_GPU_ERR_ARG; }

int pihm_gpu_set_host_path(pihm_gpu_ctx *c, int mode) {
  if (!c || (mode != 0 && mode != 1)) return PIHM_GPU_ERR_ARG;
  c->host_path = mode;
  return PIHM_GPU_OK;
}

int pihm_gpu_host_path_info(const pihm_gpu_ctx *c, int *last_direct, int *pageable_access) {
  if (!c) return PIHM_GPU_ERR_ARG;
  if (last_direct) *last_direct = c->last_direct;
  if (pageable_access) *pageable_access = c->host_pageable;
  return PIHM_GPU_OK;
}

int pihm_gpu_set_diagnostics(pihm_gpu_ctx *c, int on) {
  if (!c) return PIHM_GPU_ERR_ARG;
  c->diag = on ? 1 : 0;
  return PIHM_GPU_OK;
}

int pihm_gpu_get_fluxes(pihm_gpu_ctx *c, double *ovlflow, double *subsurf, double *infil, double *rechg,
                        double *et_split, double *rivflow) {
  if (!c) return PIHM_GPU_ERR_ARG;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  const int ne = c->ne, nr = c->nr;
  auto down_elem = [&](const double *dsrc, double *dst, int planes) {
    std::vector<double> tmp((size_t)planes * ne);
    cudaMemcpy(tmp.data(), dsrc, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost);
    for (int j = 0; j < planes; j++)
      for (int i = 0; i < ne; i++) dst[(size_t)planes * c->h_perm[i] + j] = tmp[(size_t)j * ne + i];
  };
  if (ovlflow) down_elem(c->m.d_ovl, ovlflow, 3);
  if (subsurf) down_elem(c->m.d_sub, subsurf, 3);
  if (infil) down_elem(c->m.d_infil, infil, 1);
  if (rechg) down_elem(c->m.d_rechg, rechg, 1);
  if (et_split) down_elem(c->m.d_et, et_split, 5);
  if (rivflow && nr) {
    std::vector<double> tmp(11 * (size_t)nr);
    cudaMemcpy(tmp.data(), c->m.rivflow, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost);
    for (int s = 0; s < nr; s++)
      for (int k = 0; k < 11; k++) rivflow[11 * (size_t)s + k] = tmp[(size_t)k * nr + s];
  }
  return cudaGetLastError() == cudaSuccess ? PIHM_GPU_OK : PIHM_GPU_ERR_CUDA;
}

int pihm_gpu_launch_count(const pihm_gpu_ctx *c, int64_t *count) {
  if (!c || !count) return PIHM_GPU_ERR_ARG;
  *count = c->launches;
  return PIHM_GPU_OK;
}

int pihm_gpu_set_profiling(pihm_gpu_ctx *c, int on) {
  if (!c) return PIHM_GPU_ERR_ARG;
  if (on && !c->prof) c->prof = new Profiler();
  if (!on && c->prof) {
    cudaStreamSynchronize(c->stream);
    free_profiler(c->prof);
    c->prof = nullptr;
  }
  return PIHM_GPU_OK;
}

int pihm_gpu_kernel_times(pihm_gpu_ctx *c, double *ms, int64_t *calls, int n) {
  if (!c || !c->prof || n <= 0) return PIHM_GPU_ERR_ARG;
  Profiler *p = c->prof;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  for (int r = 0; r < p->nrec; r++) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, p->recs[r].a, p->recs[r].b) == cudaSuccess) {
      p->ms[p->recs[r].kernel] += t;
      p->calls[p->recs[r].kernel] += 1;
    }
  }
  p->nrec = 0;
  p->used = 0;
  for (int k = 0; k < n && k < Profiler::kKernels; k++) {
    if (ms) ms[k] = p->ms[k];
    if (calls) calls[k] = p->calls[k];
    p->ms[k] = 0;
    p->calls[k] = 0;
  }
  return PIHM_GPU_OK;
}

int pihm_gpu_to_internal(pihm_gpu_ctx *c, const double *src, double *dst) {
  if (!c || !src || !dst || src == dst) return PIHM_GPU_ERR_ARG;
  c->launches++;
  return cuda_fail(launch_permute(src, dst, c->d_perm, c->ne, c->nr, 1, c->stream));
}

int pihm_gpu_to_reference(pihm_gpu_ctx *c, const double *src, double *dst) {
  if (!c || !src || !dst || src == dst) return PIHM_GPU_ERR_ARG;
  c->launches++;
  return cuda_fail(launch_permute(src, dst, c->d_perm, c->ne, c->nr, 0, c->stream));
}

}  // extern "C"
