// Host side of the C ABI: validation, locality renumbering, device images,
// inputs and the host-buffer entry points (include/pihm_gpu.h).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <queue>
#include <vector>

#include "pihm_internal.h"

namespace pihm {
cudaError_t launch_rhs(const DevMesh &m, const double *y, double *ydot, cudaStream_t st,
                       long long *launches, Profiler *prof);
cudaError_t launch_permute(const double *src, double *dst, const int32_t *perm, int ne, int nr,
                           int to_internal, cudaStream_t st);
}  // namespace pihm

using namespace pihm;

namespace {

// Reverse Cuthill-McKee over the element adjacency.  Returns perm with
// perm[internal] = reference index.
std::vector<int32_t> rcm_order(int ne, const int32_t *nabr) {
  std::vector<int> deg(ne, 0);
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < 3; j++) deg[i] += (nabr[3 * i + j] > 0);
  std::vector<int32_t> order;
  order.reserve(ne);
  std::vector<char> seen(ne, 0);
  std::vector<int> by_deg(ne);
  std::iota(by_deg.begin(), by_deg.end(), 0);
  std::stable_sort(by_deg.begin(), by_deg.end(), [&](int a, int b) { return deg[a] < deg[b]; });
  auto bfs_last = [&](int start, std::vector<int> &level) {
    // BFS returning the last vertex reached (a pseudo-peripheral candidate)
    std::queue<int> q;
    q.push(start);
    level[start] = 0;
    int last = start;
    std::vector<int> touched{start};
    while (!q.empty()) {
      int v = q.front();
      q.pop();
      last = v;
      for (int j = 0; j < 3; j++) {
        int k = nabr[3 * v + j] - 1;
        if (k >= 0 && level[k] < 0) {
          level[k] = level[v] + 1;
          touched.push_back(k);
          q.push(k);
        }
      }
    }
    for (int t : touched) level[t] = -1;
    return last;
  };
  std::vector<int> level(ne, -1);
  for (int seed : by_deg) {
    if (seen[seed]) continue;
    int start = bfs_last(bfs_last(seed, level), level);
    size_t head = order.size();
    order.push_back(start);
    seen[start] = 1;
    while (head < order.size()) {
      int v = order[head++];
      int nbs[3], c = 0;
      for (int j = 0; j < 3; j++) {
        int k = nabr[3 * v + j] - 1;
        if (k >= 0 && !seen[k]) {
          seen[k] = 1;
          nbs[c++] = k;
        }
      }
      std::sort(nbs, nbs + c, [&](int a, int b) { return deg[a] != deg[b] ? deg[a] < deg[b] : a < b; });
      for (int q = 0; q < c; q++) order.push_back(nbs[q]);
    }
  }
  std::reverse(order.begin(), order.end());
  return order;
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
  const int ne = g->nelem, nr = g->nriver;
  if (ne <= 0 || nr < 0) return PIHM_GPU_ERR_ARG;
  if ((surf_mode != kKinematic && surf_mode != kDiffWave) ||
      (riv_mode != kKinematic && riv_mode != kDiffWave) || !(stepsize > 0.0))
    return PIHM_GPU_ERR_ARG;
  if (order != PIHM_GPU_ORDER_REFERENCE && order != PIHM_GPU_ORDER_RCM) return PIHM_GPU_ERR_ARG;

  // ---- validation (the reference indexes these unchecked) ----
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < 3; j++) {
      int nb = g->nabr[3 * i + j];
      if (nb > ne || nb < -nr) return PIHM_GPU_ERR_MESH;
      if (nb < 0) {
        int s = -nb - 1;
        if (g->leftele[s] != i + 1 && g->rightele[s] != i + 1) return PIHM_GPU_ERR_MESH;
      }
    }
  for (int s = 0; s < nr; s++) {
    int L = g->leftele[s], R = g->rightele[s], d = g->down[s], o = g->intrpl_ord[s];
    if (L < 1 || L > ne || R < 1 || R > ne || L == R) return PIHM_GPU_ERR_MESH;
    if (d == 0 || d > nr || d == s + 1) return PIHM_GPU_ERR_MESH;
    if (d < 0 && d < kCritDpth) return PIHM_GPU_ERR_BCTYPE;
    if (o < kRectangle || o > kCubic) return PIHM_GPU_ERR_BCTYPE;
  }

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

  // ---- renumbering ----
  std::vector<int32_t> perm(ne);
  if (order == PIHM_GPU_ORDER_RCM) perm = rcm_order(ne, g->nabr);
  else std::iota(perm.begin(), perm.end(), 0);
  std::vector<int32_t> iperm(ne);
  for (int i = 0; i < ne; i++) iperm[perm[i]] = i;
  c->h_perm = (int32_t *)std::malloc(sizeof(int32_t) * ne);
  c->h_iperm = (int32_t *)std::malloc(sizeof(int32_t) * ne);
  std::memcpy(c->h_perm, perm.data(), sizeof(int32_t) * ne);
  std::memcpy(c->h_iperm, iperm.data(), sizeof(int32_t) * ne);

  // bank elements (with at least one river edge), internal order
  std::vector<int32_t> bank_slot(ne, -1), bank_elem;
  for (int i = 0; i < ne; i++) {
    int r = perm[i];
    for (int j = 0; j < 3; j++)
      if (g->nabr[3 * r + j] < 0) {
        bank_slot[i] = (int32_t)bank_elem.size();
        bank_elem.push_back(i);
        break;
      }
  }
  const int nbank = (int)bank_elem.size();
  // upstream CSR in reference order
  std::vector<int32_t> up_ptr(nr + 1, 0), up_idx;
  for (int s = 0; s < nr; s++)
    if (g->down[s] > 0) up_ptr[g->down[s]]++;
  for (int s = 0; s < nr; s++) up_ptr[s + 1] += up_ptr[s];
  up_idx.resize(up_ptr[nr] > 0 ? up_ptr[nr] : 1);
  {
    std::vector<int32_t> fill(up_ptr.begin(), up_ptr.end() - 1);
    for (int s = 0; s < nr; s++)
      if (g->down[s] > 0) up_idx[fill[g->down[s] - 1]++] = s;
  }

  // ---- interior edges, internal order ----
  // An edge is owned by the element with the smaller internal index when the
  // flux is antisymmetric: diffusion wave, both sides list each other, and the
  // distance and edge length agree bit for bit.  Otherwise every element side
  // is a one-sided edge evaluated from that side, as in the reference.
  std::vector<int32_t> e_i, e_k, emap(3 * (size_t)ne, 0);
  std::vector<double> e_invdist, e_len, e_invrough;
  for (int i = 0; i < ne; i++) {
    const int ri = perm[i];
    for (int j = 0; j < 3; j++) {
      const int nbr = g->nabr[3 * ri + j];
      if (nbr <= 0) continue;
      const int rk = nbr - 1, k = iperm[rk];
      int jr = -1;
      for (int q = 0; q < 3; q++)
        if (g->nabr[3 * rk + q] == ri + 1) {
          jr = q;
          break;
        }
      const bool sym = surf_mode == kDiffWave && jr >= 0 &&
                       g->nabrdist[3 * ri + j] == g->nabrdist[3 * rk + jr] &&
                       g->edge[3 * ri + j] == g->edge[3 * rk + jr];
      if (sym && k < i) continue;  // owned by k, recorded when k was visited
      const int e = (int)e_i.size();
      e_i.push_back(i);
      e_k.push_back(k);
      e_invdist.push_back(1.0 / g->nabrdist[3 * ri + j]);
      e_len.push_back(g->edge[3 * ri + j]);
      e_invrough.push_back(1.0 / (0.5 * (g->rough[ri] + g->rough[rk])));
      emap[(size_t)j * ne + i] = e + 1;
      if (sym) emap[(size_t)jr * ne + k] = -(e + 1);
    }
  }
  const int nedge = (int)e_i.size();

  // ---- host images of the static planes ----
  const size_t NE = ne, NR = nr > 0 ? nr : 1, NB = nbank > 0 ? nbank : 1;
  const size_t NED = nedge > 0 ? nedge : 1;
  size_t sbytes = 0;
  sbytes += 13 * carve_size<double>(NE);                       // derived element constants
  sbytes += 2 * carve_size<int32_t>(NED) + 3 * carve_size<double>(NED);  // edge list
  sbytes += carve_size<int32_t>(3 * NE);                       // emap
  sbytes += 18 * carve_size<double>(NE);                       // element scalars
  sbytes += 4 * carve_size<double>(3 * NE);                    // edge, nabrdist, nabr_x, nabr_y
  sbytes += 2 * carve_size<double>(NE);                        // den_x, den_y
  sbytes += 2 * carve_size<int32_t>(3 * NE);                   // nb, bctype
  sbytes += carve_size<int32_t>(NE) + carve_size<int32_t>(NB); // bank_slot, bank_elem
  sbytes += 5 * carve_size<int32_t>(NR);                       // river ints
  sbytes += 17 * carve_size<double>(NR);                       // river doubles
  sbytes += carve_size<int32_t>(NR + 1) + carve_size<int32_t>(up_idx.size());
  sbytes += carve_size<int32_t>(NE);                           // perm
  std::vector<char> host(sbytes, 0);
  char *hp = host.data();

  auto put_elem = [&](const double *src) {
    double *d = carve<double>(hp, NE);
    for (int i = 0; i < ne; i++) d[i] = src[perm[i]];
    return d;
  };
  double *h_area = put_elem(g->area), *h_zmin = put_elem(g->zmin), *h_zmax = put_elem(g->zmax);
  double *h_depth = put_elem(g->depth), *h_ksath = put_elem(g->ksath), *h_ksatv = put_elem(g->ksatv);
  double *h_kinfv = put_elem(g->kinfv), *h_dinf = put_elem(g->dinf), *h_alpha = put_elem(g->alpha);
  double *h_beta = put_elem(g->beta), *h_por = put_elem(g->porosity), *h_dmac = put_elem(g->dmac);
  double *h_kmach = put_elem(g->kmach), *h_kmacv = put_elem(g->kmacv), *h_areafv = put_elem(g->areafv);
  double *h_areafh = put_elem(g->areafh), *h_rough = put_elem(g->rough), *h_rzd = put_elem(g->rzd);
  auto put_edge = [&](const double *src) {
    double *d = carve<double>(hp, 3 * NE);
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < ne; i++) d[j * NE + i] = src[3 * perm[i] + j];
    return d;
  };
  double *h_edge = put_edge(g->edge), *h_dist = put_edge(g->nabrdist);
  double *h_nx = put_edge(g->nabr_x), *h_ny = put_edge(g->nabr_y);
  double *h_denx = carve<double>(hp, NE), *h_deny = carve<double>(hp, NE);
  for (int i = 0; i < ne; i++) {
    // denominators of DhByDl (src/lat_flow.c:239-246): l2[2](l1[1]-l1[0]) +
    // l2[1](l1[0]-l1[2]) + l2[0](l1[2]-l1[1]) for (l1,l2) = (y,x) and (x,y)
    const double x0 = h_nx[i], x1 = h_nx[NE + i], x2 = h_nx[2 * NE + i];
    const double y0 = h_ny[i], y1 = h_ny[NE + i], y2 = h_ny[2 * NE + i];
    h_denx[i] = x2 * (y1 - y0) + x1 * (y0 - y2) + x0 * (y2 - y1);
    h_deny[i] = y2 * (x1 - x0) + y1 * (x0 - x2) + y0 * (x2 - x1);
  }
  int32_t *h_nb = carve<int32_t>(hp, 3 * NE), *h_bct = carve<int32_t>(hp, 3 * NE);
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < ne; i++) {
      int nb = g->nabr[3 * perm[i] + j];
      h_nb[j * NE + i] = nb > 0 ? iperm[nb - 1] : (nb < 0 ? -1 - (-nb - 1) : kBoundary);
      h_bct[j * NE + i] = g->bc_type[3 * perm[i] + j];
    }
  int32_t *h_bslot = carve<int32_t>(hp, NE), *h_belem = carve<int32_t>(hp, NB);
  std::memcpy(h_bslot, bank_slot.data(), sizeof(int32_t) * ne);
  if (nbank) std::memcpy(h_belem, bank_elem.data(), sizeof(int32_t) * nbank);
  int32_t *h_down = carve<int32_t>(hp, NR), *h_left = carve<int32_t>(hp, NR);
  int32_t *h_right = carve<int32_t>(hp, NR), *h_ord = carve<int32_t>(hp, NR);
  int32_t *h_rbct = carve<int32_t>(hp, NR);
  for (int s = 0; s < nr; s++) {
    h_down[s] = g->down[s];
    h_left[s] = iperm[g->leftele[s] - 1];
    h_right[s] = iperm[g->rightele[s] - 1];
    h_ord[s] = g->intrpl_ord[s];
    h_rbct[s] = g->riverbc_type[s];
  }
  auto put_riv = [&](const double *src) {
    double *d = carve<double>(hp, NR);
    if (nr) std::memcpy(d, src, sizeof(double) * nr);
    return d;
  };
  double *h_rarea = put_riv(g->riv_area), *h_rzmin = put_riv(g->riv_zmin), *h_rzmax = put_riv(g->riv_zmax);
  double *h_rzbed = put_riv(g->riv_zbed), *h_rnz = put_riv(g->riv_node_zmax);
  double *h_rdl = put_riv(g->riv_dist_left), *h_rdr = put_riv(g->riv_dist_right);
  double *h_rdep = put_riv(g->riv_depth), *h_rco = put_riv(g->riv_coeff), *h_rlen = put_riv(g->riv_length);
  double *h_rwid = put_riv(g->riv_width), *h_rrough = put_riv(g->riv_rough), *h_rcwr = put_riv(g->riv_cwr);
  double *h_rkh = put_riv(g->riv_ksath), *h_rkv = put_riv(g->riv_ksatv), *h_rbed = put_riv(g->riv_bedthick);
  double *h_rpor = put_riv(g->riv_porosity);
  int32_t *h_upp = carve<int32_t>(hp, NR + 1), *h_upi = carve<int32_t>(hp, up_idx.size());
  std::memcpy(h_upp, up_ptr.data(), sizeof(int32_t) * (nr + 1));
  std::memcpy(h_upi, up_idx.data(), sizeof(int32_t) * up_idx.size());
  int32_t *h_permd = carve<int32_t>(hp, NE);
  std::memcpy(h_permd, perm.data(), sizeof(int32_t) * ne);

  // derived element constants (see DevMesh); same expressions as the
  // reference's inline ones, evaluated without contraction
  double *h_inv_area = carve<double>(hp, NE), *h_inv_por = carve<double>(hp, NE);
  double *h_inv_alpha = carve<double>(hp, NE), *h_vg_m = carve<double>(hp, NE);
  double *h_vg_e = carve<double>(hp, NE), *h_vg_ib = carve<double>(hp, NE);
  double *h_kinf_mat = carve<double>(hp, NE), *h_kmac_a = carve<double>(hp, NE);
  double *h_kv2_mac = carve<double>(hp, NE), *h_d_dinf = carve<double>(hp, NE);
  double *h_d_rzd = carve<double>(hp, NE), *h_d_dmac = carve<double>(hp, NE);
  double *h_kh_k1 = carve<double>(hp, NE);
  for (int i = 0; i < ne; i++) {
    h_inv_area[i] = 1.0 / h_area[i];
    h_inv_por[i] = 1.0 / h_por[i];
    h_inv_alpha[i] = 1.0 / h_alpha[i];
    h_vg_m[i] = h_beta[i] / (h_beta[i] - 1.0);
    h_vg_e[i] = (h_beta[i] - 1.0) / h_beta[i];
    h_vg_ib[i] = 1.0 / h_beta[i];
    h_kinf_mat[i] = h_kinfv[i] * (1.0 - h_areafh[i]);
    h_kmac_a[i] = h_kmacv[i] * h_areafh[i];
    h_kv2_mac[i] = (h_areafh[i] > 0.0) ? h_kmacv[i] * h_areafh[i] + h_ksatv[i] * (1.0 - h_areafh[i])
                                       : h_ksatv[i];
    h_d_dinf[i] = h_depth[i] - h_dinf[i];
    h_d_rzd[i] = h_depth[i] - h_rzd[i];
    h_d_dmac[i] = h_depth[i] - h_dmac[i];
    h_kh_k1[i] = h_kmach[i] * h_areafv[i] + h_ksath[i] * (1.0 - h_areafv[i]);
  }
  int32_t *h_ei = carve<int32_t>(hp, NED), *h_ek = carve<int32_t>(hp, NED);
  double *h_einvd = carve<double>(hp, NED), *h_elen = carve<double>(hp, NED);
  double *h_einvr = carve<double>(hp, NED);
  int32_t *h_emap = carve<int32_t>(hp, 3 * NE);
  if (nedge) {
    std::memcpy(h_ei, e_i.data(), sizeof(int32_t) * nedge);
    std::memcpy(h_ek, e_k.data(), sizeof(int32_t) * nedge);
    std::memcpy(h_einvd, e_invdist.data(), sizeof(double) * nedge);
    std::memcpy(h_elen, e_len.data(), sizeof(double) * nedge);
    std::memcpy(h_einvr, e_invrough.data(), sizeof(double) * nedge);
  }
  std::memcpy(h_emap, emap.data(), sizeof(int32_t) * 3 * ne);

  // ---- device allocations ----
  if (cudaMalloc(&c->d_static, sbytes) != cudaSuccess) {
    pihm_gpu_destroy(c);
    return PIHM_GPU_ERR_NOMEM;
  }
  c->static_bytes = sbytes;
  if (cudaMemcpy(c->d_static, host.data(), sbytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    pihm_gpu_destroy(c);
    return PIHM_GPU_ERR_CUDA;
  }
  char *base = host.data();
  char *dbase = (char *)c->d_static;
  auto dev = [&](const void *h) { return (void *)(dbase + ((const char *)h - base)); };
  DevMesh &m = c->m;
  m.ne = ne;
  m.nr = nr;
  m.nbank = nbank;
  m.surf_mode = surf_mode;
  m.riv_mode = riv_mode;
  m.dt = stepsize;
  m.area = (double *)dev(h_area); m.zmin = (double *)dev(h_zmin); m.zmax = (double *)dev(h_zmax);
  m.depth = (double *)dev(h_depth); m.ksath = (double *)dev(h_ksath); m.ksatv = (double *)dev(h_ksatv);
  m.kinfv = (double *)dev(h_kinfv); m.dinf = (double *)dev(h_dinf); m.alpha = (double *)dev(h_alpha);
  m.beta = (double *)dev(h_beta); m.porosity = (double *)dev(h_por); m.dmac = (double *)dev(h_dmac);
  m.kmach = (double *)dev(h_kmach); m.kmacv = (double *)dev(h_kmacv); m.areafv = (double *)dev(h_areafv);
  m.areafh = (double *)dev(h_areafh); m.rough = (double *)dev(h_rough); m.rzd = (double *)dev(h_rzd);
  m.edge = (double *)dev(h_edge); m.nabrdist = (double *)dev(h_dist);
  m.nabr_x = (double *)dev(h_nx); m.nabr_y = (double *)dev(h_ny);
  m.den_x = (double *)dev(h_denx); m.den_y = (double *)dev(h_deny);
  m.nb = (int32_t *)dev(h_nb); m.bctype = (int32_t *)dev(h_bct);
  m.bank_slot = (int32_t *)dev(h_bslot); m.bank_elem = (int32_t *)dev(h_belem);
  m.down = (int32_t *)dev(h_down); m.left = (int32_t *)dev(h_left); m.right = (int32_t *)dev(h_right);
  m.intrpl_ord = (int32_t *)dev(h_ord); m.bctype_riv = (int32_t *)dev(h_rbct);
  m.r_area = (double *)dev(h_rarea); m.r_zmin = (double *)dev(h_rzmin); m.r_zmax = (double *)dev(h_rzmax);
  m.r_zbed = (double *)dev(h_rzbed); m.r_node_zmax = (double *)dev(h_rnz);
  m.r_dist_left = (double *)dev(h_rdl); m.r_dist_right = (double *)dev(h_rdr);
  m.r_depth = (double *)dev(h_rdep); m.r_coeff = (double *)dev(h_rco); m.r_length = (double *)dev(h_rlen);
  m.r_width = (double *)dev(h_rwid); m.r_rough = (double *)dev(h_rrough); m.r_cwr = (double *)dev(h_rcwr);
  m.r_ksath = (double *)dev(h_rkh); m.r_ksatv = (double *)dev(h_rkv); m.r_bedthick = (double *)dev(h_rbed);
  m.r_porosity = (double *)dev(h_rpor);
  m.up_ptr = (int32_t *)dev(h_upp); m.up_idx = (int32_t *)dev(h_upi);
  c->d_perm = (int32_t *)dev(h_permd);
  m.inv_area = (double *)dev(h_inv_area); m.inv_por = (double *)dev(h_inv_por);
  m.inv_alpha = (double *)dev(h_inv_alpha); m.vg_m = (double *)dev(h_vg_m);
  m.vg_e = (double *)dev(h_vg_e); m.vg_ib = (double *)dev(h_vg_ib);
  m.kinf_mat = (double *)dev(h_kinf_mat); m.kmac_a = (double *)dev(h_kmac_a);
  m.kv2_mac = (double *)dev(h_kv2_mac); m.d_dinf = (double *)dev(h_d_dinf);
  m.d_rzd = (double *)dev(h_d_rzd); m.d_dmac = (double *)dev(h_d_dmac);
  m.kh_k1 = (double *)dev(h_kh_k1);
  m.nedge = nedge;
  m.e_i = (int32_t *)dev(h_ei); m.e_k = (int32_t *)dev(h_ek);
  m.e_invdist = (double *)dev(h_einvd); m.e_len = (double *)dev(h_elen);
  m.e_invrough = (double *)dev(h_einvr);
  m.emap = (int32_t *)dev(h_emap);

  // dynamic block: inputs, scratch, diagnostics, staging, error word
  size_t dbytes = 0;
  dbytes += 4 * carve_size<double>(NE);       // pcpdrp, edir, ett, ws0
  dbytes += carve_size<double>(3 * NE);       // elem_bc
  dbytes += carve_size<double>(NR);           // river_bc
  dbytes += 4 * carve_size<double>(NE);       // surfh, head, effk, gradmag
  dbytes += carve_size<double>(11 * NR);      // rivflow
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
  m.eflux_ovl = carve<double>(dp, NED); m.eflux_sub = carve<double>(dp, NED);
  m.bank_part = carve<double>(dp, 8 * NB);
  m.d_ovl = carve<double>(dp, 3 * NE); m.d_sub = carve<double>(dp, 3 * NE);
  m.d_infil = carve<double>(dp, NE); m.d_rechg = carve<double>(dp, NE); m.d_et = carve<double>(dp, 5 * NE);
  c->d_stage_in = carve<double>(dp, c->neq);
  c->d_stage_out = carve<double>(dp, c->neq);
  m.err = carve<unsigned int>(dp, 1);
  m.diag = 0;
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

void pihm_gpu_destroy(pihm_gpu_ctx *c) {
  if (!c) return;
  free_profiler(c->prof);
  if (c->d_static) cudaFree(c->d_static);
  if (c->d_dyn) cudaFree(c->d_dyn);
  std::free(c->h_perm);
  std::free(c->h_iperm);
  delete c;
}

int pihm_gpu_set_stream(pihm_gpu_ctx *c, void *stream) {
  if (!c) return PIHM_GPU_ERR_ARG;
  c->stream = (cudaStream_t)stream;
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

int pihm_gpu_set_ws0_surf(pihm_gpu_ctx *c, const double *ws0) {
  if (!c || !ws0) return PIHM_GPU_ERR_ARG;
  return upload_elem(c, ws0, (double *)c->m.ws0_surf, 1, 1);
}

int pihm_gpu_set_river_edge_ovlflow(pihm_gpu_ctx *c, const double *ovl) {
  if (!c || !ovl) return PIHM_GPU_ERR_ARG;
  if (!c->nr) return PIHM_GPU_OK;
  // the carried value of element e's river edge is -rivflow[LEFT/RIGHT_SURF2CHANL]
  // of that river (src/river_flow.c:159-182); rebuild those two slots
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
  return cuda_fail(cudaMemcpyAsync(F + LEFT_SURF2CHANL * (size_t)c->nr, slots.data(),
                                   sizeof(double) * c->nr, cudaMemcpyHostToDevice, c->stream)) ?:
         cuda_fail(cudaMemcpyAsync(F + RIGHT_SURF2CHANL * (size_t)c->nr, slots.data() + c->nr,
                                   sizeof(double) * c->nr, cudaMemcpyHostToDevice, c->stream)) ?:
         cuda_fail(cudaStreamSynchronize(c->stream));
}

int pihm_gpu_rhs(pihm_gpu_ctx *c, double t, const double *y, double *ydot) {
  (void)t;
  if (!c || !y || !ydot) return PIHM_GPU_ERR_ARG;
  c->m.diag = c->diag;
  return cuda_fail(launch_rhs(c->m, y, ydot, c->stream, &c->launches, c->prof));
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

int pihm_gpu_rhs_host(pihm_gpu_ctx *c, double t, const double *y_host, double *ydot_host) {
  if (!c || !y_host || !ydot_host) return PIHM_GPU_ERR_ARG;
  const size_t bytes = sizeof(double) * c->neq;
  cudaError_t e = cudaMemcpyAsync(c->d_stage_in, y_host, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    e = launch_permute(c->d_stage_in, c->d_stage_out, c->d_perm, c->ne, c->nr, 1, c->stream);
    c->launches++;
  }
  double *y_int = c->d_stage_out, *ydot_int = c->d_stage_in;
  if (e == cudaSuccess) {
    c->m.diag = c->diag;
    e = launch_rhs(c->m, y_int, ydot_int, c->stream, &c->launches, c->prof);
  }
  if (e == cudaSuccess) {
    e = launch_permute(ydot_int, c->d_stage_out, c->d_perm, c->ne, c->nr, 0, c->stream);
    c->launches++;
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ydot_host, c->d_stage_out, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return PIHM_GPU_ERR_CUDA;
  return pihm_gpu_status(c);
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
