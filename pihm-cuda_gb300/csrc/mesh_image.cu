// Host image of one watershed (mesh_image.h): validation, renumbering,
// edge ownership, bank elements, upstream lists and derived constants.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <queue>
#include <vector>

#include "mesh_image.h"

namespace pihm {

const double *DevMesh::*const kElemMember[EP_COUNT] = {
    &DevMesh::area, &DevMesh::zmin, &DevMesh::zmax, &DevMesh::depth, &DevMesh::ksath, &DevMesh::ksatv,
    &DevMesh::kinfv, &DevMesh::dinf, &DevMesh::alpha, &DevMesh::beta, &DevMesh::porosity, &DevMesh::dmac,
    &DevMesh::kmach, &DevMesh::kmacv, &DevMesh::areafv, &DevMesh::areafh, &DevMesh::rough, &DevMesh::rzd,
    &DevMesh::inv_den_x, &DevMesh::inv_den_y,
    &DevMesh::inv_area, &DevMesh::inv_por, &DevMesh::inv_alpha, &DevMesh::vg_m, &DevMesh::vg_e,
    &DevMesh::vg_ib, &DevMesh::kinf_mat, &DevMesh::kmac_a, &DevMesh::kv2_mac, &DevMesh::d_dinf,
    &DevMesh::d_rzd, &DevMesh::d_dmac, &DevMesh::kh_k1, &DevMesh::inv_depth};
const double *DevMesh::*const kEdgeMember[XP_COUNT] = {&DevMesh::edge, &DevMesh::nabrdist, &DevMesh::nabr_x,
                                                       &DevMesh::nabr_y};
const double *DevMesh::*const kRiverMember[RP_COUNT] = {
    &DevMesh::r_area, &DevMesh::r_zmin, &DevMesh::r_zmax, &DevMesh::r_zbed, &DevMesh::r_node_zmax,
    &DevMesh::r_dist_left, &DevMesh::r_dist_right, &DevMesh::r_depth, &DevMesh::r_coeff, &DevMesh::r_length,
    &DevMesh::r_width, &DevMesh::r_rough, &DevMesh::r_cwr, &DevMesh::r_ksath, &DevMesh::r_ksatv,
    &DevMesh::r_bedthick, &DevMesh::r_porosity, &DevMesh::r_inv_half_len, &DevMesh::r_inv_dist_down,
    &DevMesh::r_inv_dist_left, &DevMesh::r_inv_dist_right, &DevMesh::r_inv_bedthick, &DevMesh::r_ovl_coef,
    &DevMesh::r_geo0, &DevMesh::r_geo1, &DevMesh::r_geo2, &DevMesh::r_geo3, &DevMesh::r_geo4};

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

}  // namespace

int build_image(const pihm_gpu_mesh *g, int surf_mode, int riv_mode, double stepsize, int order,
                SystemImage *im) {
  if (!g || !im) return PIHM_GPU_ERR_ARG;
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
  im->ne = ne;
  im->nr = nr;

  // ---- renumbering ----
  std::vector<int32_t> &perm = im->perm, &iperm = im->iperm;
  perm.resize(ne);
  if (order == PIHM_GPU_ORDER_RCM) perm = rcm_order(ne, g->nabr);
  else std::iota(perm.begin(), perm.end(), 0);
  iperm.assign(ne, 0);
  for (int i = 0; i < ne; i++) iperm[perm[i]] = i;

  // bank elements (with at least one river edge), internal order
  im->bank_slot.assign(ne, -1);
  im->bank_elem.clear();
  for (int i = 0; i < ne; i++) {
    int r = perm[i];
    for (int j = 0; j < 3; j++)
      if (g->nabr[3 * r + j] < 0) {
        im->bank_slot[i] = (int32_t)im->bank_elem.size();
        im->bank_elem.push_back(i);
        break;
      }
  }
  im->nbank = (int)im->bank_elem.size();
  // upstream lists (CSR) in reference order
  std::vector<int32_t> &up_ptr = im->up_ptr, &up_idx = im->up_idx;
  up_ptr.assign(nr + 1, 0);
  for (int s = 0; s < nr; s++)
    if (g->down[s] > 0) up_ptr[g->down[s]]++;
  for (int s = 0; s < nr; s++) up_ptr[s + 1] += up_ptr[s];
  up_idx.assign(up_ptr[nr], 0);
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
  im->emap.assign(3 * (size_t)ne, 0);
  im->e_i.clear();
  im->e_k.clear();
  im->e_invdist.clear();
  im->e_subk.clear();
  im->e_ovlk.clear();
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
      const int e = (int)im->e_i.size();
      im->e_i.push_back(i);
      im->e_k.push_back(k);
      // the edge's constant factors: 1/distance, and the products the two
      // flux formulas multiply by, edge/(2 distance) for the Darcy flux
      // (avg_ksat grad_h avg_h edge with avg_ksat a mean and grad_h a
      // difference over the distance) and edge/(distance avg_rough) for the
      // Manning flux (src/lat_flow.c:279-338)
      const double invdist = 1.0 / g->nabrdist[3 * ri + j], len = g->edge[3 * ri + j];
      im->e_invdist.push_back(invdist);
      im->e_subk.push_back(0.5 * len * invdist);
      im->e_ovlk.push_back(len * invdist / (0.5 * (g->rough[ri] + g->rough[rk])));
      im->emap[(size_t)j * ne + i] = e + 1;
      if (sym) im->emap[(size_t)jr * ne + k] = -(e + 1);
    }
  }
  im->nedge = (int)im->e_i.size();

  // ---- element planes ----
  const double *src[EP_DEN_X] = {g->area, g->zmin, g->zmax, g->depth, g->ksath, g->ksatv, g->kinfv,
                                 g->dinf, g->alpha, g->beta, g->porosity, g->dmac, g->kmach, g->kmacv,
                                 g->areafv, g->areafh, g->rough, g->rzd};
  for (int k = 0; k < EP_DEN_X; k++) {
    im->el[k].resize(ne);
    for (int i = 0; i < ne; i++) im->el[k][i] = src[k][perm[i]];
  }
  const double *esrc[XP_COUNT] = {g->edge, g->nabrdist, g->nabr_x, g->nabr_y};
  for (int k = 0; k < XP_COUNT; k++) {
    im->ed[k].resize(3 * (size_t)ne);
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < ne; i++) im->ed[k][(size_t)j * ne + i] = esrc[k][3 * perm[i] + j];
  }
  for (int k = EP_DEN_X; k < EP_COUNT; k++) im->el[k].resize(ne);
  const std::vector<double> &nx = im->ed[XP_NABR_X], &ny = im->ed[XP_NABR_Y];
  for (int i = 0; i < ne; i++) {
    // reciprocals of the denominators of DhByDl (src/lat_flow.c:239-246):
    // l2[2](l1[1]-l1[0]) + l2[1](l1[0]-l1[2]) + l2[0](l1[2]-l1[1]) for
    // (l1,l2) = (y,x) and (x,y)
    const double x0 = nx[i], x1 = nx[ne + i], x2 = nx[2 * (size_t)ne + i];
    const double y0 = ny[i], y1 = ny[ne + i], y2 = ny[2 * (size_t)ne + i];
    im->el[EP_DEN_X][i] = 1.0 / (x2 * (y1 - y0) + x1 * (y0 - y2) + x0 * (y2 - y1));
    im->el[EP_DEN_Y][i] = 1.0 / (y2 * (x1 - x0) + y1 * (x0 - x2) + y0 * (x2 - x1));
  }
  // derived element constants (see DevMesh); same expressions as the
  // reference's inline ones, evaluated without contraction
  std::vector<double> *e = im->el;
  for (int i = 0; i < ne; i++) {
    const double area = e[EP_AREA][i], por = e[EP_POROSITY][i], alpha = e[EP_ALPHA][i];
    const double beta = e[EP_BETA][i], kinfv = e[EP_KINFV][i], areafh = e[EP_AREAFH][i];
    const double kmacv = e[EP_KMACV][i], ksatv = e[EP_KSATV][i], depth = e[EP_DEPTH][i];
    e[EP_INV_AREA][i] = 1.0 / area;
    e[EP_INV_POR][i] = 1.0 / por;
    e[EP_INV_ALPHA][i] = 1.0 / alpha;
    e[EP_VG_M][i] = beta / (beta - 1.0);
    e[EP_VG_E][i] = (beta - 1.0) / beta;
    e[EP_VG_IB][i] = 1.0 / beta;
    e[EP_KINF_MAT][i] = kinfv * (1.0 - areafh);
    e[EP_KMAC_A][i] = kmacv * areafh;
    e[EP_KV2_MAC][i] = (areafh > 0.0) ? kmacv * areafh + ksatv * (1.0 - areafh) : ksatv;
    e[EP_D_DINF][i] = depth - e[EP_DINF][i];
    e[EP_D_RZD][i] = depth - e[EP_RZD][i];
    e[EP_D_DMAC][i] = depth - e[EP_DMAC][i];
    e[EP_KH_K1][i] = e[EP_KMACH][i] * e[EP_AREAFV][i] + e[EP_KSATH][i] * (1.0 - e[EP_AREAFV][i]);
    e[EP_INV_DEPTH][i] = 1.0 / depth;
  }
  im->nb.resize(3 * (size_t)ne);
  im->bct.resize(3 * (size_t)ne);
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < ne; i++) {
      int nb = g->nabr[3 * perm[i] + j];
      im->nb[(size_t)j * ne + i] = nb > 0 ? iperm[nb - 1] : (nb < 0 ? -1 - (-nb - 1) : kBoundary);
      im->bct[(size_t)j * ne + i] = g->bc_type[3 * perm[i] + j];
    }

  // ---- rivers (reference order) ----
  im->down.resize(nr);
  im->left.resize(nr);
  im->right.resize(nr);
  im->ord.resize(nr);
  im->rbct.resize(nr);
  for (int s = 0; s < nr; s++) {
    im->down[s] = g->down[s];
    im->left[s] = iperm[g->leftele[s] - 1];
    im->right[s] = iperm[g->rightele[s] - 1];
    im->ord[s] = g->intrpl_ord[s];
    im->rbct[s] = g->riverbc_type[s];
  }
  const double *rsrc[RP_COUNT] = {g->riv_area, g->riv_zmin, g->riv_zmax, g->riv_zbed, g->riv_node_zmax,
                                  g->riv_dist_left, g->riv_dist_right, g->riv_depth, g->riv_coeff,
                                  g->riv_length, g->riv_width, g->riv_rough, g->riv_cwr, g->riv_ksath,
                                  g->riv_ksatv, g->riv_bedthick, g->riv_porosity};
  for (int k = 0; k < RP_INV_HALF_LEN; k++) im->rv[k].assign(rsrc[k], rsrc[k] + nr);
  // reciprocals of the static distances the river fluxes divide by, and the
  // weir coefficient of OvlFlowElemToRiver, cwr 2 sqrt(2 g) length / 3
  // (src/river_flow.c:185-255, 257-331, 333-390, 429-518)
  for (int k = RP_INV_HALF_LEN; k < RP_COUNT; k++) im->rv[k].assign(nr, 0.0);
  for (int s = 0; s < nr; s++) {
    const double len = g->riv_length[s];
    im->rv[RP_INV_HALF_LEN][s] = 1.0 / (0.5 * len);
    if (g->down[s] > 0) im->rv[RP_INV_DIST_DOWN][s] = 1.0 / (0.5 * (len + g->riv_length[g->down[s] - 1]));
    im->rv[RP_INV_DIST_LEFT][s] = 1.0 / g->riv_dist_left[s];
    im->rv[RP_INV_DIST_RIGHT][s] = 1.0 / g->riv_dist_right[s];
    im->rv[RP_INV_BEDTHICK][s] = 1.0 / g->riv_bedthick[s];
    im->rv[RP_OVL_COEF][s] = g->riv_cwr[s] * 2.0 * std::sqrt(2.0 * kGrav) * len / 3.0;
    // the coefficient-only factors of RivCsArea / RivPerim
    // (src/river_flow.c:520-583) for the segment's shape
    const double c = g->riv_coeff[s];
    double *geo[5] = {&im->rv[RP_GEO0][s], &im->rv[RP_GEO1][s], &im->rv[RP_GEO2][s],
                      &im->rv[RP_GEO3][s], &im->rv[RP_GEO4][s]};
    switch (g->intrpl_ord[s]) {
      case kRectangle:  // area d c, perimeter 2 d + c
        *geo[0] = c;
        break;
      case kTriangle:  // area d^2 / c, perimeter 2 d sqrt(1 + c^2) / c
        *geo[0] = 1.0 / c;
        *geo[1] = 2.0 * std::sqrt(1.0 + c * c) / c;
        break;
      case kQuadratic:  // area 4 d^1.5 / (3 sqrt c), perimeter
                        // sqrt(d (1 + 4 c d) / c) + ln(2 sqrt(c d) + sqrt(1 + 4 c d)) / (2 c)
        *geo[0] = 4.0 / (3.0 * std::sqrt(c));
        *geo[1] = 4.0 * c;
        *geo[2] = 1.0 / c;
        *geo[3] = 1.0 / (2.0 * c);
        *geo[4] = 2.0 * std::sqrt(c);
        break;
      case kCubic: {  // area 3 d^(4/3) / (2 c^(1/3)), perimeter
                      // 2 (sqrt(d (1 + 9 c^(2/3) d)) / 3 + ln(3 c^(1/3) sqrt(d) + sqrt(1 + 9 c^(2/3) d)) / (9 c^(1/3)))
        const double c13 = std::pow(c, 1.0 / 3.0), c23 = std::pow(c, 2.0 / 3.0);
        *geo[0] = 3.0 / (2.0 * c13);
        *geo[1] = 9.0 * c23;
        *geo[2] = 3.0 * c13;
        *geo[3] = 1.0 / (9.0 * c13);
        break;
      }
    }
  }
  return PIHM_GPU_OK;
}

}  // namespace pihm
