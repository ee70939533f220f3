// Host image of one watershed in the library's internal layout: validation,
// locality renumbering, interior-edge ownership, bank elements, the upstream
// river lists and the element constants derived once at load.  A
// single-watershed context uploads one image into its own device block
// (context.cu); the batch engine places many images into ranges of a shared
// arena, translating their indices (batch.cu).
#pragma once

#include <cstdint>
#include <vector>

#include "pihm_internal.h"

namespace pihm {

// Element planes [ne], in DevMesh member order.
enum ElemPlane {
  EP_AREA = 0, EP_ZMIN, EP_ZMAX, EP_DEPTH, EP_KSATH, EP_KSATV, EP_KINFV, EP_DINF, EP_ALPHA, EP_BETA,
  EP_POROSITY, EP_DMAC, EP_KMACH, EP_KMACV, EP_AREAFV, EP_AREAFH, EP_ROUGH, EP_RZD,
  EP_DEN_X, EP_DEN_Y,
  EP_INV_AREA, EP_INV_POR, EP_INV_ALPHA, EP_VG_M, EP_VG_E, EP_VG_IB, EP_KINF_MAT, EP_KMAC_A,
  EP_KV2_MAC, EP_D_DINF, EP_D_RZD, EP_D_DMAC, EP_KH_K1, EP_INV_DEPTH,
  EP_COUNT
};
// Edge planes [3][ne] of doubles.
enum EdgePlane { XP_EDGE = 0, XP_NABRDIST, XP_NABR_X, XP_NABR_Y, XP_COUNT };
// River planes [nr] of doubles.
enum RiverPlane {
  RP_AREA = 0, RP_ZMIN, RP_ZMAX, RP_ZBED, RP_NODE_ZMAX, RP_DIST_LEFT, RP_DIST_RIGHT, RP_DEPTH,
  RP_COEFF, RP_LENGTH, RP_WIDTH, RP_ROUGH, RP_CWR, RP_KSATH, RP_KSATV, RP_BEDTHICK, RP_POROSITY,
  RP_INV_HALF_LEN, RP_INV_DIST_DOWN, RP_INV_DIST_LEFT, RP_INV_DIST_RIGHT, RP_INV_BEDTHICK, RP_OVL_COEF,
  RP_GEO0, RP_GEO1, RP_GEO2, RP_GEO3, RP_GEO4,
  RP_COUNT
};

extern const double *DevMesh::*const kElemMember[EP_COUNT];
extern const double *DevMesh::*const kEdgeMember[XP_COUNT];
extern const double *DevMesh::*const kRiverMember[RP_COUNT];

struct SystemImage {
  int ne = 0, nr = 0, nbank = 0, nedge = 0;
  std::vector<int32_t> perm, iperm;            // perm[internal] = reference element
  std::vector<double> el[EP_COUNT];            // [ne]
  std::vector<double> ed[XP_COUNT];            // [3*ne], plane j at j*ne
  std::vector<int32_t> nb, bct, emap;          // [3*ne]; nb: >= 0 element, -1-s river, kBoundary
  std::vector<int32_t> bank_slot, bank_elem;   // [ne] (-1: no river edge), [nbank]
  std::vector<int32_t> e_i, e_k;               // [nedge]
  std::vector<double> e_invdist, e_subk, e_ovlk;
  std::vector<int32_t> down, left, right, ord, rbct;  // [nr]; down as in the reference (1-based or BC code)
  std::vector<double> rv[RP_COUNT];            // [nr]
  std::vector<int32_t> up_ptr, up_idx;         // [nr+1], [up_ptr[nr]]
};

// Validate a watershed and build its image.  Returns PIHM_GPU_OK or an error
// code of pihm_gpu.h.
int build_image(const pihm_gpu_mesh *g, int surf_mode, int riv_mode, double stepsize, int order,
                SystemImage *im);

}  // namespace pihm
