// Device side of the batch engine: the arena that holds many watersheds'
// meshes, CVODE vectors and right-hand-side staging, and the per-round
// "program" that applies each watershed's queued vector operations.
//
// One round executes, for every watershed that is waiting on the device, the
// element-wise N_Vector operations its integrator issued since it last
// suspended, followed by the operation it suspended on: a reduction (WRMS
// norm, dot product, max norm, min) or a right-hand-side evaluation.  The
// program kernel runs all the watersheds' programs in one launch; the
// right-hand side then runs once over the whole arena for the watersheds that
// asked for it.
//
// Each watershed's vectors are contiguous ranges of the vector slots, and the
// program kernel gives watershed s the same number of blocks, the same
// grid-stride element order and the same block and last-block combination as
// the single-vector reduction kernel over a vector of that length.  Together
// with the shared element-wise arithmetic (nv_ops.cuh) and the shared
// right-hand-side kernels, a watershed's trajectory in a batch is bit-for-bit
// the one the single-watershed library computes for it, whatever else shares
// the batch.
#pragma once

#include <cstdint>

#include "pihm_internal.h"

namespace pihm {
namespace batch {

constexpr int kVecSlots = 24;    // CVODE vectors per watershed (21 used)
constexpr int kMaxProgOps = 48;  // element-wise operations queued per round and watershed

// Operation codes below 32 are the element-wise N_Vector operations (EwOp).
enum : uint8_t {
  OP_STAGE_IN = 32,  // rhs_in[global position of entry j] = x[j]
  OP_STAGE_OUT,      // z[j] = rhs_out[global position of entry j]
  OP_FORCING,        // element j: pcpdrp = a, edir = b, ett = c
  OP_WS0,            // element j: ws0_surf = x[j]    (post-step update)
  OP_RECORD          // rec[i0] = rivflow[DOWN_CHANL2CHANL][segment i1]
};

struct Op {
  uint8_t code, x, y, z;  // vector slots
  int32_t i0, i1, pad;
  double a, b, c;
};

// A watershed's place in the arena.
struct SysInfo {
  int64_t off;                   // first entry of its vectors in every slot
  int32_t neq, ne, nr, eoff, roff;
  int32_t nblk;                  // blocks of its reductions (red_grid_for(neq))
  int64_t rec_off;               // first entry of its hydrograph record
};

// One watershed's work in one round.
struct RoundSys {
  int32_t sys, prog_off, prog_len;
  int32_t red;      // -1: none, else a pihm_nv::RedOp (R_DOT, R_MAXABS, R_WSQ, R_MIN)
  int32_t bstart;   // first block of the program kernel that works on it
  uint8_t rx, ry, pad0, pad1;
};

struct DeviceArena {
  DevMesh m;            // capacities in ne, nr, nedge, nbank; launch extents = high-water marks
  double *vec;          // [kVecSlots][neq_cap]
  int64_t neq_cap;
  double *rhs_in, *rhs_out;  // [3 ne_cap + 2 nr_cap], the single-watershed state layout
  SysInfo *sysinfo;     // [max_sys]
  double *partials;     // [max_sys][2 * kMaxBlocks]
  unsigned int *tickets;  // [max_sys]
  double *results;      // [max_sys][2]
  double *rec;          // hydrograph records
  RoundSys *round;      // round list, then the ops, one upload per round
  Op *ops;
  int max_sys;
};

// Run one round's programs: nrs watersheds over nblocks blocks in total.
// variant 0, 1, 2: entries a thread keeps in flight (1, 2, 4); same results.
constexpr int kProgramVariants = 3;
cudaError_t launch_program(const DeviceArena &a, int nrs, int nblocks, int variant, cudaStream_t st);

// One host-to-device copy of a watershed's upload: bytes from src (host
// memory) to dst (arena).
struct CopyDesc {
  const void *src;
  void *dst;
  uint64_t bytes;
};
// Copies every descriptor with one kernel that reads the host memory
// directly.  Only for a device that can access pageable host memory
// (cudaDevAttrPageableMemoryAccess): desc and every src may be ordinary
// host allocations, and they must stay valid until the stream has passed
// the kernel.
cudaError_t launch_gather_host(const CopyDesc *desc, int n, uint64_t max_bytes, cudaStream_t st);

}  // namespace batch


}  // namespace pihm
