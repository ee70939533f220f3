// Derived from SUNDIALS 2.7.0 (CVODE 2.9.0). Copyright (c) 2002-2016,
// Lawrence Livermore National Security; produced at the Lawrence Livermore
// National Laboratory (UCRL-CODE-155951). Redistributed under the SUNDIALS
// BSD-3 licence: its full text, conditions and disclaimer are in
// pihm-cuda_gb300/NOTICE.SUNDIALS.
//
// Device-resident N_Vector (SUNDIALS 2.7 / CVODE 2.9 operations table) for
// sm_103a.  See include/pihm_nvector.h for the contract.
//
// Element-wise kernels use __dmul_rn/__dadd_rn so the compiler cannot fuse a
// multiply and an add: every element equals what the serial N_Vector computes
// (cvode/src/nvec_ser/nvector_serial.c:421-1060), including its special cases
// (a == 1, b == -1, a == b, ...) which change the rounding.
//
// Reductions: each block reduces a fixed, grid-strided slice of the vector
// with a warp-shuffle tree, writes one partial, and the last block to finish
// (atomic ticket) combines the partials in index order.  The grid size depends
// only on the length, so the result is identical from run to run.
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

#include "pihm_nvector.h"
#include "nv_ops.cuh"

namespace pihm_nv {

constexpr double kBigReal = DBL_MAX;

struct Scratch {
  double *partials = nullptr;   // [kMaxBlocks]
  unsigned int *ticket = nullptr;
  double *result = nullptr;     // [2] value, flag
  double *slots = nullptr;      // [2 * PIHM_NV_SLOTS] value, flag per slot
  double *host = nullptr;       // pinned [2 + 2 * PIHM_NV_SLOTS + 1]
};

// Scratch layout: partial values [kMaxBlocks], partial flags [kMaxBlocks],
// result [2], ticket, one spare, slots [2 * PIHM_NV_SLOTS].
constexpr size_t kScratchDoubles = 2 * kMaxBlocks + 4 + 2 * PIHM_NV_SLOTS;
constexpr size_t kHostDoubles = 2 + 2 * PIHM_NV_SLOTS + 1;

static int scratch_alloc(Scratch &s) {
  void *p = nullptr;
  if (cudaMalloc(&p, sizeof(double) * kScratchDoubles) != cudaSuccess) return -1;
  char *c = (char *)p;
  s.partials = (double *)c;
  s.result = (double *)(c + sizeof(double) * 2 * kMaxBlocks);
  s.ticket = (unsigned int *)(c + sizeof(double) * (2 * kMaxBlocks + 2));
  s.slots = (double *)(c + sizeof(double) * (2 * kMaxBlocks + 4));
  if (cudaMemset(p, 0, sizeof(double) * kScratchDoubles) != cudaSuccess) return -1;
  if (cudaMallocHost(&s.host, sizeof(double) * kHostDoubles) != cudaSuccess) return -1;
  return 0;
}

static void scratch_free(Scratch &s) {
  if (s.partials) cudaFree(s.partials);
  if (s.host) cudaFreeHost(s.host);
  s = Scratch();
}

// A vector family: the stream plus reduction scratch, shared by clones.
struct Family {
  cudaStream_t stream;
  Scratch scratch;
  int refs;
};

struct Content {
  long int length;
  int own_data;
  double *data;
  Family *fam;
};

static inline Content *C(N_Vector v) { return (Content *)v->content; }
static inline double *D(N_Vector v) { return C(v)->data; }
static inline long int L(N_Vector v) { return C(v)->length; }
static inline cudaStream_t S(N_Vector v) { return C(v)->fam->stream; }

static inline unsigned grid_for(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  if (b > 16 * 152) b = 16 * 152;
  return (unsigned)(b > 0 ? b : 1);
}

// ---------------------------------------------------------------------------
// element-wise kernels
// ---------------------------------------------------------------------------
template <int OP>
__global__ void k_ew(long long n, double a, double b, const double *__restrict__ x,
                     const double *__restrict__ y, double *z) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double xv = ew_reads_x(OP) ? x[i] : 0.0;
    const double yv = ew_reads_y(OP) ? y[i] : 0.0;
    const double zv = ew_reads_z(OP) ? z[i] : 0.0;
    z[i] = ew_eval<OP>(a, b, xv, yv, zv);
  }
}

template <int OP>
static int ew(long long n, double a, double b, const double *x, const double *y, double *z,
              cudaStream_t st) {
  if (n <= 0) return 0;
  k_ew<OP><<<grid_for(n), kThreads, 0, st>>>(n, a, b, x, y, z);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

// One element-wise call after the serial N_Vector's case analysis.
static int ew_call(const EwCall<const double *> &c, long long n, cudaStream_t st) {
  double *z = const_cast<double *>(c.z);
  switch (c.op) {
    case EW_LIN: return ew<EW_LIN>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_LIN1: return ew<EW_LIN1>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_LIN2: return ew<EW_LIN2>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_SUM: return ew<EW_SUM>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_DIFF: return ew<EW_DIFF>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_SCALESUM: return ew<EW_SCALESUM>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_SCALEDIFF: return ew<EW_SCALEDIFF>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_AXPY: return ew<EW_AXPY>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_AXPY1: return ew<EW_AXPY1>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_AXPYM1: return ew<EW_AXPYM1>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_SCALE: return ew<EW_SCALE>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_COPY: return ew<EW_COPY>(n, c.a, c.b, c.x, c.y, z, st);
    case EW_NEG: return ew<EW_NEG>(n, c.a, c.b, c.x, c.y, z, st);
    default: return -1;
  }
}

// z = a*x + b*y (cvode/src/nvec_ser/nvector_serial.c:421-506)
static int linear_sum(double a, const double *x, double b, const double *y, double *z, long long n,
                      cudaStream_t st) {
  return ew_call(select_linear_sum<const double *>(a, x, b, y, z), n, st);
}

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
// x, y, w are the operands; m (optional) receives the ConstrMask output and
// z the InvTest output.
template <int OP>
__global__ void __launch_bounds__(kThreads) k_red(long long n, const double *__restrict__ x,
                                                  const double *__restrict__ y, double *__restrict__ z,
                                                  double *partials, double *partials_f,
                                                  unsigned int *ticket, double *result,
                                                  long long wrms_n) {
  __shared__ Pair sh[kThreads / 32];
  __shared__ bool last;
  Pair acc = red_identity<OP>();
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (OP == R_DOT || OP == R_WSQ || OP == R_MAXABS || OP == R_MIN || OP == R_L1) {
    // four grid-stride entries at a time (their loads in flight together),
    // accumulated in grid-stride order
    constexpr int U = 4;
    for (; i0 < n; i0 += U * stride) {
      double xv[U], yv[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const long long i = i0 + u * stride;
        xv[u] = (i < n) ? x[i] : 0.0;
        yv[u] = (i < n && (OP == R_DOT || OP == R_WSQ)) ? y[i] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < U; u++)
        if (i0 + u * stride < n) acc = red_combine<OP>(acc, red_term<OP>(xv[u], yv[u]));
    }
  }
  for (long long i = i0; i < n; i += stride) {
    Pair t = red_identity<OP>();
    if (OP == R_DOT || OP == R_WSQ) t = red_term<OP>(x[i], y[i]);
    else if (OP == R_MAXABS || OP == R_MIN || OP == R_L1) t = red_term<OP>(x[i], 0.0);
    else if (OP == R_WSQ_MASK) {
      if (z[i] > 0.0) { double p = __dmul_rn(x[i], y[i]); t.v = __dmul_rn(p, p); }
    } else if (OP == R_INVTEST) {
      if (x[i] == 0.0) t.f = 1.0;
      else z[i] = div_rn(1.0, x[i]);
    } else if (OP == R_CONSTR) {
      // cvode/src/nvec_ser/nvector_serial.c:813-841: c = x, x = y, m = z
      const double c = x[i], v = y[i];
      double mi = 0.0;
      if (c != 0.0) {
        if (c > 1.5 || c < -1.5) {
          if (__dmul_rn(v, c) <= 0.0) { t.f = 1.0; mi = 1.0; }
        } else if (c > 0.5 || c < -0.5) {
          if (__dmul_rn(v, c) < 0.0) { t.f = 1.0; mi = 1.0; }
        }
      }
      z[i] = mi;
    } else if (OP == R_MINQ) {
      if (y[i] != 0.0) { t.v = div_rn(x[i], y[i]); t.f = 1.0; }
    }
    acc = red_combine<OP>(acc, t);
  }
  acc = red_block<OP>(acc, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = acc.v;
    partials_f[blockIdx.x] = acc.f;
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last block combines the partials in a fixed order
  Pair v = red_identity<OP>();
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    Pair q = {((volatile double *)partials)[b], ((volatile double *)partials_f)[b]};
    v = red_combine<OP>(v, q);
  }
  v = red_block<OP>(v, sh);
  if (threadIdx.x == 0) {
    // wrms_n > 0: the WRMS norm sqrt(sum / n) itself, as N_VWrmsNorm forms it
    result[0] = wrms_n > 0 ? __dsqrt_rn(__ddiv_rn(v.v, (double)wrms_n)) : v.v;
    result[1] = v.f;
    *ticket = 0u;
  }
}

// z = a*x + b*y with a and b formed from device-resident slots: one thread
// of each block forms the coefficients and makes the serial N_Vector's case
// analysis from their values (operand tags 0 = x, 1 = y; ztag 0 when z is x,
// 1 when z is y, 2 otherwise), then the block runs the chosen variant.
template <int OP>
__device__ __forceinline__ void ew_loop(long long n, double a, double b, const double *x, const double *y,
                                        double *z) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double xv = ew_reads_x(OP) ? x[i] : 0.0;
    const double yv = ew_reads_y(OP) ? y[i] : 0.0;
    const double zv = ew_reads_z(OP) ? z[i] : 0.0;
    z[i] = ew_eval<OP>(a, b, xv, yv, zv);
  }
}

__global__ void k_lin_coef(long long n, int ka, int sa, double va, int kb, int sb, double vb, int ztag,
                           const double *x, const double *y, double *z, const double *slots) {
  __shared__ int s_op, s_xt, s_yt;
  __shared__ double s_a, s_b;
  if (threadIdx.x == 0) {
    const double a = coef_value(ka, va, ka == COEF_HOST ? 0.0 : slots[2 * sa]);
    const double b = coef_value(kb, vb, kb == COEF_HOST ? 0.0 : slots[2 * sb]);
    const EwCall<int> c = select_linear_sum<int>(a, 0, b, 1, ztag);
    s_op = c.op;
    s_a = c.a;
    s_b = c.b;
    s_xt = c.x;
    s_yt = c.y;
  }
  __syncthreads();
  const double *px = s_xt == 0 ? x : y, *py = s_yt == 0 ? x : y;
  const double a = s_a, b = s_b;
  switch (s_op) {
    case EW_LIN: ew_loop<EW_LIN>(n, a, b, px, py, z); break;
    case EW_LIN1: ew_loop<EW_LIN1>(n, a, b, px, py, z); break;
    case EW_LIN2: ew_loop<EW_LIN2>(n, a, b, px, py, z); break;
    case EW_SUM: ew_loop<EW_SUM>(n, a, b, px, py, z); break;
    case EW_DIFF: ew_loop<EW_DIFF>(n, a, b, px, py, z); break;
    case EW_SCALESUM: ew_loop<EW_SCALESUM>(n, a, b, px, py, z); break;
    case EW_SCALEDIFF: ew_loop<EW_SCALEDIFF>(n, a, b, px, py, z); break;
    case EW_AXPY: ew_loop<EW_AXPY>(n, a, b, px, py, z); break;
    case EW_AXPY1: ew_loop<EW_AXPY1>(n, a, b, px, py, z); break;
    default: ew_loop<EW_AXPYM1>(n, a, b, px, py, z); break;
  }
}

}  // namespace pihm_nv

namespace pihm_nv {

// Launch a reduction into `scratch` (partials [kMaxBlocks] then flags [kMaxBlocks]
// carved from the caller's buffer), leave the result in result_dev[0..1].
template <int OP>
static int red_launch(long long n, const double *x, const double *y, double *z, double *partials,
                      unsigned int *ticket, double *result_dev, cudaStream_t st, long long wrms_n = 0) {
  const unsigned g = red_grid_for(n);
  k_red<OP><<<g, kThreads, 0, st>>>(n, x, y, z, partials, partials + kMaxBlocks, ticket, result_dev, wrms_n);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

template <int OP>
static int red_family(Family *f, long long n, const double *x, const double *y, double *z, double out[2]) {
  Scratch &s = f->scratch;
  if (red_launch<OP>(n, x, y, z, s.partials, s.ticket, s.result, f->stream)) return -2;
  if (cudaMemcpyAsync(s.host, s.result, sizeof(double) * 2, cudaMemcpyDeviceToHost, f->stream) != cudaSuccess)
    return -2;
  if (cudaStreamSynchronize(f->stream) != cudaSuccess) return -2;
  out[0] = s.host[0];
  out[1] = s.host[1];
  return 0;
}

}  // namespace pihm_nv

using namespace pihm_nv;

extern "C" {

static N_Vector new_empty(Family *fam);

static struct _generic_N_Vector_Ops *make_ops() {
  struct _generic_N_Vector_Ops *o = (struct _generic_N_Vector_Ops *)calloc(1, sizeof(*o));
  o->nvgetvectorid = N_VGetVectorID_PihmGpu;
  o->nvclone = N_VClone_PihmGpu;
  o->nvcloneempty = N_VCloneEmpty_PihmGpu;
  o->nvdestroy = N_VDestroy_PihmGpu;
  o->nvspace = N_VSpace_PihmGpu;
  o->nvgetarraypointer = N_VGetArrayPointer_PihmGpu;
  o->nvsetarraypointer = N_VSetArrayPointer_PihmGpu;
  o->nvlinearsum = N_VLinearSum_PihmGpu;
  o->nvconst = N_VConst_PihmGpu;
  o->nvprod = N_VProd_PihmGpu;
  o->nvdiv = N_VDiv_PihmGpu;
  o->nvscale = N_VScale_PihmGpu;
  o->nvabs = N_VAbs_PihmGpu;
  o->nvinv = N_VInv_PihmGpu;
  o->nvaddconst = N_VAddConst_PihmGpu;
  o->nvdotprod = N_VDotProd_PihmGpu;
  o->nvmaxnorm = N_VMaxNorm_PihmGpu;
  o->nvwrmsnorm = N_VWrmsNorm_PihmGpu;
  o->nvwrmsnormmask = N_VWrmsNormMask_PihmGpu;
  o->nvmin = N_VMin_PihmGpu;
  o->nvwl2norm = N_VWL2Norm_PihmGpu;
  o->nvl1norm = N_VL1Norm_PihmGpu;
  o->nvcompare = N_VCompare_PihmGpu;
  o->nvinvtest = N_VInvTest_PihmGpu;
  o->nvconstrmask = N_VConstrMask_PihmGpu;
  o->nvminquotient = N_VMinQuotient_PihmGpu;
  return o;
}

static N_Vector new_empty(Family *fam) {
  N_Vector v = (N_Vector)calloc(1, sizeof(*v));
  Content *c = (Content *)calloc(1, sizeof(Content));
  if (!v || !c) {
    free(v);
    free(c);
    return nullptr;
  }
  v->ops = make_ops();
  v->content = c;
  c->fam = fam;
  fam->refs++;
  return v;
}

static Family *new_family(void *stream) {
  Family *f = new Family();
  f->stream = (cudaStream_t)stream;
  f->refs = 0;
  if (scratch_alloc(f->scratch)) {
    scratch_free(f->scratch);
    delete f;
    return nullptr;
  }
  return f;
}

N_Vector N_VNew_PihmGpu(long int length, void *stream) {
  if (length < 0) return nullptr;
  Family *f = new_family(stream);
  if (!f) return nullptr;
  N_Vector v = new_empty(f);
  if (!v) return nullptr;
  Content *c = C(v);
  c->length = length;
  c->own_data = 1;
  if (length > 0 && cudaMalloc(&c->data, sizeof(double) * length) != cudaSuccess) {
    N_VDestroy_PihmGpu(v);
    return nullptr;
  }
  return v;
}

N_Vector N_VMake_PihmGpu(long int length, double *dev_data, void *stream) {
  if (length < 0) return nullptr;
  Family *f = new_family(stream);
  if (!f) return nullptr;
  N_Vector v = new_empty(f);
  if (!v) return nullptr;
  C(v)->length = length;
  C(v)->own_data = 0;
  C(v)->data = dev_data;
  return v;
}

double *N_VGetDeviceArrayPointer_PihmGpu(N_Vector v) { return D(v); }
long int N_VGetLength_PihmGpu(N_Vector v) { return L(v); }

int N_VCopyFromHost_PihmGpu(N_Vector v, const double *host) {
  if (cudaMemcpyAsync(D(v), host, sizeof(double) * L(v), cudaMemcpyHostToDevice, S(v)) != cudaSuccess) return -2;
  return cudaStreamSynchronize(S(v)) == cudaSuccess ? 0 : -2;
}

int N_VCopyToHost_PihmGpu(N_Vector v, double *host) {
  if (cudaMemcpyAsync(host, D(v), sizeof(double) * L(v), cudaMemcpyDeviceToHost, S(v)) != cudaSuccess) return -2;
  return cudaStreamSynchronize(S(v)) == cudaSuccess ? 0 : -2;
}

N_Vector_ID N_VGetVectorID_PihmGpu(N_Vector v) {
  (void)v;
  return SUNDIALS_NVEC_CUSTOM;
}

N_Vector N_VCloneEmpty_PihmGpu(N_Vector w) {
  N_Vector v = new_empty(C(w)->fam);
  if (!v) return nullptr;
  C(v)->length = L(w);
  C(v)->own_data = 0;
  C(v)->data = nullptr;
  return v;
}

N_Vector N_VClone_PihmGpu(N_Vector w) {
  N_Vector v = N_VCloneEmpty_PihmGpu(w);
  if (!v) return nullptr;
  if (L(w) > 0) {
    if (cudaMalloc(&C(v)->data, sizeof(double) * L(w)) != cudaSuccess) {
      N_VDestroy_PihmGpu(v);
      return nullptr;
    }
    C(v)->own_data = 1;
  }
  return v;
}

void N_VDestroy_PihmGpu(N_Vector v) {
  if (!v) return;
  Content *c = C(v);
  if (c) {
    if (c->own_data && c->data) cudaFree(c->data);
    Family *f = c->fam;
    if (f && --f->refs == 0) {
      scratch_free(f->scratch);
      delete f;
    }
    free(c);
  }
  free(v->ops);
  free(v);
}

void N_VSpace_PihmGpu(N_Vector v, long int *lrw, long int *liw) {
  *lrw = L(v);
  *liw = 1;
}

double *N_VGetArrayPointer_PihmGpu(N_Vector v) { return D(v); }
void N_VSetArrayPointer_PihmGpu(double *v_data, N_Vector v) {
  if (L(v) > 0) C(v)->data = v_data;
}

void N_VLinearSum_PihmGpu(double a, N_Vector x, double b, N_Vector y, N_Vector z) {
  linear_sum(a, D(x), b, D(y), D(z), L(x), S(z));
}
void N_VConst_PihmGpu(double c, N_Vector z) { ew<EW_CONST>(L(z), c, 0, nullptr, nullptr, D(z), S(z)); }
void N_VProd_PihmGpu(N_Vector x, N_Vector y, N_Vector z) { ew<EW_PROD>(L(x), 0, 0, D(x), D(y), D(z), S(z)); }
void N_VDiv_PihmGpu(N_Vector x, N_Vector y, N_Vector z) { ew<EW_DIV>(L(x), 0, 0, D(x), D(y), D(z), S(z)); }
void N_VScale_PihmGpu(double c, N_Vector x, N_Vector z) {
  // cvode/src/nvec_ser/nvector_serial.c:559-584
  ew_call(select_scale<const double *>(c, D(x), D(z)), L(x), S(z));
}
void N_VAbs_PihmGpu(N_Vector x, N_Vector z) { ew<EW_ABS>(L(x), 0, 0, D(x), nullptr, D(z), S(z)); }
void N_VInv_PihmGpu(N_Vector x, N_Vector z) { ew<EW_INV>(L(x), 0, 0, D(x), nullptr, D(z), S(z)); }
void N_VAddConst_PihmGpu(N_Vector x, double b, N_Vector z) {
  ew<EW_ADDCONST>(L(x), 0, b, D(x), nullptr, D(z), S(z));
}
void N_VCompare_PihmGpu(double c, N_Vector x, N_Vector z) {
  ew<EW_COMPARE>(L(x), c, 0, D(x), nullptr, D(z), S(z));
}

double N_VDotProd_PihmGpu(N_Vector x, N_Vector y) {
  double r[2] = {NAN, 0};
  red_family<R_DOT>(C(x)->fam, L(x), D(x), D(y), nullptr, r);
  return r[0];
}
double N_VMaxNorm_PihmGpu(N_Vector x) {
  double r[2] = {NAN, 0};
  red_family<R_MAXABS>(C(x)->fam, L(x), D(x), nullptr, nullptr, r);
  return r[0];
}
double N_VWrmsNorm_PihmGpu(N_Vector x, N_Vector w) {
  double r[2] = {NAN, 0};
  red_family<R_WSQ>(C(x)->fam, L(x), D(x), D(w), nullptr, r);
  return sqrt(r[0] / (double)L(x));
}
double N_VWrmsNormMask_PihmGpu(N_Vector x, N_Vector w, N_Vector id) {
  double r[2] = {NAN, 0};
  red_family<R_WSQ_MASK>(C(x)->fam, L(x), D(x), D(w), D(id), r);
  return sqrt(r[0] / (double)L(x));
}
double N_VMin_PihmGpu(N_Vector x) {
  double r[2] = {NAN, 0};
  red_family<R_MIN>(C(x)->fam, L(x), D(x), nullptr, nullptr, r);
  return r[0];
}
double N_VWL2Norm_PihmGpu(N_Vector x, N_Vector w) {
  double r[2] = {NAN, 0};
  red_family<R_WSQ>(C(x)->fam, L(x), D(x), D(w), nullptr, r);
  return sqrt(r[0]);
}
double N_VL1Norm_PihmGpu(N_Vector x) {
  double r[2] = {NAN, 0};
  red_family<R_L1>(C(x)->fam, L(x), D(x), nullptr, nullptr, r);
  return r[0];
}
int N_VInvTest_PihmGpu(N_Vector x, N_Vector z) {
  double r[2] = {0, 1};
  red_family<R_INVTEST>(C(x)->fam, L(x), D(x), nullptr, D(z), r);
  return r[1] == 0.0;
}
int N_VConstrMask_PihmGpu(N_Vector c, N_Vector x, N_Vector m) {
  double r[2] = {0, 1};
  red_family<R_CONSTR>(C(x)->fam, L(x), D(c), D(x), D(m), r);
  return r[1] == 0.0;
}
double N_VMinQuotient_PihmGpu(N_Vector num, N_Vector denom) {
  double r[2] = {NAN, 0};
  red_family<R_MINQ>(C(num)->fam, L(num), D(num), D(denom), nullptr, r);
  return (r[1] != 0.0) ? r[0] : kBigReal;
}

// ---------------------------------------------------------------------------
// device-resident scalars
// ---------------------------------------------------------------------------
int N_VDotProdSlot_PihmGpu(N_Vector x, N_Vector y, int slot) {
  if (!x || !y || slot < 0 || slot >= PIHM_NV_SLOTS) return -1;
  Scratch &s = C(x)->fam->scratch;
  return red_launch<R_DOT>(L(x), D(x), D(y), nullptr, s.partials, s.ticket, s.slots + 2 * slot, S(x));
}

int N_VWrmsNormSlot_PihmGpu(N_Vector x, N_Vector w, int slot) {
  if (!x || !w || slot < 0 || slot >= PIHM_NV_SLOTS || L(x) <= 0) return -1;
  Scratch &s = C(x)->fam->scratch;
  return red_launch<R_WSQ>(L(x), D(x), D(w), nullptr, s.partials, s.ticket, s.slots + 2 * slot, S(x), L(x));
}

int N_VLinearSumCoef_PihmGpu(const pihm_nv_coef *a, N_Vector x, const pihm_nv_coef *b, N_Vector y,
                             N_Vector z) {
  if (!a || !b || !x || !y || !z) return -1;
  for (const pihm_nv_coef *c : {a, b})
    if (c->kind < PIHM_NV_COEF_HOST || c->kind > PIHM_NV_COEF_NEG_INV_INV ||
        (c->kind != PIHM_NV_COEF_HOST && (c->slot < 0 || c->slot >= PIHM_NV_SLOTS)))
      return -1;
  const long long n = L(x);
  if (a->kind == PIHM_NV_COEF_HOST && b->kind == PIHM_NV_COEF_HOST)
    return linear_sum(a->value, D(x), b->value, D(y), D(z), n, S(z));
  if (n <= 0) return 0;
  const int ztag = D(z) == D(x) ? 0 : (D(z) == D(y) ? 1 : 2);
  k_lin_coef<<<grid_for(n), kThreads, 0, S(z)>>>(n, a->kind, a->slot, a->value, b->kind, b->slot, b->value, ztag,
                                                  D(x), D(y), D(z), C(z)->fam->scratch.slots);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int N_VFetchSlots_PihmGpu(N_Vector v, int count, double *out, const unsigned int *dev_word,
                          unsigned int *word_out) {
  if (!v || count < 0 || count > PIHM_NV_SLOTS || (count > 0 && !out) || (dev_word && !word_out)) return -1;
  Scratch &s = C(v)->fam->scratch;
  double *h = s.host + 2;  // after the reductions' own result pair
  if (count > 0 &&
      cudaMemcpyAsync(h, s.slots, sizeof(double) * 2 * count, cudaMemcpyDeviceToHost, S(v)) != cudaSuccess)
    return -2;
  unsigned int *hw = (unsigned int *)(h + 2 * PIHM_NV_SLOTS);
  if (dev_word && cudaMemcpyAsync(hw, dev_word, sizeof(unsigned int), cudaMemcpyDeviceToHost, S(v)) != cudaSuccess)
    return -2;
  if (cudaStreamSynchronize(S(v)) != cudaSuccess) return -2;
  for (int i = 0; i < count; i++) out[i] = h[2 * i];
  if (dev_word) *word_out = *hw;
  return 0;
}

void *N_VGetStream_PihmGpu(N_Vector v) { return v ? (void *)S(v) : nullptr; }

// ---------------------------------------------------------------------------
// raw-pointer entry points: a library workspace per stream, created on first
// use and kept until the process exits
// ---------------------------------------------------------------------------
static std::mutex g_ws_mu;
static std::map<cudaStream_t, Family *> g_ws;

static Family *stream_family(void *stream) {
  std::lock_guard<std::mutex> lk(g_ws_mu);
  auto it = g_ws.find((cudaStream_t)stream);
  if (it != g_ws.end()) return it->second;
  Family *f = new_family(stream);
  if (f) g_ws[(cudaStream_t)stream] = f;
  return f;
}

int pihm_gpu_nv_linear_sum(double a, const double *x, double b, const double *y, double *z, int64_t n,
                           void *stream) {
  if (n < 0 || (n > 0 && (!x || !y || !z))) return -1;
  return linear_sum(a, x, b, y, z, n, (cudaStream_t)stream);
}

int pihm_gpu_nv_wrms_norm(const double *x, const double *w, int64_t n, void *stream, double *result) {
  if (n <= 0 || !x || !w || !result) return -1;
  Family *f = stream_family(stream);
  if (!f) return -5;
  double r[2];
  if (red_family<R_WSQ>(f, n, x, w, nullptr, r)) return -2;
  *result = sqrt(r[0] / (double)n);
  return 0;
}

int pihm_gpu_nv_dot_prod(const double *x, const double *y, int64_t n, void *stream, double *result) {
  if (n <= 0 || !x || !y || !result) return -1;
  Family *f = stream_family(stream);
  if (!f) return -5;
  double r[2];
  if (red_family<R_DOT>(f, n, x, y, nullptr, r)) return -2;
  *result = r[0];
  return 0;
}

}  // extern "C"
