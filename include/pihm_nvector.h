/*
 * pihm_nvector.h -- device-resident N_Vector for CVODE 2.9 (SUNDIALS 2.7).
 *
 * The data of these vectors live in GPU memory and every operation of the
 * SUNDIALS 2.7 operations table (cvode/include/sundials/sundials_nvector.h:
 * 90-117 in the reference tree) runs as a kernel on the vector family's CUDA
 * stream.  Element-wise operations reproduce the serial N_Vector's arithmetic
 * exactly, special cases included (cvode/src/nvec_ser/nvector_serial.c:
 * 421-1060), so they agree bit for bit with it; reductions (dot product and
 * norms) use a fixed two-level tree, so they are deterministic run to run and
 * differ from the serial left-to-right sum only by rounding.
 *
 * Reductions return their value to the host, which synchronises the stream.
 *
 * Include order: when the SUNDIALS headers are used too, include them first;
 * otherwise this header declares the layout-compatible N_Vector types itself.
 */
#ifndef PIHM_NVECTOR_H
#define PIHM_NVECTOR_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef _NVECTOR_H
/* Same layout as SUNDIALS 2.7.0 (cvode/include/sundials/sundials_nvector.h:
 * 64-130 of the reference): the ops table order is the ABI CVODE calls. */
typedef enum {
    SUNDIALS_NVEC_SERIAL,
    SUNDIALS_NVEC_PARALLEL,
    SUNDIALS_NVEC_OPENMP,
    SUNDIALS_NVEC_PTHREADS,
    SUNDIALS_NVEC_PARHYP,
    SUNDIALS_NVEC_PETSC,
    SUNDIALS_NVEC_CUSTOM
} N_Vector_ID;
typedef struct _generic_N_Vector_Ops *N_Vector_Ops;
typedef struct _generic_N_Vector *N_Vector;
struct _generic_N_Vector_Ops {
    N_Vector_ID (*nvgetvectorid)(N_Vector);
    N_Vector (*nvclone)(N_Vector);
    N_Vector (*nvcloneempty)(N_Vector);
    void (*nvdestroy)(N_Vector);
    void (*nvspace)(N_Vector, long int *, long int *);
    double *(*nvgetarraypointer)(N_Vector);
    void (*nvsetarraypointer)(double *, N_Vector);
    void (*nvlinearsum)(double, N_Vector, double, N_Vector, N_Vector);
    void (*nvconst)(double, N_Vector);
    void (*nvprod)(N_Vector, N_Vector, N_Vector);
    void (*nvdiv)(N_Vector, N_Vector, N_Vector);
    void (*nvscale)(double, N_Vector, N_Vector);
    void (*nvabs)(N_Vector, N_Vector);
    void (*nvinv)(N_Vector, N_Vector);
    void (*nvaddconst)(N_Vector, double, N_Vector);
    double (*nvdotprod)(N_Vector, N_Vector);
    double (*nvmaxnorm)(N_Vector);
    double (*nvwrmsnorm)(N_Vector, N_Vector);
    double (*nvwrmsnormmask)(N_Vector, N_Vector, N_Vector);
    double (*nvmin)(N_Vector);
    double (*nvwl2norm)(N_Vector, N_Vector);
    double (*nvl1norm)(N_Vector);
    void (*nvcompare)(double, N_Vector, N_Vector);
    int (*nvinvtest)(N_Vector, N_Vector);
    int (*nvconstrmask)(N_Vector, N_Vector, N_Vector);
    double (*nvminquotient)(N_Vector, N_Vector);
};
struct _generic_N_Vector {
    void *content;
    struct _generic_N_Vector_Ops *ops;
};
#endif

/* ---------------------------------------------------------------------
 * Drop-in CVODE callback and post-step update.
 * --------------------------------------------------------------------- */
struct pihm_gpu_ctx;

/* CVRhsFn replacing the reference's ODE() (src/ode.c:4, registered with
 * CVodeInit at src/ode.c:436): user_data is the pihm_gpu_ctx.  y and ydot are
 * either device N_Vectors of this library (internal element order, evaluated
 * in place on the context's stream) or SUNDIALS serial/OpenMP vectors (host
 * memory, reference order; copied in and out).  Returns 0, or -1 when a
 * derivative is NaN (the reference exits there, src/ode.c:401-410) or the
 * vectors do not fit the context. */
int pihm_gpu_ode(double t, N_Vector y, N_Vector ydot, void *user_data);
/* Summary's effect on later right-hand sides (src/update.c:3-99): ws0 <- y
 * (the previous-step surface storage that caps infiltration,
 * src/vert_flow.c:122).  y as for pihm_gpu_ode. */
int pihm_gpu_summary(struct pihm_gpu_ctx *ctx, N_Vector y);

/* Create a vector family's first member: `length` doubles of device memory,
 * operations on `stream` (cudaStream_t, NULL = legacy default stream).
 * Clones share the family's stream and reduction scratch. */
N_Vector N_VNew_PihmGpu(long int length, void *stream);
/* Wrap caller-owned device memory (not freed by N_VDestroy). */
N_Vector N_VMake_PihmGpu(long int length, double *dev_data, void *stream);
double *N_VGetDeviceArrayPointer_PihmGpu(N_Vector v);
long int N_VGetLength_PihmGpu(N_Vector v);
/* Host <-> device copies of the whole vector (synchronous). */
int N_VCopyFromHost_PihmGpu(N_Vector v, const double *host);
int N_VCopyToHost_PihmGpu(N_Vector v, double *host);

/* The operations table, callable directly as well. */
N_Vector_ID N_VGetVectorID_PihmGpu(N_Vector v);
N_Vector N_VClone_PihmGpu(N_Vector w);
N_Vector N_VCloneEmpty_PihmGpu(N_Vector w);
void N_VDestroy_PihmGpu(N_Vector v);
void N_VSpace_PihmGpu(N_Vector v, long int *lrw, long int *liw);
double *N_VGetArrayPointer_PihmGpu(N_Vector v);
void N_VSetArrayPointer_PihmGpu(double *v_data, N_Vector v);
void N_VLinearSum_PihmGpu(double a, N_Vector x, double b, N_Vector y, N_Vector z);
void N_VConst_PihmGpu(double c, N_Vector z);
void N_VProd_PihmGpu(N_Vector x, N_Vector y, N_Vector z);
void N_VDiv_PihmGpu(N_Vector x, N_Vector y, N_Vector z);
void N_VScale_PihmGpu(double c, N_Vector x, N_Vector z);
void N_VAbs_PihmGpu(N_Vector x, N_Vector z);
void N_VInv_PihmGpu(N_Vector x, N_Vector z);
void N_VAddConst_PihmGpu(N_Vector x, double b, N_Vector z);
double N_VDotProd_PihmGpu(N_Vector x, N_Vector y);
double N_VMaxNorm_PihmGpu(N_Vector x);
double N_VWrmsNorm_PihmGpu(N_Vector x, N_Vector w);
double N_VWrmsNormMask_PihmGpu(N_Vector x, N_Vector w, N_Vector id);
double N_VMin_PihmGpu(N_Vector x);
double N_VWL2Norm_PihmGpu(N_Vector x, N_Vector w);
double N_VL1Norm_PihmGpu(N_Vector x);
void N_VCompare_PihmGpu(double c, N_Vector x, N_Vector z);
int N_VInvTest_PihmGpu(N_Vector x, N_Vector z);
int N_VConstrMask_PihmGpu(N_Vector c, N_Vector x, N_Vector m);
double N_VMinQuotient_PihmGpu(N_Vector num, N_Vector denom);

/* Raw-pointer entry points (device pointers, length n, the given stream):
 * the same kernels for callers that keep their own vector objects. */
int pihm_gpu_nv_linear_sum(double a, const double *x, double b, const double *y, double *z,
                           int64_t n, void *stream);
int pihm_gpu_nv_wrms_norm(const double *x, const double *w, int64_t n, void *stream,
                          double *result);
int pihm_gpu_nv_dot_prod(const double *x, const double *y, int64_t n, void *stream,
                         double *result);

/* ---------------------------------------------------------------------
 * Device-resident scalars (no counterpart in SUNDIALS 2.7, whose reductions
 * all return to the host).  Inside one GMRES iteration (SpgmrSolve,
 * cvode/src/sundials/sundials_spgmr.c:165-405) the norm that sets the
 * difference-quotient increment (CVSpilsDQJtimes, cvode_spils.c:665-705)
 * and the Gram-Schmidt dot products (ModifiedGS, sundials_iterative.c) are
 * only coefficients of the next linear sums until the Hessenberg column is
 * complete.  These entry points keep such values in the vector family's
 * slot array on the device, use them there, and read them back in one copy.
 * --------------------------------------------------------------------- */
#define PIHM_NV_SLOTS 16
/* A linear-sum coefficient: a host constant, or derived from slot s. */
typedef struct pihm_nv_coef {
  int32_t kind; /* PIHM_NV_COEF_* */
  int32_t slot;
  double value; /* for PIHM_NV_COEF_HOST */
} pihm_nv_coef;
enum {
  PIHM_NV_COEF_HOST = 0,   /* value */
  PIHM_NV_COEF_NEG,        /* -s */
  PIHM_NV_COEF_INV,        /* 1/s */
  PIHM_NV_COEF_INV_INV,    /* 1/(1/s), rounded twice */
  PIHM_NV_COEF_NEG_INV_INV /* -(1/(1/s)) */
};
/* slot <- N_VDotProd(x, y), left on the device; asynchronous. */
int N_VDotProdSlot_PihmGpu(N_Vector x, N_Vector y, int slot);
/* slot <- N_VWrmsNorm(x, w), left on the device; asynchronous. */
int N_VWrmsNormSlot_PihmGpu(N_Vector x, N_Vector w, int slot);
/* N_VLinearSum(a, x, b, y, z) with a and b formed on the device from the
 * slots; the serial N_Vector's case analysis (a == 1, b == -1, a == b, ...)
 * is made there from the values, so every element equals N_VLinearSum's
 * with the same coefficients.  Asynchronous. */
int N_VLinearSumCoef_PihmGpu(const pihm_nv_coef *a, N_Vector x, const pihm_nv_coef *b, N_Vector y,
                             N_Vector z);
/* Copy slots 0..count-1 of v's family to out[] -- and, when dev_word is not
 * null, one 32-bit device word to *word_out -- with one synchronisation of
 * v's stream.  Returns 0, -1 (bad argument) or -2 (CUDA error). */
int N_VFetchSlots_PihmGpu(N_Vector v, int count, double *out, const unsigned int *dev_word,
                          unsigned int *word_out);
/* The stream a device vector's operations run on. */
void *N_VGetStream_PihmGpu(N_Vector v);

/* pihm_gpu_ode for device vectors without reading back the status: the
 * evaluation is queued on the context's stream and a NaN derivative shows
 * in the context's error word (pihm_gpu_error_word), which pihm_gpu_status
 * reads and clears.  Returns 0, or -1 if the evaluation could not be
 * queued. */
int pihm_gpu_ode_launch(double t, N_Vector y, N_Vector ydot, void *user_data);
/* Device address of the context's error word (nonzero after a NaN). */
const unsigned int *pihm_gpu_error_word(struct pihm_gpu_ctx *ctx);

/* WRMS norm, sqrt(sum_i (x_i w_i)^2 / n), for callers that cannot allocate
 * device memory (no counterpart in the reference).  pihm_gpu_nv_wrms_norm
 * creates a workspace with cudaMalloc the first time a stream uses it; code
 * running during CUDA-graph capture, inside a framework that owns every
 * device allocation, or in a per-call integrator callback cannot do that.
 * This entry point allocates nothing: it works in a fixed library-static
 * device array (about 64 KiB, held by every GPU that loads the library until
 * the process exits) and writes the norm to `result_dev`, caller-owned device
 * memory, on `stream` without synchronising.
 *   - n must be 1 .. PIHM_GPU_NOALLOC_MAX_LEN; longer vectors return
 *     PIHM_GPU_NOALLOC_ERR_TOO_LONG and launch nothing.
 *   - All calls share the array: calls that overlap on the GPU (different
 *     streams without ordering) race and give wrong results.
 *   - The first call on a device looks up the array's device address with
 *     that device current; make it before any stream capture begins.
 * Returns 0, -1 (bad argument), -2 (CUDA error) or
 * PIHM_GPU_NOALLOC_ERR_TOO_LONG. */
#define PIHM_GPU_NOALLOC_MAX_LEN 33554432L
#define PIHM_GPU_NOALLOC_ERR_TOO_LONG (-7)
int pihm_gpu_nv_wrms_norm_noalloc(const double *x, const double *w, int64_t n, void *stream,
                                  double *result_dev);

#ifdef __cplusplus
}
#endif
#endif /* PIHM_NVECTOR_H */
