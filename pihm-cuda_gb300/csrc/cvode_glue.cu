// CVODE-facing glue: the drop-in right-hand-side callback and the post-step
// update, for both the device N_Vector of this library and host N_Vectors
// (SUNDIALS serial or OpenMP, whose content starts with length, own_data,
// data -- cvode/include/nvector/nvector_serial.h:69-73 and
// nvector_openmp.h of the reference tree).
#include <cstring>

#include "pihm_internal.h"
#include "pihm_nvector.h"

namespace {

struct HostContentPrefix {  // SUNDIALS 2.7 serial / OpenMP content layout prefix
  long int length;
  int own_data;
  double *data;
};

bool is_device_vector(N_Vector v) { return v && v->ops && v->ops->nvgetvectorid == N_VGetVectorID_PihmGpu; }

bool is_host_vector(N_Vector v) {
  if (!v || !v->ops || !v->ops->nvgetvectorid) return false;
  const N_Vector_ID id = v->ops->nvgetvectorid(v);
  return id == SUNDIALS_NVEC_SERIAL || id == SUNDIALS_NVEC_OPENMP || id == SUNDIALS_NVEC_PTHREADS;
}

double *host_data(N_Vector v) { return ((HostContentPrefix *)v->content)->data; }
long int host_length(N_Vector v) { return ((HostContentPrefix *)v->content)->length; }

}  // namespace

extern "C" {

// CVRhsFn: ydot = f(t, y).  Device N_Vectors are evaluated in place on the
// vectors' stream; host N_Vectors go through the host-buffer path.  A NaN
// derivative returns -1 (CV_RHSFUNC_FAIL path) where the reference exits
// (src/ode.c:401-410).
static int ode_launch_device(pihm_gpu_ctx *c, N_Vector y, N_Vector ydot) {
  if (N_VGetLength_PihmGpu(y) != c->neq || N_VGetLength_PihmGpu(ydot) != c->neq) return -1;
  c->m.diag = c->diag;
  return pihm::launch_rhs(c->m, N_VGetDeviceArrayPointer_PihmGpu(y), N_VGetDeviceArrayPointer_PihmGpu(ydot),
                          c->stream, &c->launches, c->prof, &c->side) == cudaSuccess
             ? 0
             : -1;
}

int pihm_gpu_ode(double t, N_Vector y, N_Vector ydot, void *user_data) {
  pihm_gpu_ctx *c = (pihm_gpu_ctx *)user_data;
  if (!c || !y || !ydot) return -1;
  if (is_device_vector(y) && is_device_vector(ydot)) {
    if (ode_launch_device(c, y, ydot)) return -1;
    if (c->nan_check_deferred) return 0;
    return pihm_gpu_status(c) == PIHM_GPU_OK ? 0 : -1;
  }
  if (is_host_vector(y) && is_host_vector(ydot)) {
    if (host_length(y) != c->neq || host_length(ydot) != c->neq) return -1;
    return pihm_gpu_rhs_host(c, t, host_data(y), host_data(ydot)) == PIHM_GPU_OK ? 0 : -1;
  }
  return -1;
}

int pihm_gpu_ode_launch(double t, N_Vector y, N_Vector ydot, void *user_data) {
  (void)t;
  pihm_gpu_ctx *c = (pihm_gpu_ctx *)user_data;
  if (!c || !is_device_vector(y) || !is_device_vector(ydot)) return -1;
  return ode_launch_device(c, y, ydot);
}

const unsigned int *pihm_gpu_error_word(pihm_gpu_ctx *c) { return c ? c->m.err : nullptr; }

int pihm_gpu_set_nan_check(pihm_gpu_ctx *c, int deferred) {
  if (!c) return PIHM_GPU_ERR_ARG;
  c->nan_check_deferred = deferred ? 1 : 0;
  return PIHM_GPU_OK;
}

// Summary (src/update.c:3-99) as far as the right-hand side depends on it:
// ws0 <- ws <- y, i.e. the next evaluations cap infiltration with this step's
// surface storage (Infil, src/vert_flow.c:122).
int pihm_gpu_post_step(pihm_gpu_ctx *c, const double *y_dev) {
  if (!c || !y_dev) return PIHM_GPU_ERR_ARG;
  return cudaMemcpyAsync((double *)c->m.ws0_surf, y_dev, sizeof(double) * c->ne, cudaMemcpyDeviceToDevice,
                         c->stream) == cudaSuccess
             ? PIHM_GPU_OK
             : PIHM_GPU_ERR_CUDA;
}

int pihm_gpu_summary(pihm_gpu_ctx *c, N_Vector y) {
  if (!c || !y) return PIHM_GPU_ERR_ARG;
  if (is_device_vector(y)) return pihm_gpu_post_step(c, N_VGetDeviceArrayPointer_PihmGpu(y));
  if (is_host_vector(y)) return pihm_gpu_set_ws0_surf(c, host_data(y));
  return PIHM_GPU_ERR_ARG;
}

}  // extern "C"
