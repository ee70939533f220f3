/*
 * pihm_bdf.h -- variable-order BDF integrator (Newton iteration, GMRES with
 * difference-quotient Jacobian-vector products) restating CVODE 2.9.0 as the
 * reference PIHM configures it (src/ode.c:413-529).  It works on any
 * SUNDIALS 2.7 N_Vector through its operations table, in particular the
 * device N_Vector of pihm_nvector.h, and calls the right-hand side through a
 * CVRhsFn such as pihm_gpu_ode.
 *
 * Each entry point replaces the CVODE call of the same meaning
 * (cvode/include/cvode/cvode.h of the reference tree):
 *   pihm_bdf_create           CVodeCreate(CV_BDF, CV_NEWTON)
 *   pihm_bdf_init / _reinit   CVodeInit / CVodeReInit
 *   pihm_bdf_ss_tolerances    CVodeSStolerances
 *   pihm_bdf_set_user_data    CVodeSetUserData
 *   pihm_bdf_set_init_step    CVodeSetInitStep
 *   pihm_bdf_set_max_step     CVodeSetMaxStep
 *   pihm_bdf_set_max_num_steps CVodeSetMaxNumSteps
 *   pihm_bdf_set_stab_lim_det CVodeSetStabLimDet
 *   pihm_bdf_set_stop_time    CVodeSetStopTime
 *   pihm_bdf_solve            CVode(..., CV_NORMAL)
 *   pihm_bdf_get_stats        CVodeGetNumSteps / NumRhsEvals / NumNonlinSolvIters ...
 *   pihm_bdf_free             CVodeFree
 * The linear solver is fixed to CVSpgmr(PREC_NONE, maxl = 5) with modified
 * Gram-Schmidt (cvode/src/cvode/cvode_spgmr.c).
 */
#ifndef PIHM_BDF_H
#define PIHM_BDF_H

#include "pihm_nvector.h"

#ifdef __cplusplus
extern "C" {
#endif

/* return codes (CVODE's values, cvode/include/cvode/cvode.h) */
#define PIHM_BDF_SUCCESS 0
#define PIHM_BDF_TSTOP_RETURN 1
#define PIHM_BDF_TOO_MUCH_WORK (-1)
#define PIHM_BDF_TOO_MUCH_ACC (-2)
#define PIHM_BDF_ERR_FAILURE (-3)
#define PIHM_BDF_CONV_FAILURE (-4)
#define PIHM_BDF_LSOLVE_FAIL (-7)
#define PIHM_BDF_RHSFUNC_FAIL (-8)
#define PIHM_BDF_FIRST_RHSFUNC_ERR (-9)
#define PIHM_BDF_REPTD_RHSFUNC_ERR (-10)
#define PIHM_BDF_UNREC_RHSFUNC_ERR (-11)
#define PIHM_BDF_MEM_FAIL (-20)
#define PIHM_BDF_ILL_INPUT (-22)
#define PIHM_BDF_TOO_CLOSE (-27)

typedef int (*pihm_bdf_rhs_fn)(double t, N_Vector y, N_Vector ydot, void *user_data);
typedef struct pihm_bdf pihm_bdf;

typedef struct pihm_bdf_stats {
    long nst, nfe, nni, ncfn, netf, nli, nfes, njtimes, ncfl, nor;
    int qlast, qcur;
    double hlast, hcur, tcur;
} pihm_bdf_stats;

pihm_bdf *pihm_bdf_create(void);
int pihm_bdf_init(pihm_bdf *mem, pihm_bdf_rhs_fn f, double t0, N_Vector y0);
int pihm_bdf_reinit(pihm_bdf *mem, double t0, N_Vector y0);
int pihm_bdf_ss_tolerances(pihm_bdf *mem, double reltol, double abstol);
int pihm_bdf_set_user_data(pihm_bdf *mem, void *user_data);
int pihm_bdf_set_init_step(pihm_bdf *mem, double hin);
int pihm_bdf_set_max_step(pihm_bdf *mem, double hmax);
int pihm_bdf_set_max_num_steps(pihm_bdf *mem, long mxsteps);
int pihm_bdf_set_stab_lim_det(pihm_bdf *mem, int on);
int pihm_bdf_set_stop_time(pihm_bdf *mem, double tstop);
/* GMRES scalars kept with the vectors (no CVODE counterpart; the solution is
 * the same to the last bit).  Within each GMRES iteration the norm that sets
 * the difference-quotient increment and the modified Gram-Schmidt dot
 * products feed the linear sums that use them where the vectors live
 * (N_VDotProdSlot_PihmGpu, N_VLinearSumCoef_PihmGpu, ...) and are read back
 * once, together with the right-hand side's status when that is this
 * library's pihm_gpu_ode on the vectors' stream (pihm_gpu_ode_launch): one
 * host round trip per iteration instead of one per reduction and per
 * evaluation.  setting -1 (default): on for device vectors of this library
 * integrated with pihm_gpu_ode; 1: on for any vectors (host vectors keep
 * the values on the host; a right-hand side other than pihm_gpu_ode reports
 * at once, and recoverable failures are retried as CVODE retries them);
 * 0: off. */
int pihm_bdf_set_deferred_scalars(pihm_bdf *mem, int setting);
/* How the last solve ran its GMRES iterations: 0 plain, 1 scalars kept on
 * the host side of the operations table, 2 kept on the device (3: and the
 * right-hand side's status read back with them); -1 before the first. */
int pihm_bdf_get_deferred_scalars(const pihm_bdf *mem);
/* Host time inside the integrator's vector operations (no CVODE
 * counterpart), accumulated while on (pihm_bdf_set_op_timing resets it):
 * issuing element-wise operations (and reductions left on the device),
 * reductions until their value is back on the host (and slot read-backs),
 * right-hand-side calls until they return.  Wall time outside these is the
 * integrator's own host work plus the device time the calls waited for. */
enum { PIHM_BDF_OPT_ELEMENTWISE = 0, PIHM_BDF_OPT_REDUCTION, PIHM_BDF_OPT_RHS, PIHM_BDF_OPT_COUNT };
int pihm_bdf_set_op_timing(pihm_bdf *mem, int on);
int pihm_bdf_get_op_times(const pihm_bdf *mem, double *ms, int64_t *calls);
/* Advance to tout (CV_NORMAL): yout receives y(tout) (or y(tstop)). */
int pihm_bdf_solve(pihm_bdf *mem, double tout, N_Vector yout, double *tret);
int pihm_bdf_get_stats(const pihm_bdf *mem, pihm_bdf_stats *stats);
void pihm_bdf_free(pihm_bdf *mem);

#ifdef __cplusplus
}
#endif
#endif /* PIHM_BDF_H */
