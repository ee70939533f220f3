/*
 * pihm_oracle.h -- CPU restatement of the PIHM right-hand side (test
 * infrastructure only).
 *
 * This is the checker for the GPU library, not part of the product: only the
 * test-suite, the smoke check and the CPU-baseline leg of the benchmark load
 * it.  It restates, loop for loop and in the same floating-point operation
 * order, the reference's serial/OpenMP ODE() (lj-cug/PIHM-CUDA src/ode.c:4-399)
 * and its callees in src/hydrol.c, src/lat_flow.c, src/vert_flow.c,
 * src/river_flow.c and src/soil.c, reading the watershed from the same
 * structure-of-arrays description the GPU library takes (include/pihm_gpu.h).
 * Built with -fopenmp it parallelises the same loops the reference does.
 */
#ifndef PIHM_ORACLE_H
#define PIHM_ORACLE_H

#include "pihm_gpu.h"
#include "pihm_land.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_model oracle_model;

oracle_model *oracle_create(const pihm_gpu_mesh *mesh, int surf_mode,
                            int riv_mode, double stepsize);
void oracle_destroy(oracle_model *m);
void oracle_set_forcing(oracle_model *m, const double *pcpdrp,
                        const double *edir, const double *ett);
void oracle_set_bc(oracle_model *m, const double *elem_bc,
                   const double *river_bc);
void oracle_set_ws0_surf(oracle_model *m, const double *ws0_surf);
/* Switch to the Flux-PIHM (_NOAH_) right-hand side with Noah's per-step
 * inputs: transpiration per soil layer et[nelem][nlayers], water-table and
 * root layers, top-layer unfrozen moisture with the soil's smcmin/smcmax, and
 * the frozen-soil infiltration factor. */
int oracle_set_noah(oracle_model *m, const double *et, int nlayers, const int *nwtbl, const int *nroot,
                    const double *sh2o0, const double *smcmin, const double *smcmax, const double *fcr);
void oracle_set_river_edge_ovlflow(oracle_model *m, const double *ovlflow);
/* ydot = f(t, y); returns 0, or -3 when a derivative is NaN (the reference
 * exits there, src/ode.c:401-410). */
int oracle_rhs(oracle_model *m, double t, const double *y, double *ydot);
void oracle_get_fluxes(const oracle_model *m, double *ovlflow, double *subsurf,
                       double *infil, double *rechg, double *et_split,
                       double *rivflow);
/* Post-step update (Summary, src/update.c:3-99): ws0 <- y. */
void oracle_post_step(oracle_model *m, const double *y);
/* CVRhsFn over SUNDIALS serial N_Vectors, user_data = oracle_model. */
int oracle_cvrhs(double t, void *y, void *ydot, void *user_data);
/* Land-surface step (land_oracle.c): ApplyForc + IntcpSnowEt of the
 * non-Noah model, elements in reference order.  zmax, depth, porosity, rzd
 * are the mesh's planes. */
typedef struct oracle_land oracle_land;
oracle_land *oracle_land_create(const pihm_land_params *p, const pihm_forcing_series *s, const double *zmax,
                                const double *depth, const double *porosity, const double *rzd);
void oracle_land_destroy(oracle_land *l);
void oracle_land_set_state(oracle_land *l, const double *cmc, const double *sneqv);
/* one step at time t (seconds since 1970 UTC) over stepsize seconds with the
 * soil state unsat, gw [nelem]; 0, or -1 when t lies outside a series */
int oracle_land_step(oracle_land *l, long long t, double stepsize, const double *unsat, const double *gw);
void oracle_land_get(const oracle_land *l, int field, double *out);
void oracle_land_monthly(long long t, int lc, double *out3);

/* Number of OpenMP threads the oracle runs with (1 without OpenMP). */
int oracle_num_threads(void);
void oracle_set_num_threads(int n);
/* s = +1 / -1: every pow() and log() result of this model's evaluations moves
 * by one unit in the last place in that direction (the last-bit sensitivity
 * the tests measure); 0, the default: the reference's arithmetic exactly. */
void oracle_set_ulp_perturb(oracle_model *m, int s);

#ifdef __cplusplus
}
#endif
#endif
