/*
 * pihm_gpu.h -- C ABI of the GB300 (sm_103a) PIHM right-hand-side library.
 *
 * The library evaluates the CVODE right-hand side of the PIHM hydrologic
 * model -- surface, unsaturated and groundwater storage of every triangular
 * element plus stage and bed groundwater of every river segment -- with
 * hand-written FP64 CUDA kernels, and supplies a device-resident N_Vector
 * whose operations run on the same GPU.
 *
 * Everything here is plain C: pointers, sizes and status codes.  No CUDA or
 * torch type appears in a signature; CUDA streams travel as `void *`
 * (a cudaStream_t, NULL = the legacy default stream).
 *
 * Conventions shared with the reference model (lj-cug/PIHM-CUDA):
 *   - state vector y, length NEQ = 3*nelem + 2*nriver, blocks
 *     [surf | unsat | gw | stage | rivgw]      (src/include/pihm_func.h:7-11)
 *   - element neighbour ids are 1-based, a negative id -k is river segment k,
 *     0 is the domain boundary                 (src/include/elem_struct.h:1561,
 *                                               src/init_river.c:23-33)
 *   - river `down` is a 1-based segment id, or an outlet boundary type
 *     -1..-4 (DIRICHLET, NEUMANN, ZERO_DPTH_GRAD, CRIT_DPTH)
 *                                              (src/include/pihm_const.h:140-143)
 *   - all arithmetic is IEEE double.
 *
 * Ordering.  Host arrays passed to or returned from this library are in the
 * reference's element / segment order.  Inside the library elements are
 * renumbered for locality (reverse Cuthill-McKee over the element adjacency)
 * and device state vectors (the `*_dev` arguments and the device N_Vector) are
 * stored in that internal order; pihm_gpu_to_internal / pihm_gpu_to_reference
 * convert between the two.
 *
 * Status codes: 0 = success, > 0 = recoverable (CVODE retries the step),
 * < 0 = unrecoverable (see PIHM_GPU_ERR_*).  The CVODE-facing callback follows
 * CVODE's CVRhsFn contract (cvode/include/cvode/cvode.h, CVRhsFn).
 */
#ifndef PIHM_GPU_H
#define PIHM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PIHM_GPU_NUM_EDGE   3
#define PIHM_GPU_NUM_RIVFLX 11

/* Overland / river flow formulation (src/include/pihm_const.h:152-153). */
#define PIHM_GPU_KINEMATIC 1
#define PIHM_GPU_DIFF_WAVE 2

/* Element ordering inside the library. */
#define PIHM_GPU_ORDER_REFERENCE 0 /* keep the caller's order */
#define PIHM_GPU_ORDER_RCM       1 /* reverse Cuthill-McKee (default) */

enum {
    PIHM_GPU_OK = 0,
    PIHM_GPU_ERR_ARG = -1,     /* bad argument or size */
    PIHM_GPU_ERR_CUDA = -2,    /* a CUDA runtime call failed */
    PIHM_GPU_ERR_NAN = -3,     /* a derivative came out NaN (reference CheckDy,
                                  src/ode.c:401-410, exits instead) */
    PIHM_GPU_ERR_MESH = -4,    /* inconsistent mesh / river topology */
    PIHM_GPU_ERR_NOMEM = -5,   /* device allocation failed */
    PIHM_GPU_ERR_BCTYPE = -6   /* unknown river outlet or shape type
                                  (reference PIHMexit, src/river_flow.c:384-389) */
};

/*
 * Static description of one watershed, structure of arrays, reference order.
 * Field meanings follow the reference element and river records
 * (src/include/elem_struct.h:28-99, src/include/river_struct.h:5-120); only the
 * fields read by the right-hand side are present.  Per-edge arrays are
 * row-major [nelem][3].  All pointers are host pointers and are copied by
 * pihm_gpu_create; the caller keeps ownership.
 */
typedef struct pihm_gpu_mesh {
    int32_t nelem;
    int32_t nriver;
    /* element topology */
    const int32_t *nabr;      /* [nelem*3] neighbour ids (see conventions) */
    const int32_t *bc_type;   /* [nelem*3] 0 no-flow, >0 Dirichlet, <0 Neumann */
    /* element topography (topo_struct) */
    const double *area;       /* [nelem] m2 */
    const double *zmin;       /* [nelem] soil bottom elevation, m */
    const double *zmax;       /* [nelem] surface elevation, m */
    const double *edge;       /* [nelem*3] edge length, m */
    const double *nabrdist;   /* [nelem*3] distance to neighbour, m */
    const double *nabr_x;     /* [nelem*3] neighbour centroid x, m */
    const double *nabr_y;     /* [nelem*3] neighbour centroid y, m */
    /* element soil (soil_struct) */
    const double *depth, *ksath, *ksatv, *kinfv, *dinf, *alpha, *beta,
                 *porosity, *dmac, *kmach, *kmacv, *areafv, *areafh;
    /* land cover / plant (lc.rough, ps.rzd) */
    const double *rough;      /* [nelem] Manning n, s m-1/3 */
    const double *rzd;        /* [nelem] root zone depth, m */
    /* river topology */
    const int32_t *down;       /* [nriver] */
    const int32_t *leftele;    /* [nriver] 1-based */
    const int32_t *rightele;   /* [nriver] 1-based */
    const int32_t *intrpl_ord; /* [nriver] 1 rectangle .. 4 cubic */
    const int32_t *riverbc_type; /* [nriver] upstream boundary type */
    /* river topography, shape and material */
    const double *riv_area, *riv_zmin, *riv_zmax, *riv_zbed, *riv_node_zmax,
                 *riv_dist_left, *riv_dist_right;
    const double *riv_depth, *riv_coeff, *riv_length, *riv_width;
    const double *riv_rough, *riv_cwr, *riv_ksath, *riv_ksatv, *riv_bedthick,
                 *riv_porosity;
} pihm_gpu_mesh;

typedef struct pihm_gpu_ctx pihm_gpu_ctx;

/* ---------------------------------------------------------------------
 * Lifetime.  Replaces the reference's per-field cudaMallocManaged mirror
 * (src/initialize_cuda.c:5, AoS_to_SoA :430) with one packed device image.
 * --------------------------------------------------------------------- */

/* Validate the mesh, renumber it (`order`), upload it and allocate all
 * persistent device buffers.  `surf_mode` / `riv_mode` are KINEMATIC or
 * DIFF_WAVE (ctrl.surf_mode / ctrl.riv_mode, src/hydrol.c:24-28);
 * `stepsize` is the model step in seconds that caps infiltration
 * (src/hydrol.c:26, src/vert_flow.c:124).  Forcing, boundary values and the
 * carried fluxes start at zero. */
int pihm_gpu_create(const pihm_gpu_mesh *mesh, int surf_mode, int riv_mode,
                    double stepsize, int order, pihm_gpu_ctx **out);
void pihm_gpu_destroy(pihm_gpu_ctx *ctx);

/* Stream all later work of this context is issued on (cudaStream_t). */
int pihm_gpu_set_stream(pihm_gpu_ctx *ctx, void *stream);
/* The stream the context issues its work on (NULL = legacy default). */
void *pihm_gpu_get_stream(const pihm_gpu_ctx *ctx);
/* Block shape of the element kernel: 0: 512 threads x 2 blocks per SM,
 * 1 (default): 256 x 4, 2: 128 x 8; identical results (the batch engine's
 * pihm_batch_set_rhs_shape). */
int pihm_gpu_set_kernel_shape(pihm_gpu_ctx *ctx, int shape);
int pihm_gpu_sizes(const pihm_gpu_ctx *ctx, int32_t *nelem, int32_t *nriver,
                   int64_t *neq);
/* Internal position of every element and segment: perm[internal] = reference
 * index (0-based).  Either pointer may be NULL. */
int pihm_gpu_get_permutation(const pihm_gpu_ctx *ctx, int32_t *elem_perm,
                             int32_t *river_perm);

/* ---------------------------------------------------------------------
 * Inputs the right-hand side reads besides y (reference order, host arrays).
 * They stand for ApplyBc / ApplyForc / IntcpSnowEt (src/pihm.c:21-66) and the
 * post-step update (src/update.c:3-99).  NULL leaves a field unchanged.
 * --------------------------------------------------------------------- */
int pihm_gpu_set_forcing(pihm_gpu_ctx *ctx, const double *pcpdrp,
                         const double *edir, const double *ett);
/* Element boundary values, [nelem*3] (bc.head or bc.flux, one union per edge,
 * src/include/elem_struct.h:720-728) and river boundary values [nriver]. */
int pihm_gpu_set_bc(pihm_gpu_ctx *ctx, const double *elem_bc,
                    const double *river_bc);
/* ws0.surf of the previous model step (read by Infil, src/vert_flow.c:122). */
int pihm_gpu_set_ws0_surf(pihm_gpu_ctx *ctx, const double *ws0_surf);
/* Seed of the river-edge overland fluxes that Infil reads before RiverToElem
 * overwrites them (src/vert_flow.c:61 vs src/river_flow.c:159-182):
 * [nelem*3] wf.ovlflow, only entries on river edges are used. */
int pihm_gpu_set_river_edge_ovlflow(pihm_gpu_ctx *ctx, const double *ovlflow);

/* ---------------------------------------------------------------------
 * Right-hand side.
 * --------------------------------------------------------------------- */

/* ydot = f(t, y) on the context's stream, device pointers in internal order.
 * Asynchronous: it neither synchronises nor allocates.  A NaN derivative sets
 * a device error word that pihm_gpu_status reads. */
int pihm_gpu_rhs(pihm_gpu_ctx *ctx, double t, const double *y_dev,
                 double *ydot_dev);
/* Synchronise the context's stream and return (then clear) the error word:
 * 0 or PIHM_GPU_ERR_NAN / PIHM_GPU_ERR_CUDA. */
int pihm_gpu_status(pihm_gpu_ctx *ctx);

/* Same evaluation from host arrays in reference order: y in, run, ydot out,
 * synchronise.  This is the call a CPU-side integrator makes in place of the
 * serial ODE() (src/ode.c:4-399).  When the device can address both arrays
 * (pinned or registered host memory, or any host memory on a device with
 * pageable-memory access, as Grace-based GB300 systems over NVLink-C2C), the
 * reordering kernels read y from and write ydot to host memory directly;
 * otherwise the arrays are copied through device staging.  Both paths give
 * the same bits. */
int pihm_gpu_rhs_host(pihm_gpu_ctx *ctx, double t, const double *y_host,
                      double *ydot_host);
/* pihm_gpu_rhs_host's path: mode 0 (default) reads and writes host arrays
 * directly where the device can address them, 1 always copies. */
int pihm_gpu_set_host_path(pihm_gpu_ctx *ctx, int mode);
/* pihm_gpu_rhs_host without waiting (no counterpart in the reference, whose
 * evaluations are sequential): the evaluation is queued on the context's
 * stream and pihm_gpu_wait returns its status; y_host must stay unchanged and
 * both buffers valid until then, and the buffers should be pinned for the
 * copies to be asynchronous.  Several evaluations may be queued on one
 * context before a wait; they run in the order queued, each seeing the
 * carried state the previous one left.  Two contexts on one mesh, each on its own
 * stream, then evaluate independent states with one's host-link transfers
 * beside the other's kernels. */
int pihm_gpu_rhs_host_async(pihm_gpu_ctx *ctx, double t, const double *y_host, double *ydot_host);
/* Wait for the context's queued work: PIHM_GPU_OK, or PIHM_GPU_ERR_NAN if any
 * of its evaluations since the last status read produced a NaN. */
int pihm_gpu_wait(pihm_gpu_ctx *ctx);
/* Whether the last pihm_gpu_rhs_host call accessed host memory directly, and
 * whether the device can access pageable host memory (either may be NULL). */
int pihm_gpu_host_path_info(const pihm_gpu_ctx *ctx, int *last_direct, int *pageable_access);

/* pihm_gpu_ode on device vectors synchronises after each evaluation to read
 * the NaN error word (the reference checks every call).  deferred = 1 skips
 * that; the word is then read by the next pihm_gpu_status. */
int pihm_gpu_set_nan_check(pihm_gpu_ctx *ctx, int deferred);
/* Post-step update on device state (internal order): ws0.surf <- y_dev[0:nelem]
 * (Summary, src/update.c:3-99; asynchronous on the context's stream). */
int pihm_gpu_post_step(pihm_gpu_ctx *ctx, const double *y_dev);
/* Switch to the Flux-PIHM right-hand side (the reference built with _NOAH_)
 * and set Noah's per-step inputs, all in reference element order:
 * transpiration per soil layer et[nelem][nlayers] (wf.et, m/s), the
 * water-table layer nwtbl and the root layers nroot (ps.nwtbl, ps.nroot;
 * nroot <= nlayers <= 11), the top layer's unfrozen moisture sh2o0
 * (ws.sh2o[0]) with the soil's smcmin / smcmax, and the frozen-soil factor
 * fcr (ps.fcr).  EtExtract then splits ET as src/hydrol.c:43-55,79-83 (with
 * GwTransp, noah/lsm_func.c:163-185) and Infil takes its saturation from
 * sh2o0 and is scaled by fcr (src/vert_flow.c:16-19,94-98).  Call again
 * after every Noah step. */
int pihm_gpu_set_noah(pihm_gpu_ctx *ctx, const double *et, int nlayers, const int32_t *nwtbl,
                      const int32_t *nroot, const double *sh2o0, const double *smcmin,
                      const double *smcmax, const double *fcr);
/* The watershed water balance of a model step of dt seconds, from the state
 * y_dev (device, internal order) and the current forcing and river fluxes:
 * out[0] sources (prcp area dt), out[1] sinks ((edir + ett + ec) area dt
 * plus the outlet segments' discharge dt), out[2] storage (canopy, snow,
 * surface, pore water and river water volume), the three sums of
 * PrintWaterBal (src/print.c:337-542).  Without the land-surface model
 * (include/pihm_land.h) prcp is pcpdrp and there is no canopy or snow.  The reference's cumulative error is the
 * running sum of out[0] - out[1] - (out[2] - previous out[2]).  Synchronous. */
int pihm_gpu_water_balance(pihm_gpu_ctx *ctx, const double *y_dev, double dt, double *out);

/* Restart files in the reference's binary .ic format (host only, no GPU):
 * per element cmc, sneqv, surf, unsat, gw, then per segment stage, gw, as
 * ReadIc reads them (src/read_ic.c:3-39) and PrintInit writes them
 * (src/print.c:213-330).  y is the state vector in reference order
 * [surf | unsat | gw | stage | rivgw]; cmc and sneqv (canopy and snow
 * storage, not part of y) may be NULL (written as 0 / not returned).
 * pihm_ic_read returns PIHM_GPU_ERR_MESH when the file size does not match
 * nelem and nriver, as the reference refuses such a file. */
int pihm_ic_write(const char *path, int32_t nelem, int32_t nriver, const double *y,
                  const double *cmc, const double *sneqv);
int pihm_ic_read(const char *path, int32_t nelem, int32_t nriver, double *y, double *cmc,
                 double *sneqv);

/* Keep per-element and per-segment fluxes of every later call so that
 * pihm_gpu_get_fluxes can read them (costs extra stores). */
int pihm_gpu_set_diagnostics(pihm_gpu_ctx *ctx, int on);
/* Fluxes of the last right-hand side evaluated with diagnostics on, reference
 * order, host arrays, any may be NULL:
 *   ovlflow, subsurf [nelem*3] (wf.ovlflow / wf.subsurf, m3 s-1)
 *   infil, rechg     [nelem]   (wf.infil / wf.rechg, m s-1)
 *   et_split         [nelem*5] (edir_surf, edir_unsat, edir_gw, ett_unsat, ett_gw)
 *   rivflow          [nriver*11] (river wf.rivflow, m3 s-1) */
int pihm_gpu_get_fluxes(pihm_gpu_ctx *ctx, double *ovlflow, double *subsurf,
                        double *infil, double *rechg, double *et_split,
                        double *rivflow);

/* Reorder a device state vector (length NEQ) between the reference order and
 * the internal order.  src and dst must not overlap. */
int pihm_gpu_to_internal(pihm_gpu_ctx *ctx, const double *src_ref_dev,
                         double *dst_int_dev);
int pihm_gpu_to_reference(pihm_gpu_ctx *ctx, const double *src_int_dev,
                          double *dst_ref_dev);

/* ---------------------------------------------------------------------
 * Instrumentation (no counterpart in the reference, which has no GPU timers).
 * --------------------------------------------------------------------- */

/* Number of kernels this context has launched so far. */
int pihm_gpu_launch_count(const pihm_gpu_ctx *ctx, int64_t *count);
/* Bracket every later kernel launch with CUDA events on the context's
 * stream. */
int pihm_gpu_set_profiling(pihm_gpu_ctx *ctx, int on);
/* Synchronise, then return and reset the accumulated device time (ms) and
 * launch count per kernel: 0 prep, 1 gradient, 2 element, 3 river,
 * 4 finish, 5 edge, 6 permute; n entries are written. */
int pihm_gpu_kernel_times(pihm_gpu_ctx *ctx, double *ms, int64_t *calls, int n);

/* Diagnostic: the power of the right-hand-side kernels (the integer-pipe
 * power, the table-driven FP64 pow outside its ranges),
 * fast[i] = pow(x[i], y[i]), and CUDA's pow into cuda_pow[i] when it is not
 * NULL; device arrays of length n, asynchronous on `stream`.  Used by the
 * tests to measure the error of the fast path. */
int pihm_gpu_selftest_pow(const double *x, const double *y, double *fast,
                          double *cuda_pow, int64_t n, void *stream);
/* Diagnostic: the Manning-exponent power of the right-hand-side kernels,
 * out[i] = x[i]^0.6666667 (river == 0, overland flow) or x[i]^(2.0/3.0)
 * (river != 0, channel flow); device arrays of length n, asynchronous on
 * `stream`. */
int pihm_gpu_selftest_pow_manning(const double *x, int river, double *out, int64_t n,
                                  void *stream);
/* Diagnostic: the integer-pipe power alone, out[i] = x[i]^y[i] and ok[i] = 1
 * where x[i] and y[i] are inside its ranges, ok[i] = 0 elsewhere; device
 * arrays of length n, asynchronous on `stream`.  The tests compare its bits
 * with the host build of the same integer arithmetic. */
int pihm_gpu_selftest_pow_int(const double *x, const double *y, double *out, int32_t *ok,
                              int64_t n, void *stream);
/* Diagnostic: the integer-pipe division and square root alone,
 * q[i] = a[i] / b[i] and r[i] = sqrt(a[i]); bit 0 of ok[i] is set where the
 * division took the integer path, bit 1 where the square root did; device
 * arrays of length n, asynchronous on `stream`.  Where they are taken, both
 * are the IEEE results bit for bit. */
int pihm_gpu_selftest_div_sqrt_int(const double *a, const double *b, double *q, double *r,
                                   int32_t *ok, int64_t n, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PIHM_GPU_H */
