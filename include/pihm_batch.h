/*
 * pihm_batch.h -- many PIHM watersheds (or calibration parameter sets) of
 * uneven size integrated together on one GPU.
 *
 * Each watershed runs the reference's model-step loop (src/pihm.c:7-187:
 * forcing, CVODE to the end of the step with the stop time set, the post-step
 * update, AdjCVodeMaxStep, src/ode.c:555-661) with its own integrator state,
 * step sizes, model step and tolerances.  The engine packs the watersheds'
 * meshes and CVODE vectors into one device arena and advances them in rounds:
 * every watershed runs until it needs a device result (a norm, a dot product
 * or a right-hand-side evaluation); one launch then applies all their queued
 * vector operations and reductions, and one right-hand-side evaluation covers
 * every watershed that asked for one.
 *
 * A watershed's results do not depend on what else is in the batch: each is
 * bit-for-bit the trajectory the single-watershed path (pihm_bdf_* over
 * N_VNew_PihmGpu with pihm_gpu_ode) computes for it.
 *
 * Admission is by arena capacity (elements, segments, interior edges, state
 * entries and watershed slots fixed at creation): pihm_batch_add returns
 * PIHM_GPU_ERR_NOMEM when a watershed does not fit now, and succeeds again
 * after finished watersheds have been released.  Watersheds can be added while
 * others are running.
 */
#ifndef PIHM_BATCH_H
#define PIHM_BATCH_H

#include <stdint.h>

#include "pihm_bdf.h"
#include "pihm_gpu.h"
#include "pihm_land.h"
#include "pihm_noah.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pihm_batch pihm_batch;

/* Arena capacity. */
typedef struct pihm_batch_limits {
    int64_t max_elem;      /* elements over all resident watersheds */
    int64_t max_river;     /* river segments */
    int64_t max_edge;      /* interior edges (about 1.5 x elements) */
    int64_t max_record;    /* hydrograph entries (model steps) over all resident watersheds */
    int32_t max_systems;   /* resident watersheds */
} pihm_batch_limits;

/* The reference's solver controls (ctrl_struct, src/read_para.c:23-108). */
typedef struct pihm_step_control {
    double stepsize;   /* model step (s); also caps infiltration (src/vert_flow.c:122) */
    double reltol, abstol, initstep;
    double nncfn, nnimax, nnimin, decr, incr, stmin;  /* AdjCVodeMaxStep, src/ode.c:601-661 */
    long mxstep;       /* internal steps per model step; 0 = 10 x stepsize (src/ode.c:497) */
} pihm_step_control;

/* One simulation request. */
typedef struct pihm_batch_job {
    const pihm_gpu_mesh *mesh;
    const double *elem_bc;    /* [3*nelem] reference order, or NULL (zeros) */
    const double *river_bc;   /* [nriver], or NULL */
    const double *y0;         /* [3*nelem + 2*nriver] initial state, reference order */
    pihm_step_control ctrl;
    int32_t nsteps;           /* model steps */
    /* spatially uniform forcing per model step [nsteps]: pcpdrp, edir, ett (m/s) */
    const double *pcpdrp, *edir, *ett;
    int32_t outlet;           /* segment whose DOWN_CHANL2CHANL flux is recorded per step, -1: none */
    /* An input deck's own forcing, as the reference's main loop applies it
     * (src/pihm.c:15-66); all optional, zero/NULL for the uniform series
     * above.  The pointers must stay valid until the watershed is released.
     *   deck      ApplyBc every model step from the deck's .bc series
     *             (pihm_deck_bc at start + k stepsize); elem_bc/river_bc
     *             are then unused
     *   land, forcing   the land-surface step (include/pihm_land.h) every
     *             lsm_step seconds, ApplyForc + IntcpSnowEt writing this
     *             watershed's pcpdrp, edir and ett; the uniform series are
     *             then unused (may be NULL).  The series must cover the run
     *   cmc0, sneqv0    initial canopy storage and snow (NULL: zeros)
     *   start     model time of step 0 (s since 1970 UTC) */
    const struct pihm_deck *deck;
    const pihm_land_params *land;
    const pihm_forcing_series *forcing;
    const double *cmc0, *sneqv0;
    int64_t start, lsm_step;
    /* Flux-PIHM: Noah on the device (include/pihm_noah.h) instead of the
     * uniform series, as the reference's _NOAH_ build runs it
     * (src/pihm.c:21-123): the watershed's Noah parameters and initial
     * state, and noah_nforcing forcing sets, the k-th for the land-surface
     * step from model time k noah_lsm_step (Noah() runs over noah_lsm_step
     * seconds), and after every model step Summary's _NOAH_ part and
     * NoahHydrol.  Not with .land.  The pointers must stay valid until the
     * watershed is released. */
    const pihm_noah_params *noah;
    const pihm_noah_state *noah_state;
    const pihm_noah_forcing *noah_forcing;
    int32_t noah_nforcing;
    double noah_lsm_step;
} pihm_batch_job;

enum { PIHM_BATCH_RUNNING = 0, PIHM_BATCH_DONE = 1, PIHM_BATCH_FAILED = 2 };

int pihm_batch_create(const pihm_batch_limits *lim, int surf_mode, int riv_mode, int order,
                      pihm_batch **out);
/* Device memory an arena with these limits takes (all of pihm_batch_create's
 * allocations, at the allocator's 512-byte granularity). */
int pihm_batch_arena_bytes(const pihm_batch_limits *lim, int64_t *bytes);
/* The largest arena that fits in `bytes` of device memory -- e.g. a share of
 * cudaMemGetInfo's free memory -- for watersheds with about rivers_per_elem
 * segments, edges_per_elem interior edges and records_per_elem hydrograph
 * entries per element: admission (pihm_batch_add, the serving layer) is then
 * gated by that memory.  PIHM_GPU_ERR_NOMEM if not even one element fits. */
int pihm_batch_limits_for_memory(int64_t bytes, double rivers_per_elem, double edges_per_elem,
                                 double records_per_elem, int32_t max_systems, pihm_batch_limits *out);
void pihm_batch_destroy(pihm_batch *b);
int pihm_batch_set_stream(pihm_batch *b, void *stream);

/* Scheduling: a watershed waiting for a right-hand-side evaluation is held
 * back while others have reductions to run, until the watersheds waiting for
 * one hold at least `gate` (0..1) of the waiting elements.  0 evaluates every
 * request at once; 1 (the default) gathers every waiting watershed into each
 * evaluation.  Results do not depend on it; throughput does. */
int pihm_batch_set_rhs_gate(pihm_batch *b, double gate);

/* Admit a watershed; *id receives its handle.  PIHM_GPU_ERR_NOMEM: no room now. */
int pihm_batch_add(pihm_batch *b, const pihm_batch_job *job, int32_t *id);

/* Admit n watersheds, preparing them (validation, renumbering, derived
 * constants) on `threads` host threads and admitting them in order; ids[k]
 * receives each handle, or -1 from the first one that fails or does not fit
 * on (the return code says why).  *admitted: how many were admitted. */
int pihm_batch_add_many(pihm_batch *b, const pihm_batch_job *jobs, int32_t n, int32_t threads, int32_t *ids,
                        int32_t *admitted);

/* Advance every resident watershed by up to max_rounds rounds (<= 0: until
 * all have finished).  *running receives the number still running. */
int pihm_batch_step(pihm_batch *b, int32_t max_rounds, int32_t *running);

/* PIHM_BATCH_RUNNING / _DONE / _FAILED, and the integrator's return code. */
int pihm_batch_poll(const pihm_batch *b, int32_t id, int32_t *status, int32_t *solver_rc);

/* Results of a finished (or failed) watershed; any output may be NULL.
 * y: [neq] reference order; outlet: [nsteps] */
int pihm_batch_result(pihm_batch *b, int32_t id, double *y, double *outlet, pihm_bdf_stats *stats,
                      int32_t *steps_done);

/* Free a watershed's arena ranges (after its results have been read). */
int pihm_batch_release(pihm_batch *b, int32_t id);

/* Rounds executed, kernels launched, arena occupancy and time so far:
 * host_ms building rounds and running the integrators, wait_ms blocked on the
 * device, and (with profiling on) the device time of the program kernel and
 * of the right-hand-side evaluations, from CUDA events. */
typedef struct pihm_batch_info {
    int64_t rounds, rhs_rounds, launches;
    int64_t elem_used, elem_hwm, resident;
    double host_ms, wait_ms, program_ms, rhs_ms;
    int32_t program_variant;  /* variant of the program kernel in use */
    int32_t tuning;           /* 1 while the tuner is still timing variants */
    int32_t rhs_shape;        /* block shape of the element kernel in use (pihm_batch_set_rhs_shape) */
    int32_t rhs_tuning;       /* 1 while the tuner is still timing shapes */
} pihm_batch_info;
int pihm_batch_get_info(const pihm_batch *b, pihm_batch_info *info);
int pihm_batch_set_profiling(pihm_batch *b, int on);

/* The program kernel comes in variants (0, 1, 2: a thread keeps 1, 2 or 4 of
 * its grid-stride entries in flight) that give identical results.  By default
 * (-1) the engine times them on its first large rounds and keeps the fastest;
 * 0..2 forces one. */
int pihm_batch_set_program_variant(pihm_batch *b, int32_t variant);

/* The right-hand side's element kernel (k_elem_main) comes in three block
 * shapes with the same register budget -- 0: 512 threads x 2 blocks per SM,
 * 1: 256 x 4, 2: 128 x 8 -- that give identical results: 256 x 4 is fastest
 * on one large mesh, smaller blocks spread a small or sparsely occupied
 * arena over more SMs.  By default (-1) the engine uses 256 x 4 until it has
 * timed the three on its first evaluations over at least 20,000 elements,
 * then keeps the fastest per element; 0..2 forces one. */
int pihm_batch_set_rhs_shape(pihm_batch *b, int32_t shape);

/* ---- serving --------------------------------------------------------------
 * Requests are submitted with an arrival time (seconds after the start of
 * pihm_serve_run).  From its arrival on, a request is prepared on one of
 * `workers` host threads while the GPU keeps integrating the resident
 * watersheds; prepared requests are admitted in arrival order as soon as the
 * arena has room, join the rounds in flight, and are retired (results copied
 * to the host, arena ranges freed) the moment they finish.  A request larger
 * than the whole arena fails with PIHM_GPU_ERR_NOMEM.  Submit every request
 * before pihm_serve_run; it returns when all have been served.  The job's
 * arrays are copied at submission; a deck job's deck, land parameters and
 * forcing series are not and must stay valid until pihm_serve_run returns. */
typedef struct pihm_serve_record {
    int32_t status;      /* PIHM_BATCH_RUNNING (queued or resident), _DONE, _FAILED */
    int32_t solver_rc;   /* integrator return code, or the admission error */
    int32_t nelem;
    double t_arrival, t_admit, t_done;  /* s from the start of pihm_serve_run; -1 if not reached */
} pihm_serve_record;

int pihm_serve_submit(pihm_batch *b, const pihm_batch_job *job, double arrival_s, int32_t *ticket);
int pihm_serve_run(pihm_batch *b, int32_t workers);
int pihm_serve_record_get(const pihm_batch *b, int32_t ticket, pihm_serve_record *rec);
/* y: [neq] reference order, outlet: [nsteps] (when the job recorded one) */
int pihm_serve_result(const pihm_batch *b, int32_t ticket, double *y, double *outlet, pihm_bdf_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* PIHM_BATCH_H */
