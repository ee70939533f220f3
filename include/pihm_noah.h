/*
 * pihm_noah.h -- the Noah land-surface model of Flux-PIHM on the device.
 *
 * Flux-PIHM (the reference built with _NOAH_) runs, every land-surface step,
 * Noah() (src/noah/noah.c:3-55: CalHum, FrozRain, net radiation and the
 * surface-flux driver SFlx with its snowpack, frozen-soil, soil-heat and
 * canopy physics) before the solve, and after every model step the _NOAH_
 * part of Summary (src/update.c:34-41: MassBalance's infiltration and
 * subsurface runoff, FindWaterTable, CalcLatFlx) followed by NoahHydrol
 * (src/noah/noah.c:57-160: FindWaterTable, the moisture clamps and SmFlx).
 * These entry points do the same on the GPU, one thread per element, and
 * write what the Flux-PIHM right-hand side reads (per-layer transpiration,
 * the water-table layer, the top layer's liquid moisture, the frozen-soil
 * factor, edir, ett and pcpdrp) into the context's own input planes, so a
 * coupled run keeps the land-surface state on the device.
 *
 * Arrays are in the reference's element order; per-layer arrays are
 * [nelem][PIHM_NOAH_MAXLYR] (layer index fastest), as elem_struct holds them
 * (MAXLYR = 11, src/include/pihm_const.h:84).  Units are the reference's.
 */
#ifndef PIHM_NOAH_H
#define PIHM_NOAH_H

#include <stdint.h>

#include "pihm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PIHM_NOAH_MAXLYR 11

/* Static per-element parameters of Noah (InitLsm, src/noah/lsm_init.c:3-44;
 * the soil and land-cover parameters InitSoil / InitLc derive, and the
 * universal parameters of the .lsm file). */
typedef struct pihm_noah_params {
  int32_t nelem;
  const int32_t *nsoil;   /* soil layers (2..11), DefSldpth */
  const double *sldpth;   /* layer thicknesses [nelem][11] (m) */
  const int32_t *nroot;   /* root layers, FindLayer(rzd) */
  const double *rtdis;    /* root distribution [nelem][11], RootDist */
  const int32_t *isurban; /* land cover is urban (SFlx's urban overrides); may be null */
  /* soil */
  const double *smcmax, *smcmin, *smcref, *smcwlt, *smcdry, *quartz, *csoil;
  const double *alpha, *beta, *ksatv, *porosity, *depth;
  const double *area; /* element area (MassBalance's subsurface runoff) */
  /* land cover (vegetation table) and the canopy parameters of epconst */
  const double *shdfac, *cmcfactr, *laimax, *laimin, *emissmax, *emissmin;
  const double *albedomax, *albedomin, *z0max, *z0min, *snup, *cfactr;
  const double *rgl, *rsmin, *rsmax, *topt, *hs;
  /* per-element universal parameters */
  const double *sbeta, *salp, *frzx, *fxexp, *czil, *lvcoef, *zbot, *tbot;
  const double *zlvl, *zlvl_wind, *snoalb;
} pihm_noah_params;

/* State Noah carries from step to step (the reference initialises it in
 * Initialize, src/initialize.c:139-175 and :619-700). */
typedef struct pihm_noah_state {
  const double *smc, *sh2o, *stc; /* [nelem][11] */
  const double *t1, *cmc, *sneqv, *snowh, *sndens, *ch, *cm, *snotime1;
  const double *albedo, *emissi, *q1, *ribb, *fcr;
} pihm_noah_state;

/* Forcing of one land-surface step, per element (ApplyForc's outputs:
 * wf.prcp (m/s), es.sfctmp (K), ps.rh (%), ps.sfcspd (m/s), ef.soldn and
 * ef.longwave (W/m2), ps.sfcprs (Pa), ps.proj_lai). */
typedef struct pihm_noah_forcing {
  const double *prcp, *sfctmp, *rh, *sfcspd, *soldn, *longwave, *sfcprs, *lai;
} pihm_noah_forcing;

/* Attach Noah to a context (allocates its planes; copies params and state).
 * The context's right-hand side switches to its Flux-PIHM form and reads
 * Noah's outputs from then on (and keeps its per-edge fluxes, which
 * MassBalance reads after each model step). */
int pihm_gpu_noah_init(pihm_gpu_ctx *ctx, const pihm_noah_params *p, const pihm_noah_state *s);
/* Replace the carried state (null fields keep theirs). */
int pihm_gpu_noah_set_state(pihm_gpu_ctx *ctx, const pihm_noah_state *s);
/* Upload the forcing of the next land-surface step. */
int pihm_gpu_noah_set_forcing(pihm_gpu_ctx *ctx, const pihm_noah_forcing *f);
/* Noah() over dt seconds (the land-surface step), then the right-hand side's
 * Flux-PIHM inputs from its results; asynchronous on the context's stream. */
int pihm_gpu_noah_step(pihm_gpu_ctx *ctx, double dt);
/* The state a run starts from (device, internal order): the previous state
 * MassBalance compares the first model step's end with, as the reference's
 * Initialize sets ws0 (src/initialize.c:700).  Without it the first
 * pihm_gpu_noah_post_step takes its own y as the previous state. */
int pihm_gpu_noah_begin(pihm_gpu_ctx *ctx, const double *y0_dev);
/* After a model step of `stepsize` seconds that ended at the device state
 * y (internal order): Summary's _NOAH_ part and NoahHydrol, then the
 * right-hand side's inputs.  Needs the last evaluation's fluxes, which the
 * context keeps while Noah is attached. */
int pihm_gpu_noah_post_step(pihm_gpu_ctx *ctx, const double *y_dev, double stepsize);

/* Fields that can be read back (reference order). */
enum {
  PIHM_NOAH_SMC = 0, PIHM_NOAH_SH2O, PIHM_NOAH_STC, PIHM_NOAH_ET, /* per layer */
  PIHM_NOAH_RUNOFF2_LYR, PIHM_NOAH_SMFLXV,                        /* per layer */
  PIHM_NOAH_T1 = 16, PIHM_NOAH_CMC, PIHM_NOAH_SNEQV, PIHM_NOAH_SNOWH, PIHM_NOAH_SNDENS,
  PIHM_NOAH_CH, PIHM_NOAH_CM, PIHM_NOAH_ALBEDO, PIHM_NOAH_EMISSI, PIHM_NOAH_Q1,
  PIHM_NOAH_FCR, PIHM_NOAH_EDIR, PIHM_NOAH_EC, PIHM_NOAH_ETT, PIHM_NOAH_ESNOW,
  PIHM_NOAH_ETP, PIHM_NOAH_DRIP, PIHM_NOAH_PCPDRP, PIHM_NOAH_SNOMLT, PIHM_NOAH_SSOIL,
  PIHM_NOAH_SHEAT, PIHM_NOAH_RUNOFF2, PIHM_NOAH_RUNOFF3, PIHM_NOAH_INFIL, PIHM_NOAH_NWTBL,
  PIHM_NOAH_SNOTIME1, PIHM_NOAH_SNCOVR, PIHM_NOAH_BETA, PIHM_NOAH_ETA, PIHM_NOAH_SOILM,
  PIHM_NOAH_NFIELDS
};
/* Copy field `field` to host memory: nelem values, or nelem x 11 for the
 * per-layer fields (layer fastest); synchronous. */
int pihm_gpu_noah_get(pihm_gpu_ctx *ctx, int field, double *out);

#ifdef __cplusplus
}
#endif
#endif /* PIHM_NOAH_H */
