/* PIHM land-surface step on the GPU: the forcing and the interception, snow
 * and evapotranspiration model that run before each land-surface interval of
 * the model-step loop (src/pihm.c:30-66, when (t - start) % LSM_STEP == 0):
 *
 *   ApplyForc (src/forcing.c:44-87)   the meteorological series of each
 *       station and the LAI series interpolated at t (IntrplForc,
 *       src/forcing.c:482-531; ApplyMeteoForc :262-376, ApplyLai :382-480),
 *       each element taking its station's precipitation (/1000), air
 *       temperature, relative humidity, wind speed and solar radiation
 *       (negative radiation as 0);
 *   IntcpSnowEt (src/is_sm_et.c:5-226) degree-day snow, canopy interception
 *       and drip, and the Penman-Monteith potential evaporation split into
 *       soil evaporation, canopy evaporation and transpiration.
 *
 * The step runs as one kernel over the elements.  It reads the state vector
 * the integrator holds (unsat and gw, which Summary leaves in ws) and writes
 * pcpdrp, edir and ett straight into the planes the right-hand side reads,
 * so nothing crosses to the host between land-surface steps; canopy storage
 * cmc and snow water equivalent sneqv stay on the device.  Only the
 * reference's non-Noah build has this path (its Flux-PIHM build runs Noah
 * instead; pihm_gpu_set_noah takes Noah's outputs).
 *
 * A context created with pihm_gpu_create gets the land-surface model by
 * pihm_gpu_land_init; pihm_gpu_set_forcing then stays available to override
 * the forcing planes by hand.  pihm_gpu_water_balance includes precipitation,
 * canopy evaporation, canopy storage and snow once the model is attached, as
 * PrintWaterBal does (src/print.c:337-542). */
#ifndef PIHM_LAND_H
#define PIHM_LAND_H

#include <stdint.h>

#include "pihm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Number of variables of a meteorological station record, in the order of
 * the .meteo file (src/include/pihm_const.h:48-55). */
#define PIHM_METEO_NVAR 7
enum { PIHM_METEO_PRCP = 0, PIHM_METEO_SFCTMP, PIHM_METEO_RH, PIHM_METEO_SFCSPD, PIHM_METEO_SOLAR,
       PIHM_METEO_LONGWV, PIHM_METEO_PRES };

/* Land types the monthly LAI and roughness-length tables cover (MonthlyLai,
 * MonthlyRl: src/forcing.c:532-716, 40 rows). */
#define PIHM_LAND_NLC 40

/* Per-element land-surface parameters (reference order, nelem each), as
 * Initialize leaves them in elem_struct:
 *   lc_type, meteo_type, lai_type  attrib.* (1-based; lai_type 0 = monthly
 *                                  LAI table of the land type)
 *   albedomin, albedomax           lc.* (the calibration's ALBEDO applied)
 *   shdfac                         lc.shdfac (VEGFRAC applied; 0 on bare soil)
 *   cmcfactr, cfactr               lc.* (canopy capacity per LAI, exponent)
 *   rgl, rsmin, rsmax, topt        epc.* (canopy resistance parameters)
 *   smcmin, smcwlt, smcref         soil.* (residual, wilting, reference moisture)
 *   zlvl_wind                      ps.zlvl_wind (the station's wind height)
 * The soil depth, porosity, root depth and surface elevation come from the
 * mesh the context was created with.  cal_edir, cal_ec, cal_ett are the
 * calibration's EDIR, EC and ETT factors. */
typedef struct pihm_land_params {
    int32_t nelem;
    const int32_t *lc_type, *meteo_type, *lai_type;
    const double *albedomin, *albedomax, *shdfac, *cmcfactr, *cfactr;
    const double *rgl, *rsmin, *rsmax, *topt;
    const double *smcmin, *smcwlt, *smcref;
    const double *zlvl_wind;
    double cal_edir, cal_ec, cal_ett;
} pihm_land_params;

/* Forcing series (tsdata_struct), concatenated: series k has len[k] knots
 * starting at knot off_k = len[0] + ... + len[k-1], knot times in seconds
 * since 1970-01-01 UTC (non-decreasing) and values [knot][nvar] with nvar
 * PIHM_METEO_NVAR for stations (the calibration's climate scenario already
 * applied, as InitForc does: src/init_forc.c:8-17) and 1 for LAI. */
typedef struct pihm_forcing_series {
    int32_t nmeteo;
    const int32_t *meteo_len;
    const int64_t *meteo_time;
    const double *meteo_data;
    int32_t nlai;
    const int32_t *lai_len;
    const int64_t *lai_time;
    const double *lai_data;
} pihm_forcing_series;

/* Attach the land-surface model to a context: copies the parameters and the
 * series to the device and sets cmc = sneqv = 0 (RelaxIc,
 * src/initialize.c:509-510).  Returns PIHM_GPU_ERR_ARG for a size mismatch,
 * a type outside 1..PIHM_LAND_NLC or outside the series given, or a series
 * with fewer than two knots or decreasing times.  May be called again to
 * replace the model. */
int pihm_gpu_land_init(pihm_gpu_ctx *ctx, const pihm_land_params *params, const pihm_forcing_series *series);

/* Canopy storage and snow water equivalent [nelem] from host arrays (a
 * restart file's ic.cmc and ic.sneqv, src/read_ic.c:3-39); NULL sets zero. */
int pihm_gpu_land_set_state(pihm_gpu_ctx *ctx, const double *cmc, const double *sneqv);

/* One land-surface step at model time t (seconds since 1970-01-01 UTC) over
 * a step of `stepsize` seconds (the reference passes LSM_STEP), reading unsat
 * and gw from the state y_dev [3*nelem + 2*nriver] (device, internal order,
 * like pihm_gpu_rhs).  Enqueued on the context's stream, nothing waits for
 * it.  Returns PIHM_GPU_ERR_ARG, with nothing enqueued, when t lies outside
 * one of the series (the reference exits there). */
int pihm_gpu_land_step(pihm_gpu_ctx *ctx, int64_t t, double stepsize, const double *y_dev);

/* A field of the last land-surface step copied to a host array [nelem] in
 * reference order (synchronises the context's stream). */
enum {
    PIHM_LAND_PRCP = 0,  /* wf.prcp, m s-1 */
    PIHM_LAND_PCPDRP,    /* wf.pcpdrp: throughfall, drip and melt reaching the surface */
    PIHM_LAND_EDIR,      /* wf.edir: soil evaporation */
    PIHM_LAND_ETT,       /* wf.ett: transpiration */
    PIHM_LAND_EC,        /* wf.ec: canopy evaporation */
    PIHM_LAND_DRIP,      /* wf.drip */
    PIHM_LAND_CMC,       /* ws.cmc, m */
    PIHM_LAND_SNEQV,     /* ws.sneqv, m */
    PIHM_LAND_NFIELD
};
int pihm_gpu_land_get(pihm_gpu_ctx *ctx, int field, double *out);

#ifdef __cplusplus
}
#endif
#endif /* PIHM_LAND_H */
