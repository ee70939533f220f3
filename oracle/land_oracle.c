/*
 * land_oracle.c -- CPU restatement of the PIHM land-surface step (test
 * infrastructure only: the checker for pihm_gpu_land_*, never on a product
 * path).
 *
 * Restates, loop for loop and in the same floating-point operation order,
 * the reference's non-Noah forcing step of src/pihm.c:30-66:
 *   ApplyForc (src/forcing.c:44-87): IntrplForc (src/forcing.c:482-531) on
 *     every meteorological station and LAI series, ApplyMeteoForc
 *     (src/forcing.c:262-376) and ApplyLai (src/forcing.c:382-480) per
 *     element;
 *   IntcpSnowEt (src/is_sm_et.c:5-226) per element, with MonthlyLai,
 *     MonthlyRl and MonthlyMf (src/forcing.c:532-798) and PIHMTime's month
 *     (src/time_func.c:3-22).
 * Elements in reference order, C library exp/log/pow/cos, OpenMP on the
 * reference's loops when built with -fopenmp.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "pihm_land.h"
#include "../pihm-cuda_gb300/csrc/land_tables.h"
#include "pihm_oracle.h"

static const double lai_tbl[PIHM_LAND_NLC][12] = {PIHM_MONTHLY_LAI};
static const double rl_tbl[PIHM_LAND_NLC][12] = {PIHM_MONTHLY_ROUGHNESS};
static const double mf_tbl[12] = {PIHM_MELT_FACTOR};

/* model constants (src/include/pihm_const.h:9-15) */
#define CP 1004.0
#define LVH2O 2.501e6
#define SIGMA 5.67e-8
#define RD 287.04
#define RV 461.5

typedef struct {
    int n, nvar, off;   /* knots, variables, first knot in the flat arrays */
    const long long *t; /* [n] */
    const double *d;    /* [n][nvar] */
    double value[PIHM_METEO_NVAR];
} series_t;

struct oracle_land {
    int ne, nmeteo, nlai;
    int *lc, *meteo, *lai_type;
    double *albedomin, *albedomax, *shdfac, *cmcfactr, *cfactr, *rgl, *rsmin, *rsmax, *topt, *smcmin,
        *smcwlt, *smcref, *zlvl, *zmax, *depth, *porosity, *rzd;
    double cal_edir, cal_ec, cal_ett;
    series_t *met, *lai;
    long long *tt;
    double *dd;
    /* element state and fluxes */
    double *cmc, *sneqv, *prcp, *sfctmp, *rh, *sfcspd, *soldn, *proj_lai, *albedo, *pcpdrp, *edir, *ett, *ec,
        *drip;
};

static double *dup(const double *a, int n)
{
    double *r = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    if (n > 0) memcpy(r, a, sizeof(double) * n);
    return r;
}
static int *dupi(const int *a, int n)
{
    int *r = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
    if (n > 0) memcpy(r, a, sizeof(int) * n);
    return r;
}

oracle_land *oracle_land_create(const pihm_land_params *p, const pihm_forcing_series *s, const double *zmax,
                                const double *depth, const double *porosity, const double *rzd)
{
    oracle_land *L = (oracle_land *)calloc(1, sizeof(*L));
    int ne = p->nelem, k;
    size_t nm = 0, nl = 0, o;
    L->ne = ne;
    L->nmeteo = s->nmeteo;
    L->nlai = s->nlai;
    L->lc = dupi(p->lc_type, ne);
    L->meteo = dupi(p->meteo_type, ne);
    L->lai_type = dupi(p->lai_type, ne);
    L->albedomin = dup(p->albedomin, ne);
    L->albedomax = dup(p->albedomax, ne);
    L->shdfac = dup(p->shdfac, ne);
    L->cmcfactr = dup(p->cmcfactr, ne);
    L->cfactr = dup(p->cfactr, ne);
    L->rgl = dup(p->rgl, ne);
    L->rsmin = dup(p->rsmin, ne);
    L->rsmax = dup(p->rsmax, ne);
    L->topt = dup(p->topt, ne);
    L->smcmin = dup(p->smcmin, ne);
    L->smcwlt = dup(p->smcwlt, ne);
    L->smcref = dup(p->smcref, ne);
    L->zlvl = dup(p->zlvl_wind, ne);
    L->zmax = dup(zmax, ne);
    L->depth = dup(depth, ne);
    L->porosity = dup(porosity, ne);
    L->rzd = dup(rzd, ne);
    L->cal_edir = p->cal_edir;
    L->cal_ec = p->cal_ec;
    L->cal_ett = p->cal_ett;
    for (k = 0; k < s->nmeteo; k++) nm += (size_t)s->meteo_len[k];
    for (k = 0; k < s->nlai; k++) nl += (size_t)s->lai_len[k];
    L->tt = (long long *)malloc(sizeof(long long) * (nm + nl + 1));
    L->dd = (double *)malloc(sizeof(double) * (nm * PIHM_METEO_NVAR + nl + 1));
    for (o = 0; o < nm; o++) L->tt[o] = s->meteo_time[o];
    for (o = 0; o < nl; o++) L->tt[nm + o] = s->lai_time[o];
    memcpy(L->dd, s->meteo_data, sizeof(double) * nm * PIHM_METEO_NVAR);
    if (nl) memcpy(L->dd + nm * PIHM_METEO_NVAR, s->lai_data, sizeof(double) * nl);
    L->met = (series_t *)calloc((size_t)s->nmeteo + 1, sizeof(series_t));
    L->lai = (series_t *)calloc((size_t)s->nlai + 1, sizeof(series_t));
    o = 0;
    for (k = 0; k < s->nmeteo; k++) {
        L->met[k].n = s->meteo_len[k];
        L->met[k].nvar = PIHM_METEO_NVAR;
        L->met[k].t = L->tt + o;
        L->met[k].d = L->dd + o * PIHM_METEO_NVAR;
        o += (size_t)s->meteo_len[k];
    }
    o = 0;
    for (k = 0; k < s->nlai; k++) {
        L->lai[k].n = s->lai_len[k];
        L->lai[k].nvar = 1;
        L->lai[k].t = L->tt + nm + o;
        L->lai[k].d = L->dd + nm * PIHM_METEO_NVAR + o;
        o += (size_t)s->lai_len[k];
    }
#define Z(f) L->f = (double *)calloc((size_t)(ne > 0 ? ne : 1), sizeof(double))
    Z(cmc); Z(sneqv); Z(prcp); Z(sfctmp); Z(rh); Z(sfcspd); Z(soldn); Z(proj_lai); Z(albedo);
    Z(pcpdrp); Z(edir); Z(ett); Z(ec); Z(drip);
#undef Z
    return L;
}

void oracle_land_destroy(oracle_land *L)
{
    if (!L) return;
    free(L->lc); free(L->meteo); free(L->lai_type);
    free(L->albedomin); free(L->albedomax); free(L->shdfac); free(L->cmcfactr); free(L->cfactr);
    free(L->rgl); free(L->rsmin); free(L->rsmax); free(L->topt); free(L->smcmin); free(L->smcwlt);
    free(L->smcref); free(L->zlvl); free(L->zmax); free(L->depth); free(L->porosity); free(L->rzd);
    free(L->tt); free(L->dd); free(L->met); free(L->lai);
    free(L->cmc); free(L->sneqv); free(L->prcp); free(L->sfctmp); free(L->rh); free(L->sfcspd);
    free(L->soldn); free(L->proj_lai); free(L->albedo); free(L->pcpdrp); free(L->edir); free(L->ett);
    free(L->ec); free(L->drip);
    free(L);
}

void oracle_land_set_state(oracle_land *L, const double *cmc, const double *sneqv)
{
    int i;
    for (i = 0; i < L->ne; i++) {
        L->cmc[i] = cmc ? cmc[i] : 0.0;
        L->sneqv[i] = sneqv ? sneqv[i] : 0.0;
    }
}

/* IntrplForc (src/forcing.c:482-531); -1 where the reference exits */
static int intrpl(series_t *ts, long long t)
{
    int j, first, middle, last;
    if (t < ts->t[0] || t > ts->t[ts->n - 1]) return -1;
    first = 1;
    last = ts->n - 1;
    while (first <= last) {
        middle = (first + last) / 2;
        if (t >= ts->t[middle - 1] && t <= ts->t[middle]) {
            for (j = 0; j < ts->nvar; j++)
                ts->value[j] = ((double)(ts->t[middle] - t) * ts->d[(size_t)(middle - 1) * ts->nvar + j] +
                                (double)(t - ts->t[middle - 1]) * ts->d[(size_t)middle * ts->nvar + j]) /
                               (double)(ts->t[middle] - ts->t[middle - 1]);
            break;
        } else if (ts->t[middle] > t) {
            last = middle - 1;
        } else {
            first = middle + 1;
        }
    }
    return 0;
}

static int month_of(long long t)
{
    time_t raw = (time_t)t;
    struct tm tm;
    gmtime_r(&raw, &tm);
    return tm.tm_mon + 1;
}

/* ApplyForc + IntcpSnowEt at time t over a step of `stepsize` seconds, with
 * the soil state unsat[ne], gw[ne] (ws.unsat, ws.gw).  Returns 0, or -1 when t
 * lies outside a series. */
int oracle_land_step(oracle_land *L, long long t, double stepsize, const double *unsat, const double *gw)
{
    int i, k, bad = 0;
    const double TSNOW = -3.0, TRAIN = 1.0, T0 = 0.0;
    const int month = month_of(t);

    /* ApplyMeteoForc: every station, then every element */
    for (k = 0; k < L->nmeteo; k++)
        if (intrpl(&L->met[k], t) != 0) bad = 1;
    for (k = 0; k < L->nlai; k++)
        if (intrpl(&L->lai[k], t) != 0) bad = 1;
    if (bad) return -1;
#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < L->ne; i++) {
        const double *v = L->met[L->meteo[i] - 1].value;
        L->prcp[i] = v[PIHM_METEO_PRCP] / 1000.0;
        L->sfctmp[i] = v[PIHM_METEO_SFCTMP];
        L->rh[i] = v[PIHM_METEO_RH];
        L->sfcspd[i] = v[PIHM_METEO_SFCSPD];
        L->soldn[i] = v[PIHM_METEO_SOLAR];
        L->soldn[i] = (L->soldn[i] > 0.0) ? L->soldn[i] : 0.0;
    }
    /* ApplyLai */
#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < L->ne; i++) {
        if (L->lai_type[i] > 0)
            L->proj_lai[i] = L->lai[L->lai_type[i] - 1].value[0];
        else
            L->proj_lai[i] = lai_tbl[L->lc[i] - 1][month - 1];
    }

    /* IntcpSnowEt */
#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < L->ne; i++) {
        double satn, betas, fr, alphar, etas, gammas, rs, pc, delta, gamma, radnet, sfctmp, wind, rh, vp, pres,
            lai, z0, ra, qvsat, qv, etp, isval, frac_snow, snow_rate, melt_rate, intcp_max, meltf;

        L->albedo[i] = 0.5 * (L->albedomin[i] + L->albedomax[i]);
        radnet = L->soldn[i] * (1.0 - L->albedo[i]);
        sfctmp = L->sfctmp[i] - 273.15;
        wind = L->sfcspd[i];
        rh = L->rh[i] / 100.0;

        vp = 611.2 * exp(17.67 * sfctmp / (sfctmp + 243.5)) * rh;
        pres = 101.325 * 1.0e3 * pow((293.0 - 0.0065 * L->zmax[i]) / 293.0, 5.26);
        qv = 0.622 * vp / pres;
        qvsat = 0.622 * (vp / rh) / pres;

        if (L->lai_type[i] > 0)
            lai = L->proj_lai[i];
        else
            lai = lai_tbl[L->lc[i] - 1][month - 1];

        meltf = mf_tbl[month - 1];

        frac_snow = (sfctmp < TSNOW) ? 1.0 : ((sfctmp > TRAIN) ? 0.0 : (TRAIN - sfctmp) / (TRAIN - TSNOW));
        snow_rate = frac_snow * L->prcp[i];
        L->sneqv[i] += snow_rate * stepsize;
        melt_rate = (sfctmp > T0) ? (sfctmp - T0) * meltf : 0.0;
        if (L->sneqv[i] > melt_rate * stepsize) {
            L->sneqv[i] -= melt_rate * stepsize;
        } else {
            melt_rate = L->sneqv[i] / stepsize;
            L->sneqv[i] = 0.0;
        }

        intcp_max = L->cmcfactr[i] * lai * L->shdfac[i];
        z0 = rl_tbl[L->lc[i] - 1][month - 1];
        ra = log(L->zlvl[i] / z0) * log(10.0 * L->zlvl[i] / z0) / (wind * 0.16);
        gamma = 4.0 * 0.7 * SIGMA * RD / CP * pow(sfctmp + 273.15, 4) / (pres / ra) + 1.0;
        delta = LVH2O * LVH2O * 0.622 / RV / CP / pow(sfctmp + 273.15, 2) * qvsat;
        etp = (radnet * delta + gamma * (1.2 * LVH2O * (qvsat - qv) / ra)) / (1000.0 * LVH2O * (delta + gamma));

        if (L->depth[i] - gw[i] < L->rzd[i]) {
            satn = 1.0;
        } else {
            const double r = unsat[i] / (L->depth[i] - gw[i]);
            satn = (r > 1.0) ? 1.0 : ((r < 0.0) ? 0.0 : 0.5 * (1.0 - cos(3.14 * r)));
        }
        betas = (satn * L->porosity[i] + L->smcmin[i] - L->smcwlt[i]) / (L->smcref[i] - L->smcwlt[i]);
        betas = (betas < 0.0001) ? 0.0001 : ((betas > 1.0) ? 1.0 : betas);
        L->edir[i] = (1.0 - L->shdfac[i]) * pow(betas, 2) * etp;
        L->edir[i] *= L->cal_edir;
        L->edir[i] = (L->edir[i] < 0.0) ? 0.0 : L->edir[i];

        if (lai > 0.0) {
            const double cmc = L->cmc[i];
            L->ec[i] = L->shdfac[i] *
                       pow(((cmc < 0.0) ? 0.0 : ((cmc > intcp_max) ? intcp_max : cmc)) / intcp_max, L->cfactr[i]) *
                       etp;
            L->ec[i] *= L->cal_ec;
            L->ec[i] = (L->ec[i] < 0.0) ? 0.0 : L->ec[i];

            fr = 1.1 * radnet / (L->rgl[i] * lai);
            fr = (fr < 0.0) ? 0.0 : fr;
            alphar = (1.0 + fr) / (fr + (L->rsmin[i] / L->rsmax[i]));
            alphar = (alphar > 10000.0) ? 10000.0 : alphar;
            etas = 1.0 - 0.0016 * (pow((L->topt[i] - 273.15 - sfctmp), 2));
            etas = (etas < 0.0001) ? 0.0001 : etas;
            gammas = 1.0 / (1.0 + 0.00025 * (vp / rh - vp));
            gammas = (gammas < 0.01) ? 0.01 : gammas;
            rs = L->rsmin[i] * alphar / (betas * lai * etas * gammas);
            rs = (rs > L->rsmax[i]) ? L->rsmax[i] : rs;
            pc = (1.0 + delta / gamma) / (1.0 + rs / ra + delta / gamma);
            /* the reference divides only the unclamped branch here */
            L->ett[i] = L->shdfac[i] * pc *
                        (1.0 - pow((cmc < 0.0) ? 0.0 : ((cmc > intcp_max) ? intcp_max : cmc) / intcp_max,
                                   L->cfactr[i])) *
                        etp;
            L->ett[i] *= L->cal_ett;
            L->ett[i] = (L->ett[i] < 0.0) ? 0.0 : L->ett[i];
            L->ett[i] = ((gw[i] < (L->depth[i] - L->rzd[i])) && unsat[i] <= 0.0) ? 0.0 : L->ett[i];
            L->drip[i] = (cmc <= 0.0) ? 0.0 : 6.52E-7 * intcp_max * exp(3.89 * cmc / intcp_max);
        } else {
            L->ett[i] = 0.0;
            L->ec[i] = 0.0;
            L->drip[i] = 0.0;
        }
        if (L->drip[i] < 0.0) L->drip[i] = 0.0;
        if (L->drip[i] * stepsize > L->cmc[i]) L->drip[i] = L->cmc[i] / stepsize;

        isval = L->cmc[i] + (1.0 - frac_snow) * L->prcp[i] * L->shdfac[i] * stepsize - L->ec[i] * stepsize -
                L->drip[i] * stepsize;
        if (isval > intcp_max) {
            L->cmc[i] = intcp_max;
            L->drip[i] += (isval - intcp_max) / stepsize;
        } else if (isval < 0.0) {
            L->cmc[i] = 0.0;
            if (L->ec[i] + L->drip[i] > 0.0) {
                L->ec[i] = L->ec[i] / (L->ec[i] + L->drip[i]) *
                           (L->cmc[i] + (1.0 - frac_snow) * L->prcp[i] * L->shdfac[i] * stepsize);
                L->drip[i] = L->drip[i] / (L->ec[i] + L->drip[i]) *
                             (L->cmc[i] + (1.0 - frac_snow) * L->prcp[i] * L->shdfac[i] * stepsize);
            }
        } else {
            L->cmc[i] = isval;
        }
        L->pcpdrp[i] = (1.0 - L->shdfac[i]) * (1.0 - frac_snow) * L->prcp[i] + L->drip[i] + melt_rate;
    }
    return 0;
}

void oracle_land_get(const oracle_land *L, int field, double *out)
{
    const double *src = NULL;
    switch (field) {
    case PIHM_LAND_PRCP: src = L->prcp; break;
    case PIHM_LAND_PCPDRP: src = L->pcpdrp; break;
    case PIHM_LAND_EDIR: src = L->edir; break;
    case PIHM_LAND_ETT: src = L->ett; break;
    case PIHM_LAND_EC: src = L->ec; break;
    case PIHM_LAND_DRIP: src = L->drip; break;
    case PIHM_LAND_CMC: src = L->cmc; break;
    case PIHM_LAND_SNEQV: src = L->sneqv; break;
    default: return;
    }
    memcpy(out, src, sizeof(double) * L->ne);
}

/* The monthly tables at time t for land type lc: LAI, roughness length, melt
 * factor (MonthlyLai, MonthlyRl, MonthlyMf). */
void oracle_land_monthly(long long t, int lc, double *out3)
{
    const int m = month_of(t);
    out3[0] = lai_tbl[lc - 1][m - 1];
    out3[1] = rl_tbl[lc - 1][m - 1];
    out3[2] = mf_tbl[m - 1];
}
