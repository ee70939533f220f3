/*
 * pihm_oracle.c -- CPU restatement of the PIHM right-hand side (test
 * infrastructure only; see pihm_oracle.h).
 *
 * Every function below names the reference function it restates
 * (lj-cug/PIHM-CUDA, path within that project) and keeps its operation order,
 * so that on the same compiler and libm the results agree bit for bit with the
 * reference compiled from its own sources (oracle/Makefile, target ref).
 *
 * Two facts of the reference build that change the arithmetic:
 *   - src/include/pihm_func.h:4 defines _ARITH_ unconditionally, so AvgKv,
 *     SubFlowRiverToRiver and SubFlowElemToRiver use arithmetic means;
 *   - Infil reads wf.ovlflow on river edges before RiverFlow rewrites them in
 *     the same call, i.e. it sees the previous call's value.
 */
#include "pihm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#if defined(_OPENMP)
#include <omp.h>
#endif

/* constants, src/include/pihm_const.h:64-156 */
#define NUM_EDGE 3
#define NUM_RIVFLX 11
#define GRAV 9.80665
#define PSIMIN -70.0
#define DEPRSTG 1E-4
#define GRADMIN 5E-8
#define SATMIN 0.1
#define RIVGRADMIN 0.05
#define UP_CHANL2CHANL 0
#define DOWN_CHANL2CHANL 1
#define LEFT_SURF2CHANL 2
#define RIGHT_SURF2CHANL 3
#define LEFT_AQUIF2CHANL 4
#define RIGHT_AQUIF2CHANL 5
#define CHANL_LKG 6
#define LEFT_AQUIF2AQUIF 7
#define RIGHT_AQUIF2AQUIF 8
#define DOWN_AQUIF2AQUIF 9
#define UP_AQUIF2AQUIF 10
#define DIRICHLET -1
#define NEUMANN -2
#define ZERO_DPTH_GRAD -3
#define CRIT_DPTH -4
#define NO_FLOW 0
#define RECTANGLE 1
#define TRIANGLE 2
#define QUADRATIC 3
#define CUBIC 4
#define KINEMATIC 1
#define DIFF_WAVE 2

#define NOAH_MAXLYR 11 /* MAXLYR, src/include/pihm_const.h:84 */

typedef struct soil_p {
    double depth, ksath, ksatv, kinfv, dinf, alpha, beta, porosity, dmac,
        kmach, kmacv, areafv, areafh;
} soil_p;

typedef struct elem_t {
    int nabr[NUM_EDGE];
    int bc_type[NUM_EDGE];
    double area, zmin, zmax;
    double edge[NUM_EDGE], nabrdist[NUM_EDGE], nabr_x[NUM_EDGE],
        nabr_y[NUM_EDGE];
    soil_p soil;
    double rough, rzd;
    double bc[NUM_EDGE];
    /* water states */
    double surf, unsat, gw, surfh, ws0_surf;
    /* water fluxes */
    double ovlflow[NUM_EDGE], subsurf[NUM_EDGE];
    double pcpdrp, infil, rechg, edir, ett;
    double edir_surf, edir_unsat, edir_gw, ett_unsat, ett_gw;
    /* Flux-PIHM (_NOAH_) inputs Noah sets once per model step */
    double et[NOAH_MAXLYR], sh2o0, smcmin, smcmax, fcr, gwet;
    int nwtbl, nroot;
} elem_t;

typedef struct river_t {
    int ind, down, leftele, rightele, intrpl_ord, bc_type;
    double area, zmin, zmax, zbed, node_zmax, dist_left, dist_right;
    double depth, coeff, length, width;
    double rough, cwr, ksath, ksatv, bedthick, porosity;
    double bc;
    double stage, gw;
    double rivflow[NUM_RIVFLX];
} river_t;

struct oracle_model {
    int ulp_perturb; /* see oracle_set_ulp_perturb */
    int nelem, nriver;
    int noah; /* 1: the Flux-PIHM (_NOAH_) variants of EtExtract and Infil */
    int surf_mode, riv_mode;
    double stepsize;
    elem_t *elem;
    river_t *river;
    double *dhbydx, *dhbydy;
};

void oracle_set_ulp_perturb(oracle_model *m, int s) { m->ulp_perturb = (s > 0) - (s < 0); }

int oracle_num_threads(void)
{
#if defined(_OPENMP)
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_num_threads(int n)
{
#if defined(_OPENMP)
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

oracle_model *oracle_create(const pihm_gpu_mesh *g, int surf_mode,
                            int riv_mode, double stepsize)
{
    oracle_model *m = (oracle_model *)calloc(1, sizeof(*m));
    int i, j;
    if (!m) return NULL;
    m->nelem = g->nelem;
    m->nriver = g->nriver;
    m->surf_mode = surf_mode;
    m->riv_mode = riv_mode;
    m->stepsize = stepsize;
    m->elem = (elem_t *)calloc((size_t)g->nelem, sizeof(elem_t));
    m->river = (river_t *)calloc((size_t)(g->nriver > 0 ? g->nriver : 1),
                                 sizeof(river_t));
    m->dhbydx = (double *)calloc((size_t)g->nelem, sizeof(double));
    m->dhbydy = (double *)calloc((size_t)g->nelem, sizeof(double));
    for (i = 0; i < g->nelem; i++) {
        elem_t *e = &m->elem[i];
        for (j = 0; j < NUM_EDGE; j++) {
            e->nabr[j] = g->nabr[3 * i + j];
            e->bc_type[j] = g->bc_type[3 * i + j];
            e->edge[j] = g->edge[3 * i + j];
            e->nabrdist[j] = g->nabrdist[3 * i + j];
            e->nabr_x[j] = g->nabr_x[3 * i + j];
            e->nabr_y[j] = g->nabr_y[3 * i + j];
        }
        e->area = g->area[i];
        e->zmin = g->zmin[i];
        e->zmax = g->zmax[i];
        e->soil.depth = g->depth[i];
        e->soil.ksath = g->ksath[i];
        e->soil.ksatv = g->ksatv[i];
        e->soil.kinfv = g->kinfv[i];
        e->soil.dinf = g->dinf[i];
        e->soil.alpha = g->alpha[i];
        e->soil.beta = g->beta[i];
        e->soil.porosity = g->porosity[i];
        e->soil.dmac = g->dmac[i];
        e->soil.kmach = g->kmach[i];
        e->soil.kmacv = g->kmacv[i];
        e->soil.areafv = g->areafv[i];
        e->soil.areafh = g->areafh[i];
        e->rough = g->rough[i];
        e->rzd = g->rzd[i];
    }
    for (i = 0; i < g->nriver; i++) {
        river_t *r = &m->river[i];
        r->ind = i + 1;
        r->down = g->down[i];
        r->leftele = g->leftele[i];
        r->rightele = g->rightele[i];
        r->intrpl_ord = g->intrpl_ord[i];
        r->bc_type = g->riverbc_type[i];
        r->area = g->riv_area[i];
        r->zmin = g->riv_zmin[i];
        r->zmax = g->riv_zmax[i];
        r->zbed = g->riv_zbed[i];
        r->node_zmax = g->riv_node_zmax[i];
        r->dist_left = g->riv_dist_left[i];
        r->dist_right = g->riv_dist_right[i];
        r->depth = g->riv_depth[i];
        r->coeff = g->riv_coeff[i];
        r->length = g->riv_length[i];
        r->width = g->riv_width[i];
        r->rough = g->riv_rough[i];
        r->cwr = g->riv_cwr[i];
        r->ksath = g->riv_ksath[i];
        r->ksatv = g->riv_ksatv[i];
        r->bedthick = g->riv_bedthick[i];
        r->porosity = g->riv_porosity[i];
    }
    return m;
}

void oracle_destroy(oracle_model *m)
{
    if (!m) return;
    free(m->elem);
    free(m->river);
    free(m->dhbydx);
    free(m->dhbydy);
    free(m);
}

void oracle_set_forcing(oracle_model *m, const double *pcpdrp,
                        const double *edir, const double *ett)
{
    int i;
    for (i = 0; i < m->nelem; i++) {
        if (pcpdrp) m->elem[i].pcpdrp = pcpdrp[i];
        if (edir) m->elem[i].edir = edir[i];
        if (ett) m->elem[i].ett = ett[i];
    }
}

void oracle_set_bc(oracle_model *m, const double *elem_bc,
                   const double *river_bc)
{
    int i, j;
    if (elem_bc)
        for (i = 0; i < m->nelem; i++)
            for (j = 0; j < NUM_EDGE; j++)
                m->elem[i].bc[j] = elem_bc[3 * i + j];
    if (river_bc)
        for (i = 0; i < m->nriver; i++) m->river[i].bc = river_bc[i];
}

void oracle_set_ws0_surf(oracle_model *m, const double *ws0_surf)
{
    int i;
    for (i = 0; i < m->nelem; i++) m->elem[i].ws0_surf = ws0_surf[i];
}

/* Flux-PIHM inputs (see oracle_set_noah in pihm_oracle.h). */
int oracle_set_noah(oracle_model *m, const double *et, int nlayers, const int *nwtbl, const int *nroot,
                    const double *sh2o0, const double *smcmin, const double *smcmax, const double *fcr)
{
    int i, j;
    if (nlayers < 0 || nlayers > NOAH_MAXLYR) return -1;
    m->noah = 1;
    for (i = 0; i < m->nelem; i++) {
        elem_t *e = &m->elem[i];
        for (j = 0; j < NOAH_MAXLYR; j++) e->et[j] = (j < nlayers) ? et[(size_t)nlayers * i + j] : 0.0;
        e->nwtbl = nwtbl[i];
        e->nroot = nroot[i];
        e->sh2o0 = sh2o0[i];
        e->smcmin = smcmin[i];
        e->smcmax = smcmax[i];
        e->fcr = fcr[i];
    }
    return 0;
}

void oracle_set_river_edge_ovlflow(oracle_model *m, const double *ovlflow)
{
    int i, j;
    for (i = 0; i < m->nelem; i++)
        for (j = 0; j < NUM_EDGE; j++)
            if (m->elem[i].nabr[j] < 0)
                m->elem[i].ovlflow[j] = ovlflow[3 * i + j];
}

/* ------------------------------------------------------------------ */
/* Soil hydraulics                                                    */
/* ------------------------------------------------------------------ */

/* Last-bit sensitivity of the reference's arithmetic (test infrastructure):
 * with a model's ulp_perturb set to +1 or -1, every pow() and log() result of
 * its evaluations moves by one unit in the last place in that direction.  Two
 * correct libms can differ by that much, and the tests use the rows' movement
 * to bound how far the reference's own roundings let each row go.  With
 * ulp_perturb 0 (the default) the arithmetic is exactly the reference's.
 * Evaluations of different models must not overlap in time (they do not: one
 * evaluation at a time, each setting this from its model). */
static int g_ulp_perturb = 0;

static double nudge(double r)
{
    if (g_ulp_perturb == 0 || r == 0.0 || !isfinite(r)) return r;
    return nextafter(r, g_ulp_perturb > 0 ? INFINITY : -INFINITY);
}

/* exact results (pow(1, y) = 1, pow(x, 1) = x, log(1) = 0) are exact in
 * every libm and stay as they are */
static double ppow(double x, double y)
{
    const double r = pow(x, y);
    return (x == 1.0 || y == 1.0 || y == 0.0) ? r : nudge(r);
}
static double plog(double x) { return nudge(log(x)); }

/* KrFunc, src/soil.c:8-13 */
static double KrFunc(double beta, double satn)
{
    return sqrt(satn) *
        (1.0 - ppow(1.0 - ppow(satn, beta / (beta - 1.0)), (beta - 1.0) / beta)) *
        (1.0 - ppow(1.0 - ppow(satn, beta / (beta - 1.0)), (beta - 1.0) / beta));
}

/* Psi, src/vert_flow.c:272-278 */
static double Psi(double satn, double alpha, double beta)
{
    satn = (satn < SATMIN) ? SATMIN : satn;
    return -ppow(ppow(1.0 / satn, beta / (beta - 1.0)) - 1.0, 1.0 / beta) / alpha;
}

/* SurfH, src/hydrol.c:100-134 (DEPRSTG != 0 branch) */
static double SurfH(double surfeqv)
{
    double surfh;
    if (surfeqv < 0.0)
        surfh = 0.0;
    else if (surfeqv <= 0.5 * DEPRSTG)
        surfh = sqrt(2.0 * DEPRSTG * surfeqv);
    else
        surfh = DEPRSTG + (surfeqv - 0.5 * DEPRSTG);
    return surfh;
}

/* EffKh, src/lat_flow.c:248-277 */
static double EffKh(const soil_p *soil, double gw)
{
    double k1, k2, d1, d2;
    gw = (gw > 0.0) ? gw : 0.0;
    if (gw > soil->depth - soil->dmac) {
        k1 = soil->kmach * soil->areafv + soil->ksath * (1.0 - soil->areafv);
        k2 = soil->ksath;
        if (gw > soil->depth) {
            d1 = soil->dmac;
            d2 = soil->depth - soil->dmac;
        } else {
            d1 = gw - (soil->depth - soil->dmac);
            d2 = soil->depth - soil->dmac;
        }
        return (k1 * d1 + k2 * d2) / (d1 + d2);
    }
    return soil->ksath;
}

/* AvgHsurf, src/lat_flow.c:187-215 */
static double AvgHsurf(double diff, double hsurf, double hnabr)
{
    double avg_h;
    if (diff > 0.0)
        avg_h = (hsurf > DEPRSTG) ? 1.0 * (hsurf - DEPRSTG) : 0.0;
    else
        avg_h = (hnabr > DEPRSTG) ? 1.0 * (hnabr - DEPRSTG) : 0.0;
    return avg_h;
}

/* AvgH, src/lat_flow.c:217-237 */
static double AvgH(double diff, double hsub, double hnabr)
{
    double avg_h = 0.0;
    if (diff > 0.0) {
        if (hsub > 0.0) avg_h = hsub;
    } else {
        if (hnabr > 0.0) avg_h = hnabr;
    }
    return avg_h;
}

/* DhByDl, src/lat_flow.c:239-246 */
static double DhByDl(const double *l1, const double *l2, const double *surfh)
{
    return -1.0 *
        (l1[2] * (surfh[1] - surfh[0]) + l1[1] * (surfh[0] - surfh[2]) +
         l1[0] * (surfh[2] - surfh[1])) /
        (l2[2] * (l1[1] - l1[0]) + l2[1] * (l1[0] - l1[2]) +
         l2[0] * (l1[2] - l1[1]));
}

/* OverLandFlow, src/lat_flow.c:279-283 */
static double OverLandFlow(double avg_h, double grad_h, double avg_sf,
                           double crossa, double avg_rough)
{
    return crossa * ppow(avg_h, 0.6666667) * grad_h /
        (sqrt(avg_sf) * avg_rough);
}

/* ------------------------------------------------------------------ */
/* Element lateral flow                                               */
/* ------------------------------------------------------------------ */

/* SubFlowElemToElem, src/lat_flow.c:285-309 */
static double SubFlowElemToElem(const elem_t *e, const elem_t *n, int j)
{
    double diff_h, avg_h, grad_h, effk, effk_nabr, avg_ksat;
    diff_h = (e->gw + e->zmin) - (n->gw + n->zmin);
    avg_h = AvgH(diff_h, e->gw, n->gw);
    grad_h = diff_h / e->nabrdist[j];
    effk = EffKh(&e->soil, e->gw);
    effk_nabr = EffKh(&n->soil, n->gw);
    avg_ksat = 0.5 * (effk + effk_nabr);
    return avg_ksat * grad_h * avg_h * e->edge[j];
}

/* OvlFlowElemToElem, src/lat_flow.c:311-338 */
static double OvlFlowElemToElem(const elem_t *e, const elem_t *n, int j,
                                double avg_sf, int surf_mode)
{
    double diff_h, avg_h, grad_h, avg_rough, crossa;
    diff_h = (surf_mode == KINEMATIC) ?
        e->zmax - n->zmax :
        (e->surfh + e->zmax) - (n->surfh + n->zmax);
    avg_h = AvgHsurf(diff_h, e->surfh, n->surfh);
    grad_h = diff_h / e->nabrdist[j];
    if (surf_mode == KINEMATIC)
        avg_sf = (grad_h > 0.0) ? grad_h : GRADMIN;
    else
        avg_sf = (avg_sf > GRADMIN) ? avg_sf : GRADMIN;
    avg_rough = 0.5 * (e->rough + n->rough);
    crossa = avg_h * e->edge[j];
    return OverLandFlow(avg_h, grad_h, avg_sf, crossa, avg_rough);
}

/* BoundFluxElem, src/lat_flow.c:340-382 */
static void BoundFluxElem(elem_t *e, int j)
{
    int bc_type = e->bc_type[j];
    double diff_h, avg_h, effk, avg_ksat, grad_h;
    if (bc_type == NO_FLOW) {
        e->ovlflow[j] = 0.0;
        e->subsurf[j] = 0.0;
    } else if (bc_type > 0) {
        e->ovlflow[j] = 0.0;
        diff_h = e->gw + e->zmin - e->bc[j];
        avg_h = AvgH(diff_h, e->gw, e->bc[j] - e->zmin);
        effk = EffKh(&e->soil, e->gw);
        avg_ksat = effk;
        grad_h = diff_h / e->nabrdist[j];
        e->subsurf[j] = avg_ksat * grad_h * avg_h * e->edge[j];
    } else {
        e->ovlflow[j] = 0.0;
        e->subsurf[j] = -e->bc[j];
    }
}

/* FrictSlope, src/lat_flow.c:130-185 */
static void FrictSlope(oracle_model *m)
{
    int i;
    const elem_t *elem = m->elem;
    const river_t *river = m->river;
#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < m->nelem; i++) {
        int j;
        double surfh[NUM_EDGE];
        if (m->surf_mode == DIFF_WAVE) {
            for (j = 0; j < NUM_EDGE; j++) {
                int nb = elem[i].nabr[j];
                if (nb > 0) {
                    const elem_t *n = &elem[nb - 1];
                    surfh[j] = n->zmax + n->surfh;
                } else if (nb < 0) {
                    const river_t *r = &river[-nb - 1];
                    if (r->stage > r->depth)
                        surfh[j] = r->zbed + r->stage;
                    else
                        surfh[j] = r->zmax;
                } else {
                    if (elem[i].bc_type[j] == NO_FLOW)
                        surfh[j] = elem[i].zmax + elem[i].surfh;
                    else
                        surfh[j] = elem[i].bc[j];
                }
            }
            m->dhbydx[i] = DhByDl(elem[i].nabr_y, elem[i].nabr_x, surfh);
            m->dhbydy[i] = DhByDl(elem[i].nabr_x, elem[i].nabr_y, surfh);
        }
    }
}

/* LateralFlow, src/lat_flow.c:3-128 (no _FBR_) */
static void LateralFlow(oracle_model *m)
{
    int i;
    elem_t *elem = m->elem;
    const double *dhbydx = m->dhbydx, *dhbydy = m->dhbydy;
    FrictSlope(m);
#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < m->nelem; i++) {
        int j;
        double avg_sf;
        for (j = 0; j < NUM_EDGE; j++) {
            int nb = elem[i].nabr[j];
            if (nb > 0) {
                const elem_t *n = &elem[nb - 1];
                int k = nb - 1;
                elem[i].subsurf[j] = SubFlowElemToElem(&elem[i], n, j);
                avg_sf = 0.5 *
                    (sqrt(dhbydx[i] * dhbydx[i] + dhbydy[i] * dhbydy[i]) +
                     sqrt(dhbydx[k] * dhbydx[k] + dhbydy[k] * dhbydy[k]));
                elem[i].ovlflow[j] =
                    OvlFlowElemToElem(&elem[i], n, j, avg_sf, m->surf_mode);
            } else if (nb < 0) {
                /* river edge: written by RiverToElem */
            } else {
                BoundFluxElem(&elem[i], j);
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* Element vertical flow                                              */
/* ------------------------------------------------------------------ */

/* EffKinf, src/vert_flow.c:211-270 */
static double EffKinf(const soil_p *soil, double dh_by_dz, double ksatfunc,
                      double elemsatn, double applrate, double surfh)
{
    double keff = 0.0, kmax;
    const double BETA_CRACK = 2.0;
    if (soil->areafh == 0.0) {
        keff = soil->kinfv * ksatfunc;
    } else if (surfh > DEPRSTG) {
        keff = soil->kinfv * (1.0 - soil->areafh) * ksatfunc +
            soil->kmacv * soil->areafh;
    } else {
        if (applrate <= dh_by_dz * soil->kinfv * ksatfunc) {
            keff = soil->kinfv * ksatfunc;
        } else {
            kmax = dh_by_dz * (soil->kmacv * soil->areafh +
                               soil->kinfv * (1.0 - soil->areafh) * ksatfunc);
            if (applrate < kmax)
                keff = soil->kinfv * (1.0 - soil->areafh) * ksatfunc +
                    soil->kmacv * soil->areafh * KrFunc(BETA_CRACK, elemsatn);
            else
                keff = soil->kinfv * (1.0 - soil->areafh) * ksatfunc +
                    soil->kmacv * soil->areafh;
        }
    }
    return keff;
}

/* Infil, src/vert_flow.c:33-130; with noah, the saturation of the
 * unsaturated branch is Noah's top layer (src/vert_flow.c:94-98) */
static double Infil(const elem_t *e, double dt, int noah)
{
    double applrate, wetfrac, dh_by_dz, satn, satkfunc, infil, infil_max,
        kinf, deficit, psi_u, h_u;
    int j;
    const soil_p *soil = &e->soil;
    if (e->unsat + e->gw > soil->depth) {
        infil = 0.0;
    } else {
        applrate = 0.0;
        for (j = 0; j < NUM_EDGE; j++) applrate += -e->ovlflow[j] / e->area;
        applrate = (applrate > 0.0) ? applrate : 0.0;
        applrate += e->pcpdrp;

        wetfrac = e->surfh / DEPRSTG;
        wetfrac = (wetfrac > 0.0) ? wetfrac : 0.0;
        wetfrac = (wetfrac < 1.0) ? wetfrac : 1.0;

        if (e->gw > soil->depth - soil->dinf) {
            dh_by_dz = (e->surfh + e->zmax - (e->gw + e->zmin)) /
                (0.5 * (e->surfh + soil->dinf));
            dh_by_dz = (e->surfh <= 0.0 && dh_by_dz > 0.0) ? 0.0 : dh_by_dz;
            satn = 1.0;
            satkfunc = KrFunc(soil->beta, satn);
            kinf = EffKinf(soil, dh_by_dz, satkfunc, satn, applrate, e->surfh);
            infil = kinf * dh_by_dz;
        } else {
            deficit = soil->depth - e->gw;
            if (noah)
                satn = (e->sh2o0 - e->smcmin) / (e->smcmax - e->smcmin);
            else
                satn = e->unsat / deficit;
            satn = (satn > 1.0) ? 1.0 : satn;
            satn = (satn < SATMIN) ? SATMIN : satn;
            psi_u = Psi(satn, soil->alpha, soil->beta);
            psi_u = (psi_u > PSIMIN) ? psi_u : PSIMIN;
            h_u = psi_u + e->zmax - 0.5 * soil->dinf;
            dh_by_dz = (e->surfh + e->zmax - h_u) /
                (0.5 * (e->surfh + soil->dinf));
            dh_by_dz = (e->surfh <= 0.0 && dh_by_dz > 0.0) ? 0.0 : dh_by_dz;
            satkfunc = KrFunc(soil->beta, satn);
            kinf = EffKinf(soil, dh_by_dz, satkfunc, satn, applrate, e->surfh);
            infil = kinf * dh_by_dz;
            infil = (infil > 0.0) ? infil : 0.0;
        }
        infil_max = applrate + ((e->ws0_surf > 0.0) ? e->ws0_surf / dt : 0.0);
        infil = (infil > infil_max) ? infil_max : infil;
        infil *= wetfrac;
    }
    return infil;
}

/* AvgKv, src/vert_flow.c:172-209 (the _ARITH_ branch) */
static double AvgKv(const soil_p *soil, double deficit, double gw,
                    double satkfunc)
{
    double k1, k2, k3, d1, d2, d3;
    if (deficit > soil->dmac) {
        k1 = satkfunc * soil->ksatv;
        d1 = soil->dmac;
        k2 = satkfunc * soil->ksatv;
        d2 = deficit - soil->dmac;
        k3 = soil->ksatv;
        d3 = gw;
    } else {
        k1 = satkfunc * soil->ksatv;
        d1 = deficit;
        k2 = (soil->areafh > 0.0) ?
            soil->kmacv * soil->areafh + soil->ksatv * (1.0 - soil->areafh) :
            soil->ksatv;
        d2 = soil->dmac - deficit;
        k3 = soil->ksatv;
        d3 = gw - (soil->dmac - deficit);
    }
    return (k1 * d1 + k2 * d2 + k3 * d3) / (d1 + d2 + d3);
}

/* Recharge, src/vert_flow.c:132-170 */
static double Recharge(const elem_t *e)
{
    double satn, satkfunc, dh_by_dz, psi_u, kavg, deficit, rechg;
    const soil_p *soil = &e->soil;
    if (e->gw > soil->depth - soil->dinf) {
        rechg = e->infil;
    } else {
        deficit = soil->depth - e->gw;
        satn = e->unsat / deficit;
        satn = (satn > 1.0) ? 1.0 : satn;
        satn = (satn < SATMIN) ? SATMIN : satn;
        satkfunc = KrFunc(soil->beta, satn);
        psi_u = Psi(satn, soil->alpha, soil->beta);
        dh_by_dz = (0.5 * deficit + psi_u) / (0.5 * (deficit + e->gw));
        kavg = AvgKv(soil, deficit, e->gw, satkfunc);
        rechg = kavg * dh_by_dz;
        rechg = (rechg > 0.0 && e->unsat <= 0.0) ? 0.0 : rechg;
        rechg = (rechg < 0.0 && e->gw <= 0.0) ? 0.0 : rechg;
    }
    return rechg;
}

/* VerticalFlow, src/vert_flow.c:3-31 */
static void VerticalFlow(oracle_model *m)
{
    int i;
#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < m->nelem; i++) {
        m->elem[i].infil = Infil(&m->elem[i], m->stepsize, m->noah);
        /* frozen top soil, src/vert_flow.c:16-19 */
        if (m->noah) m->elem[i].infil *= m->elem[i].fcr;
        m->elem[i].rechg = Recharge(&m->elem[i]);
    }
}

/* GwTransp, noah/lsm_func.c:163-185: the fraction of transpiration drawn
 * from the saturated zone */
static double GwTransp(double ett, const double *et, int nwtbl, int nroot)
{
    int j;
    double gw_transp = 0.0;
    if (ett > 0.0) {
        if (nwtbl <= nroot) {
            for (j = (nwtbl <= 0 ? 0 : nwtbl - 1); j < nroot; j++) gw_transp += et[j];
            gw_transp = gw_transp / ett;
            gw_transp = (gw_transp > 1.0) ? 1.0 : gw_transp;
            gw_transp = (gw_transp < 0.0) ? 0.0 : gw_transp;
        }
    }
    return gw_transp;
}

/* EtExtract, src/hydrol.c:33-97, with its _NOAH_ branches (:43-55, :79-83) */
static void EtExtract(oracle_model *m)
{
    int i;
#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < m->nelem; i++) {
        elem_t *e = &m->elem[i];
        if (m->noah) {
            if (e->gw > e->soil.depth - e->soil.dinf) {
                e->edir_surf = 0.0;
                e->edir_unsat = 0.0;
                e->edir_gw = e->edir;
            } else {
                e->edir_surf = 0.0;
                e->edir_unsat = e->edir;
                e->edir_gw = 0.0;
            }
            e->gwet = GwTransp(e->ett, e->et, e->nwtbl, e->nroot);
            e->ett_unsat = (1.0 - e->gwet) * e->ett;
            e->ett_gw = e->gwet * e->ett;
            continue;
        }
        if (e->surfh >= DEPRSTG) {
            e->edir_surf = e->edir;
            e->edir_unsat = 0.0;
            e->edir_gw = 0.0;
        } else if (e->gw > e->soil.depth - e->soil.dinf) {
            e->edir_surf = 0.0;
            e->edir_unsat = 0.0;
            e->edir_gw = e->edir;
        } else {
            e->edir_surf = 0.0;
            e->edir_unsat = e->edir;
            e->edir_gw = 0.0;
        }
        if (e->gw > e->soil.depth - e->rzd) {
            e->ett_unsat = 0.0;
            e->ett_gw = e->ett;
        } else {
            e->ett_unsat = e->ett;
            e->ett_gw = 0.0;
        }
    }
}

/* ------------------------------------------------------------------ */
/* River                                                              */
/* ------------------------------------------------------------------ */

/* RiverCroSectArea, src/river_flow.c:520-548 */
static double RiverCroSectArea(int order, double depth, double coeff)
{
    double cs_area = 0.0;
    depth = (depth > 0.0) ? depth : 0.0;
    switch (order) {
    case RECTANGLE: cs_area = depth * coeff; break;
    case TRIANGLE: cs_area = depth * depth / coeff; break;
    case QUADRATIC:
        cs_area = 4.0 * depth * sqrt(depth) / (3.0 * sqrt(coeff));
        break;
    case CUBIC:
        cs_area = 3.0 * ppow(depth, 4.0 / 3.0) / (2.0 * ppow(coeff, 1.0 / 3.0));
        break;
    default: break;
    }
    return cs_area;
}

/* RiverPerim, src/river_flow.c:550-583 */
static double RiverPerim(int order, double depth, double coeff)
{
    double perim = 0.0;
    depth = (depth > 0.0) ? depth : 0.0;
    switch (order) {
    case RECTANGLE: perim = 2.0 * depth + coeff; break;
    case TRIANGLE:
        perim = 2.0 * depth * sqrt(1.0 + coeff * coeff) / coeff;
        break;
    case QUADRATIC:
        perim = sqrt(depth * (1.0 + 4.0 * coeff * depth) / coeff) +
            plog(2.0 * sqrt(coeff * depth) + sqrt(1.0 + 4.0 * coeff * depth)) /
            (2.0 * coeff);
        break;
    case CUBIC:
        perim = 2.0 * ((ppow(depth * (1.0 + 9.0 * ppow(coeff, 2.0 / 3.0) *
                                      depth), 0.5) / 3.0) +
                       (plog(3.0 * ppow(coeff, 1.0 / 3.0) * sqrt(depth) +
                            ppow(1.0 + 9.0 * ppow(coeff, 2.0 / 3.0) * depth,
                                0.5)) /
                        (9.0 * ppow(coeff, 1.0 / 3.0))));
        break;
    default: break;
    }
    return perim;
}

/* ChanFlowRiverToRiver, src/river_flow.c:257-300 */
static double ChanFlowRiverToRiver(const river_t *r, const river_t *d,
                                   int riv_mode)
{
    double total_h, perim, total_h_down, perim_down, avg_perim, avg_rough,
        distance, diff_h, grad_h, avg_sf, crossa, crossa_down, avg_crossa,
        avg_h;
    total_h = r->stage + r->zbed;
    perim = RiverPerim(r->intrpl_ord, r->stage, r->coeff);
    total_h_down = d->stage + d->zbed;
    perim_down = RiverPerim(d->intrpl_ord, d->stage, d->coeff);
    avg_perim = (perim + perim_down) / 2.0;
    avg_rough = (r->rough + d->rough) / 2.0;
    distance = 0.5 * (r->length + d->length);
    diff_h = (riv_mode == KINEMATIC) ? (r->zbed - d->zbed) :
                                       (total_h - total_h_down);
    grad_h = diff_h / distance;
    avg_sf = (grad_h > 0.0) ? grad_h : RIVGRADMIN;
    crossa = RiverCroSectArea(r->intrpl_ord, r->stage, r->coeff);
    crossa_down = RiverCroSectArea(d->intrpl_ord, d->stage, d->coeff);
    avg_crossa = 0.5 * (crossa + crossa_down);
    avg_h = (avg_perim == 0.0) ? 0.0 : (avg_crossa / avg_perim);
    return OverLandFlow(avg_h, grad_h, avg_sf, crossa, avg_rough);
}

/* SubFlowRiverToRiver, src/river_flow.c:302-331 (_ARITH_) */
static double SubFlowRiverToRiver(const river_t *r, double effk,
                                  const river_t *d, double effk_nabr)
{
    double total_h, total_h_down, avg_wid, diff_h, avg_h, distance, grad_h,
        avg_ksat;
    total_h = r->gw + r->zmin;
    total_h_down = d->gw + d->zmin;
    avg_wid = (r->width + d->width) / 2.0;
    diff_h = total_h - total_h_down;
    avg_h = AvgH(diff_h, r->gw, d->gw);
    distance = 0.5 * (r->length + d->length);
    grad_h = diff_h / distance;
    avg_ksat = 0.5 * (effk + effk_nabr);
    return avg_ksat * grad_h * avg_h * avg_wid;
}

/* OutletFlux, src/river_flow.c:333-390 */
static double OutletFlux(const river_t *r)
{
    double total_h, total_h_down, distance, grad_h, avg_h, avg_perim, crossa;
    double discharge = 0.0;
    switch (r->down) {
    case DIRICHLET:
        total_h = r->stage + r->zbed;
        total_h_down = r->bc;
        distance = 0.5 * r->length;
        grad_h = (total_h - total_h_down) / distance;
        avg_h = AvgH(grad_h, r->stage,
                     ((r->bc - (r->node_zmax - r->depth) > 0.0) ?
                          r->bc - (r->node_zmax - r->depth) : 0.0));
        avg_perim = RiverPerim(r->intrpl_ord, r->stage, r->coeff);
        crossa = RiverCroSectArea(r->intrpl_ord, r->stage, r->coeff);
        avg_h = (avg_perim == 0.0) ? 0.0 : (crossa / avg_perim);
        discharge = OverLandFlow(avg_h, grad_h, grad_h, crossa, r->rough);
        break;
    case NEUMANN:
        discharge = -r->bc;
        break;
    case ZERO_DPTH_GRAD:
        distance = 0.5 * r->length;
        grad_h = (r->zbed - (r->node_zmax - r->depth)) / distance;
        avg_h = r->stage;
        avg_perim = RiverPerim(r->intrpl_ord, r->stage, r->coeff);
        crossa = RiverCroSectArea(r->intrpl_ord, r->stage, r->coeff);
        discharge = sqrt(grad_h) * crossa *
            ((avg_perim > 0.0) ? ppow(crossa / avg_perim, 2.0 / 3.0) : 0.0) /
            r->rough;
        (void)avg_h;
        break;
    case CRIT_DPTH:
        crossa = RiverCroSectArea(r->intrpl_ord, r->stage, r->coeff);
        discharge = crossa * sqrt(GRAV * r->stage);
        break;
    default: break;
    }
    return discharge;
}

/* BoundFluxRiver, src/river_flow.c:392-427 */
static double BoundFluxRiver(const river_t *r)
{
    double total_h, total_h_down, distance, grad_h, avg_h, avg_perim, crossa;
    double flux = 0.0;
    if (r->bc_type > 0) {
        total_h = r->stage + r->zbed;
        total_h_down = r->bc;
        distance = 0.5 * r->length;
        grad_h = (total_h - total_h_down) / distance;
        avg_h = AvgH(grad_h, r->stage,
                     ((r->bc - r->zbed > 0.0) ? (r->bc - r->zbed) : 0.0));
        avg_perim = RiverPerim(r->intrpl_ord, r->stage, r->coeff);
        crossa = RiverCroSectArea(r->intrpl_ord, r->stage, r->coeff);
        avg_h = (avg_perim == 0.0) ? 0.0 : (crossa / avg_perim);
        flux = OverLandFlow(avg_h, grad_h, grad_h, crossa, r->rough);
    } else if (r->bc_type < 0) {
        flux = -r->bc;
    }
    return flux;
}

/* OvlFlowElemToRiver, src/river_flow.c:185-255 */
static double OvlFlowElemToRiver(const elem_t *e, const river_t *r)
{
    double zbank, flux, elem_h, rivseg_h;
    zbank = (r->zmax > e->zmax) ? r->zmax : e->zmax;
    elem_h = e->zmax + e->surfh;
    rivseg_h = r->zbed + r->stage;
    if (rivseg_h > elem_h) {
        if (elem_h > zbank) {
            flux = r->cwr * 2.0 * sqrt(2.0 * GRAV) * r->length *
                sqrt(rivseg_h - elem_h) * (rivseg_h - zbank) / 3.0;
        } else {
            if (zbank < rivseg_h)
                flux = r->cwr * 2.0 * sqrt(2.0 * GRAV) * r->length *
                    sqrt(rivseg_h - zbank) * (rivseg_h - zbank) / 3.0;
            else
                flux = 0.0;
        }
    } else if (e->surfh > DEPRSTG) {
        if (rivseg_h > zbank) {
            flux = -r->cwr * 2.0 * sqrt(2.0 * GRAV) * r->length *
                sqrt(elem_h - rivseg_h) * (elem_h - zbank) / 3.0;
        } else {
            if (zbank < elem_h)
                flux = -r->cwr * 2.0 * sqrt(2.0 * GRAV) * r->length *
                    sqrt(elem_h - zbank) * (elem_h - zbank) / 3.0;
            else
                flux = 0.0;
        }
    } else {
        flux = 0.0;
    }
    return flux;
}

/* ChanFlowElemToRiver, src/river_flow.c:429-460 */
static double ChanFlowElemToRiver(const elem_t *e, double effk,
                                  const river_t *r, double distance)
{
    double diff_h, avg_h, grad_h, avg_ksat;
    diff_h = (r->stage + r->zbed) - (e->gw + e->zmin);
    if (e->zmin > r->zbed)
        avg_h = e->gw;
    else if (e->zmin + e->gw > r->zbed)
        avg_h = e->zmin + e->gw - r->zbed;
    else
        avg_h = 0.0;
    avg_h = AvgH(diff_h, r->stage, avg_h);
    grad_h = diff_h / distance;
    avg_ksat = 0.5 * (effk + r->ksath);
    return r->length * avg_ksat * grad_h * avg_h;
}

/* SubFlowElemToRiver, src/river_flow.c:462-498 (_ARITH_) */
static double SubFlowElemToRiver(const elem_t *e, double effk,
                                 const river_t *r, double effk_riv,
                                 double distance)
{
    double diff_h, avg_h, avg_ksat, grad_h;
    diff_h = (r->gw + r->zmin) - (e->gw + e->zmin);
    if (e->zmin > r->zbed)
        avg_h = 0.0;
    else if (e->zmin + e->gw > r->zbed)
        avg_h = r->zbed - e->zmin;
    else
        avg_h = e->gw;
    avg_h = AvgH(diff_h, r->gw, avg_h);
    avg_ksat = 0.5 * (effk + effk_riv);
    grad_h = diff_h / distance;
    return r->length * avg_ksat * grad_h * avg_h;
}

/* ChanLeak, src/river_flow.c:500-518 */
static double ChanLeak(const river_t *r)
{
    double diff_h, grad_h;
    if (r->zbed - (r->gw + r->zmin) > 0.0)
        diff_h = r->stage;
    else
        diff_h = r->stage + r->zbed - (r->gw + r->zmin);
    grad_h = diff_h / r->bedthick;
    return r->ksatv * r->width * r->length * grad_h;
}

/* RiverToElem, src/river_flow.c:113-183 */
static void RiverToElem(river_t *r, elem_t *left, elem_t *right)
{
    double effk_left, effk_right;
    int j;
    if (r->leftele > 0)
        r->rivflow[LEFT_SURF2CHANL] = OvlFlowElemToRiver(left, r);
    if (r->rightele > 0)
        r->rivflow[RIGHT_SURF2CHANL] = OvlFlowElemToRiver(right, r);
    effk_left = EffKh(&left->soil, left->gw);
    effk_right = EffKh(&right->soil, right->gw);
    if (r->leftele > 0)
        r->rivflow[LEFT_AQUIF2CHANL] =
            ChanFlowElemToRiver(left, effk_left, r, r->dist_left);
    if (r->rightele > 0)
        r->rivflow[RIGHT_AQUIF2CHANL] =
            ChanFlowElemToRiver(right, effk_right, r, r->dist_right);
    if (r->leftele > 0)
        r->rivflow[LEFT_AQUIF2AQUIF] = SubFlowElemToRiver(
            left, effk_left, r, 0.5 * (effk_left + effk_right), r->dist_left);
    if (r->rightele > 0)
        r->rivflow[RIGHT_AQUIF2AQUIF] = SubFlowElemToRiver(
            right, effk_right, r, 0.5 * (effk_left + effk_right),
            r->dist_right);
    for (j = 0; j < NUM_EDGE; j++) {
        if (left->nabr[j] == -r->ind) {
            left->ovlflow[j] = -r->rivflow[LEFT_SURF2CHANL];
            left->subsurf[j] = -(r->rivflow[LEFT_AQUIF2CHANL] +
                                 r->rivflow[LEFT_AQUIF2AQUIF]);
            break;
        }
    }
    for (j = 0; j < NUM_EDGE; j++) {
        if (right->nabr[j] == -r->ind) {
            right->ovlflow[j] = -r->rivflow[RIGHT_SURF2CHANL];
            right->subsurf[j] = -(r->rivflow[RIGHT_AQUIF2CHANL] +
                                  r->rivflow[RIGHT_AQUIF2AQUIF]);
            break;
        }
    }
}

/* RiverFlow, src/river_flow.c:3-111 */
static void RiverFlow(oracle_model *m)
{
    int i;
    elem_t *elem = m->elem;
    river_t *river = m->river;
#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < m->nriver; i++) {
        river_t *down;
        elem_t *left, *right;
        double effk_nabr, effk;
        if (river[i].down > 0) {
            if (river[i].bc_type != 0)
                river[i].rivflow[UP_CHANL2CHANL] += BoundFluxRiver(&river[i]);
            down = &river[river[i].down - 1];
            river[i].rivflow[DOWN_CHANL2CHANL] =
                ChanFlowRiverToRiver(&river[i], down, m->riv_mode);
            left = &elem[river[i].leftele - 1];
            right = &elem[river[i].rightele - 1];
            effk = 0.5 * (EffKh(&left->soil, left->gw) +
                          EffKh(&right->soil, right->gw));
            left = &elem[down->leftele - 1];
            right = &elem[down->rightele - 1];
            effk_nabr = 0.5 * (EffKh(&left->soil, left->gw) +
                               EffKh(&right->soil, right->gw));
            river[i].rivflow[DOWN_AQUIF2AQUIF] =
                SubFlowRiverToRiver(&river[i], effk, down, effk_nabr);
        } else {
            river[i].rivflow[DOWN_CHANL2CHANL] = OutletFlux(&river[i]);
            river[i].rivflow[DOWN_AQUIF2AQUIF] = 0.0;
        }
        left = &elem[river[i].leftele - 1];
        right = &elem[river[i].rightele - 1];
        RiverToElem(&river[i], left, right);
        river[i].rivflow[CHANL_LKG] = ChanLeak(&river[i]);
    }
    for (i = 0; i < m->nriver; i++) {
        if (river[i].down > 0) {
            river_t *down = &river[river[i].down - 1];
            down->rivflow[UP_CHANL2CHANL] -= river[i].rivflow[DOWN_CHANL2CHANL];
            down->rivflow[UP_AQUIF2AQUIF] -= river[i].rivflow[DOWN_AQUIF2AQUIF];
        }
    }
}

/* ------------------------------------------------------------------ */
/* ODE, src/ode.c:4-399 (no _FBR_/_BGC_/_CYCLES_)                     */
/* ------------------------------------------------------------------ */
int oracle_rhs(oracle_model *m, double t, const double *y, double *dy)
{
    int i;
    const int nelem = m->nelem, nriver = m->nriver;
    const int size = 3 * nelem + 2 * nriver;
    int nan_found = 0;
    (void)t;

    g_ulp_perturb = m->ulp_perturb;
    for (i = 0; i < size; i++) dy[i] = 0.0;

#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < nelem; i++) {
        elem_t *e = &m->elem[i];
        e->surf = (y[i] >= 0.0) ? y[i] : 0.0;
        e->unsat = (y[i + nelem] >= 0.0) ? y[i + nelem] : 0.0;
        e->gw = (y[i + 2 * nelem] >= 0.0) ? y[i + 2 * nelem] : 0.0;
    }
#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < nriver; i++) {
        river_t *r = &m->river[i];
        r->stage = (y[i + 3 * nelem] >= 0.0) ? y[i + 3 * nelem] : 0.0;
        r->gw = (y[i + 3 * nelem + nriver] >= 0.0) ?
            y[i + 3 * nelem + nriver] : 0.0;
        r->rivflow[UP_CHANL2CHANL] = 0.0;
        r->rivflow[UP_AQUIF2AQUIF] = 0.0;
    }

    /* Hydrol, src/hydrol.c:3-30 */
#if defined(_OPENMP)
#pragma omp parallel for
#endif
    for (i = 0; i < nelem; i++) m->elem[i].surfh = SurfH(m->elem[i].surf);
    EtExtract(m);
    LateralFlow(m);
    VerticalFlow(m);
    RiverFlow(m);

#if defined(_OPENMP)
#pragma omp parallel for reduction(| : nan_found)
#endif
    for (i = 0; i < nelem; i++) {
        int j;
        const elem_t *e = &m->elem[i];
        dy[i] += e->pcpdrp - e->infil - e->edir_surf;
        dy[i + nelem] += e->infil - e->rechg - e->edir_unsat - e->ett_unsat;
        dy[i + 2 * nelem] += e->rechg - e->edir_gw - e->ett_gw;
        for (j = 0; j < NUM_EDGE; j++) {
            dy[i] -= e->ovlflow[j] / e->area;
            dy[i + 2 * nelem] -= e->subsurf[j] / e->area;
        }
        dy[i + nelem] /= e->soil.porosity;
        dy[i + 2 * nelem] /= e->soil.porosity;
        if (isnan(dy[i]) || isnan(dy[i + nelem]) || isnan(dy[i + 2 * nelem]))
            nan_found = 1;
    }
#if defined(_OPENMP)
#pragma omp parallel for reduction(| : nan_found)
#endif
    for (i = 0; i < nriver; i++) {
        int j;
        const river_t *r = &m->river[i];
        const int s = i + 3 * nelem, g = i + 3 * nelem + nriver;
        for (j = 0; j <= 6; j++) dy[s] -= r->rivflow[j] / r->area;
        dy[g] += -r->rivflow[LEFT_AQUIF2AQUIF] - r->rivflow[RIGHT_AQUIF2AQUIF] -
            r->rivflow[DOWN_AQUIF2AQUIF] - r->rivflow[UP_AQUIF2AQUIF] +
            r->rivflow[CHANL_LKG];
        dy[g] /= r->porosity * r->area;
        if (isnan(dy[s]) || isnan(dy[g])) nan_found = 1;
    }
    return nan_found ? -3 : 0;
}

void oracle_get_fluxes(const oracle_model *m, double *ovlflow, double *subsurf,
                       double *infil, double *rechg, double *et_split,
                       double *rivflow)
{
    int i, j;
    for (i = 0; i < m->nelem; i++) {
        const elem_t *e = &m->elem[i];
        for (j = 0; j < NUM_EDGE; j++) {
            if (ovlflow) ovlflow[3 * i + j] = e->ovlflow[j];
            if (subsurf) subsurf[3 * i + j] = e->subsurf[j];
        }
        if (infil) infil[i] = e->infil;
        if (rechg) rechg[i] = e->rechg;
        if (et_split) {
            et_split[5 * i + 0] = e->edir_surf;
            et_split[5 * i + 1] = e->edir_unsat;
            et_split[5 * i + 2] = e->edir_gw;
            et_split[5 * i + 3] = e->ett_unsat;
            et_split[5 * i + 4] = e->ett_gw;
        }
    }
    if (rivflow)
        for (i = 0; i < m->nriver; i++)
            for (j = 0; j < NUM_RIVFLX; j++)
                rivflow[NUM_RIVFLX * i + j] = m->river[i].rivflow[j];
}

/* Summary, src/update.c:3-99: ws <- y, ws0 <- ws.  Only ws0.surf feeds the
 * next right-hand side (Infil's cap, src/vert_flow.c:122). */
void oracle_post_step(oracle_model *m, const double *y)
{
    int i;
    for (i = 0; i < m->nelem; i++) m->elem[i].ws0_surf = y[i];
}

/* CVRhsFn over SUNDIALS serial N_Vectors (content: length, own_data, data;
 * cvode/include/nvector/nvector_serial.h:69-73), user_data = oracle_model:
 * lets an integrator call the restatement the way CVODE calls ODE(). */
struct serial_content_prefix {
    long int length;
    int own_data;
    double *data;
};
struct nvector_prefix {
    void *content;
    void *ops;
};

int oracle_cvrhs(double t, void *y, void *ydot, void *user_data)
{
    const double *yd =
        ((struct serial_content_prefix *)((struct nvector_prefix *)y)->content)->data;
    double *dd =
        ((struct serial_content_prefix *)((struct nvector_prefix *)ydot)->content)->data;
    return oracle_rhs((oracle_model *)user_data, t, yd, dd) == 0 ? 0 : -1;
}
