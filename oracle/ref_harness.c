/*
 * ref_harness.c -- drives the reference's own serial/OpenMP PIHM code, built
 * from its sources by oracle/Makefile (target `ref`) into oracle/_ref/.
 * Test infrastructure only: it exists to pin the CPU restatement
 * (pihm_oracle.c) and to produce golden vectors, never on a product path.
 *
 * It links every reference object except src/main.c, so it defines the
 * globals of src/main.c:10-24 and NumStateVar (src/main.c:313-339) itself.
 * Two ways in:
 *   - ref_build():        fill the reference's element/river records from the
 *                         structure-of-arrays mesh description used everywhere
 *                         else (include/pihm_gpu.h);
 *   - ref_load_example(): read a reference input deck with the reference's own
 *                         ReadAlloc/Initialize (src/read_alloc.c:3,
 *                         src/initialize.c:16), e.g. benchmark/input/example.
 * Then ref_ode() calls the reference ODE() (src/ode.c:4) directly, and
 * ref_run() steps the model the way src/main.c:217-254 and src/pihm.c:7-187 do.
 */
#include "pihm.h"
#include "pihm_gpu.h"
#if defined(_NOAH_)
#include "pihm_noah.h"
#endif

#include <unistd.h>

/* globals of src/main.c:10-24 */
int verbose_mode;
int debug_mode;
int append_mode;
int corr_mode;
int spinup_mode;
int tecplot;
char project[MAXSTRING];
int nelem;
int nriver;
#if defined(_OPENMP)
int nthreads = 1;
#endif

int NumStateVar(void) { return 3 * nelem + 2 * nriver; }

static pihm_struct g_pihm = NULL;
static int g_have_tables = 0; /* 1 when loaded through ReadAlloc */

int ref_num_threads(void)
{
#if defined(_OPENMP)
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void ref_set_num_threads(int n)
{
#if defined(_OPENMP)
    if (n > 0) {
        omp_set_num_threads(n);
        nthreads = n;
    }
#else
    (void)n;
#endif
}

static void free_model(void)
{
    if (g_pihm) {
        free(g_pihm->elem);
        free(g_pihm->river);
        free(g_pihm);
        g_pihm = NULL;
    }
}

int ref_build(const pihm_gpu_mesh *g, int surf_mode, int riv_mode,
              int stepsize)
{
    int i, j;
    free_model();
    g_pihm = (pihm_struct)calloc(1, sizeof(*g_pihm));
    nelem = g->nelem;
    nriver = g->nriver;
    g_pihm->elem = (elem_struct *)calloc(nelem, sizeof(elem_struct));
    g_pihm->river = (river_struct *)calloc(nriver > 0 ? nriver : 1,
                                           sizeof(river_struct));
    g_pihm->ctrl.surf_mode = surf_mode;
    g_pihm->ctrl.riv_mode = riv_mode;
    g_pihm->ctrl.stepsize = stepsize;
    g_have_tables = 0;
    for (i = 0; i < nelem; i++) {
        elem_struct *e = &g_pihm->elem[i];
        e->ind = i + 1;
        for (j = 0; j < NUM_EDGE; j++) {
            e->nabr[j] = g->nabr[3 * i + j];
            e->attrib.bc_type[j] = g->bc_type[3 * i + j];
            e->topo.edge[j] = g->edge[3 * i + j];
            e->topo.nabrdist[j] = g->nabrdist[3 * i + j];
            e->topo.nabr_x[j] = g->nabr_x[3 * i + j];
            e->topo.nabr_y[j] = g->nabr_y[3 * i + j];
        }
        e->topo.area = g->area[i];
        e->topo.zmin = g->zmin[i];
        e->topo.zmax = g->zmax[i];
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
        e->lc.rough = g->rough[i];
        e->ps.rzd = g->rzd[i];
    }
    for (i = 0; i < nriver; i++) {
        river_struct *r = &g_pihm->river[i];
        r->ind = i + 1;
        r->down = g->down[i];
        r->leftele = g->leftele[i];
        r->rightele = g->rightele[i];
        r->shp.intrpl_ord = g->intrpl_ord[i];
        r->attrib.riverbc_type = g->riverbc_type[i];
        r->topo.area = g->riv_area[i];
        r->topo.zmin = g->riv_zmin[i];
        r->topo.zmax = g->riv_zmax[i];
        r->topo.zbed = g->riv_zbed[i];
        r->topo.node_zmax = g->riv_node_zmax[i];
        r->topo.dist_left = g->riv_dist_left[i];
        r->topo.dist_right = g->riv_dist_right[i];
        r->shp.depth = g->riv_depth[i];
        r->shp.coeff = g->riv_coeff[i];
        r->shp.length = g->riv_length[i];
        r->shp.width = g->riv_width[i];
        r->matl.rough = g->riv_rough[i];
        r->matl.cwr = g->riv_cwr[i];
        r->matl.ksath = g->riv_ksath[i];
        r->matl.ksatv = g->riv_ksatv[i];
        r->matl.bedthick = g->riv_bedthick[i];
        r->matl.porosity = g->riv_porosity[i];
    }
    return 0;
}

#if !defined(_NOAH_)
/* Read an input deck `<workdir>/input/<proj>/<proj>.*` with the reference's
 * readers and initialise it (RelaxIc or ReadIc per the .para file). */
int ref_load_example(const char *workdir, const char *proj, double *y0,
                     int ny0)
{
    char cwd[4096];
    N_Vector cv_y;
    free_model();
    if (!getcwd(cwd, sizeof(cwd))) return -1;
    if (chdir(workdir) != 0) return -1;
    strncpy(project, proj, MAXSTRING - 1);
    verbose_mode = VL_SILENT;
    g_pihm = (pihm_struct)calloc(1, sizeof(*g_pihm));
    ReadAlloc(g_pihm);
    cv_y = N_VNew(NumStateVar());
    Initialize(g_pihm, cv_y);
    if (y0 && ny0 >= NumStateVar())
        memcpy(y0, NV_DATA(cv_y), sizeof(double) * NumStateVar());
    N_VDestroy(cv_y);
    g_have_tables = 1;
    if (chdir(cwd) != 0) return -1;
    return 0;
}

#endif /* !_NOAH_ */

#if !defined(_NOAH_)
/* Read a restart file with the reference's own ReadIc (src/read_ic.c:3) into
 * the model built by ref_build, and return what it stored: y in reference
 * order from ic.surf/unsat/gw and river ic.stage/gw, and ic.cmc, ic.sneqv. */
int ref_read_ic(const char *path, double *y, double *cmc, double *sneqv)
{
    int i;
    if (!g_pihm) return -1;
    ReadIc(path, g_pihm->elem, g_pihm->river);
    for (i = 0; i < nelem; i++) {
        y[i] = g_pihm->elem[i].ic.surf;
        y[nelem + i] = g_pihm->elem[i].ic.unsat;
        y[2 * nelem + i] = g_pihm->elem[i].ic.gw;
        cmc[i] = g_pihm->elem[i].ic.cmc;
        sneqv[i] = g_pihm->elem[i].ic.sneqv;
    }
    for (i = 0; i < nriver; i++) {
        y[3 * nelem + i] = g_pihm->river[i].ic.stage;
        y[3 * nelem + nriver + i] = g_pihm->river[i].ic.gw;
    }
    return 0;
}
#endif

int ref_sizes(int *ne, int *nr, int *stepsize, int *surf_mode, int *riv_mode)
{
    if (!g_pihm) return -1;
    if (ne) *ne = nelem;
    if (nr) *nr = nriver;
    if (stepsize) *stepsize = g_pihm->ctrl.stepsize;
    if (surf_mode) *surf_mode = g_pihm->ctrl.surf_mode;
    if (riv_mode) *riv_mode = g_pihm->ctrl.riv_mode;
    return 0;
}

/* Copy one field of the loaded model out (by name) so that the same
 * watershed can be handed to the GPU library and to the restatement. */
int ref_export_double(const char *name, double *out)
{
    int i, j;
    if (!g_pihm) return -1;
#define EF(nm, expr)                                                       \
    if (strcmp(name, nm) == 0) {                                           \
        for (i = 0; i < nelem; i++) out[i] = g_pihm->elem[i].expr;         \
        return 0;                                                          \
    }
#define EF3(nm, expr)                                                      \
    if (strcmp(name, nm) == 0) {                                           \
        for (i = 0; i < nelem; i++)                                        \
            for (j = 0; j < NUM_EDGE; j++)                                 \
                out[3 * i + j] = g_pihm->elem[i].expr[j];                  \
        return 0;                                                          \
    }
#define RF(nm, expr)                                                       \
    if (strcmp(name, nm) == 0) {                                           \
        for (i = 0; i < nriver; i++) out[i] = g_pihm->river[i].expr;       \
        return 0;                                                          \
    }
    EF("area", topo.area) EF("x", topo.x) EF("y", topo.y)
    EF("zmin", topo.zmin) EF("zmax", topo.zmax)
    EF3("edge", topo.edge) EF3("nabrdist", topo.nabrdist)
    EF3("nabr_x", topo.nabr_x) EF3("nabr_y", topo.nabr_y)
    EF("depth", soil.depth) EF("ksath", soil.ksath) EF("ksatv", soil.ksatv)
    EF("kinfv", soil.kinfv) EF("dinf", soil.dinf) EF("alpha", soil.alpha)
    EF("beta", soil.beta) EF("porosity", soil.porosity) EF("dmac", soil.dmac)
    EF("kmach", soil.kmach) EF("kmacv", soil.kmacv)
    EF("areafv", soil.areafv) EF("areafh", soil.areafh)
    EF("rough", lc.rough) EF("rzd", ps.rzd)
    EF("pcpdrp", wf.pcpdrp) EF("edir", wf.edir) EF("ett", wf.ett)
    EF("ws0_surf", ws0.surf) EF3("bc", bc.head)
    EF3("ovlflow", wf.ovlflow) EF3("subsurf", wf.subsurf)
    EF("infil", wf.infil) EF("rechg", wf.rechg)
    /* land-surface model: parameters Initialize leaves and the step's
       state and fluxes (src/init_soil.c, src/init_lc.c, src/init_forc.c,
       src/is_sm_et.c) */
    EF("cmc", ws.cmc) EF("sneqv", ws.sneqv) EF("prcp", wf.prcp) EF("ec", wf.ec)
    EF("drip", wf.drip) EF("albedomin", lc.albedomin) EF("albedomax", lc.albedomax)
    EF("shdfac", lc.shdfac) EF("cmcfactr", lc.cmcfactr) EF("cfactr", lc.cfactr)
    EF("rgl", epc.rgl) EF("rsmin", epc.rsmin) EF("rsmax", epc.rsmax) EF("topt", epc.topt)
    EF("smcmin", soil.smcmin) EF("smcwlt", soil.smcwlt) EF("smcref", soil.smcref)
    EF("zlvl_wind", ps.zlvl_wind) EF("sfctmp", es.sfctmp) EF("proj_lai", ps.proj_lai)
    EF("unsat", ws.unsat) EF("gw", ws.gw) EF("surf", ws.surf)
    RF("riv_area", topo.area) RF("riv_zmin", topo.zmin)
    RF("riv_zmax", topo.zmax) RF("riv_zbed", topo.zbed)
    RF("riv_node_zmax", topo.node_zmax) RF("riv_dist_left", topo.dist_left)
    RF("riv_dist_right", topo.dist_right) RF("riv_depth", shp.depth)
    RF("riv_coeff", shp.coeff) RF("riv_length", shp.length)
    RF("riv_width", shp.width) RF("riv_rough", matl.rough)
    RF("riv_cwr", matl.cwr) RF("riv_ksath", matl.ksath)
    RF("riv_ksatv", matl.ksatv) RF("riv_bedthick", matl.bedthick)
    RF("riv_porosity", matl.porosity) RF("river_bc", bc.head)
#undef EF
#undef EF3
#undef RF
    return -2;
}

int ref_export_int(const char *name, int *out)
{
    int i, j;
    if (!g_pihm) return -1;
    if (strcmp(name, "nabr") == 0) {
        for (i = 0; i < nelem; i++)
            for (j = 0; j < NUM_EDGE; j++) out[3 * i + j] = g_pihm->elem[i].nabr[j];
        return 0;
    }
    if (strcmp(name, "lc_type") == 0 || strcmp(name, "meteo_type") == 0 || strcmp(name, "lai_type") == 0) {
        for (i = 0; i < nelem; i++)
            out[i] = name[1] == 'c' ? g_pihm->elem[i].attrib.lc_type
                     : name[1] == 'e' ? g_pihm->elem[i].attrib.meteo_type
                                      : g_pihm->elem[i].attrib.lai_type;
        return 0;
    }
    if (strcmp(name, "bc_type") == 0) {
        for (i = 0; i < nelem; i++)
            for (j = 0; j < NUM_EDGE; j++)
                out[3 * i + j] = g_pihm->elem[i].attrib.bc_type[j];
        return 0;
    }
#define RI(nm, expr)                                                       \
    if (strcmp(name, nm) == 0) {                                           \
        for (i = 0; i < nriver; i++) out[i] = g_pihm->river[i].expr;       \
        return 0;                                                          \
    }
    RI("down", down) RI("leftele", leftele) RI("rightele", rightele)
    RI("intrpl_ord", shp.intrpl_ord) RI("riverbc_type", attrib.riverbc_type)
#undef RI
    return -2;
}

void ref_set_forcing(const double *pcpdrp, const double *edir,
                     const double *ett)
{
    int i;
    for (i = 0; i < nelem; i++) {
        if (pcpdrp) g_pihm->elem[i].wf.pcpdrp = pcpdrp[i];
        if (edir) g_pihm->elem[i].wf.edir = edir[i];
        if (ett) g_pihm->elem[i].wf.ett = ett[i];
    }
}

void ref_set_bc(const double *elem_bc, const double *river_bc)
{
    int i, j;
    if (elem_bc)
        for (i = 0; i < nelem; i++)
            for (j = 0; j < NUM_EDGE; j++)
                g_pihm->elem[i].bc.head[j] = elem_bc[3 * i + j];
    if (river_bc)
        for (i = 0; i < nriver; i++) g_pihm->river[i].bc.head = river_bc[i];
}

void ref_set_ws0_surf(const double *ws0_surf)
{
    int i;
    for (i = 0; i < nelem; i++) g_pihm->elem[i].ws0.surf = ws0_surf[i];
}

void ref_set_river_edge_ovlflow(const double *ovl)
{
    int i, j;
    for (i = 0; i < nelem; i++)
        for (j = 0; j < NUM_EDGE; j++)
            if (g_pihm->elem[i].nabr[j] < 0)
                g_pihm->elem[i].wf.ovlflow[j] = ovl[3 * i + j];
}

/* One call of the reference right-hand side. */
int ref_ode(double t, const double *y, double *ydot)
{
    int n = NumStateVar();
    N_Vector vy = N_VMake_Serial(n, (realtype *)y);
    N_Vector vd = N_VMake_Serial(n, ydot);
    int rc = ODE(t, vy, vd, g_pihm);
    N_VDestroy(vy);
    N_VDestroy(vd);
    return rc;
}

void ref_get_fluxes(double *ovlflow, double *subsurf, double *infil,
                    double *rechg, double *et_split, double *rivflow)
{
    int i, j;
    for (i = 0; i < nelem; i++) {
        const elem_struct *e = &g_pihm->elem[i];
        for (j = 0; j < NUM_EDGE; j++) {
            if (ovlflow) ovlflow[3 * i + j] = e->wf.ovlflow[j];
            if (subsurf) subsurf[3 * i + j] = e->wf.subsurf[j];
        }
        if (infil) infil[i] = e->wf.infil;
        if (rechg) rechg[i] = e->wf.rechg;
        if (et_split) {
            et_split[5 * i + 0] = e->wf.edir_surf;
            et_split[5 * i + 1] = e->wf.edir_unsat;
            et_split[5 * i + 2] = e->wf.edir_gw;
            et_split[5 * i + 3] = e->wf.ett_unsat;
            et_split[5 * i + 4] = e->wf.ett_gw;
        }
    }
    if (rivflow)
        for (i = 0; i < nriver; i++)
            for (j = 0; j < NUM_RIVFLX; j++)
                rivflow[NUM_RIVFLX * i + j] = g_pihm->river[i].wf.rivflow[j];
}

#if defined(_NOAH_)
/* Flux-PIHM (_NOAH_) inputs of the right-hand side, which Noah computes once
 * per model step: per-layer transpiration wf.et[0..nlayers) (GwTransp,
 * noah/lsm_func.c:163-185, splits ett with them), the water-table layer
 * ps.nwtbl and root layers ps.nroot, the top-layer unfrozen moisture
 * ws.sh2o[0] with soil.smcmin/smcmax (Infil's saturation,
 * src/vert_flow.c:94-98) and the frozen-soil factor ps.fcr
 * (src/vert_flow.c:16-19). */
int ref_set_noah(const double *et, int nlayers, const int *nwtbl, const int *nroot, const double *sh2o0,
                 const double *smcmin, const double *smcmax, const double *fcr)
{
    int i, j;
    if (!g_pihm || nlayers < 0 || nlayers > MAXLYR) return -1;
    for (i = 0; i < nelem; i++) {
        elem_struct *e = &g_pihm->elem[i];
        for (j = 0; j < MAXLYR; j++) e->wf.et[j] = (j < nlayers) ? et[(size_t)nlayers * i + j] : 0.0;
        e->ps.nwtbl = nwtbl[i];
        e->ps.nroot = nroot[i];
        e->ws.sh2o[0] = sh2o0[i];
        e->soil.smcmin = smcmin[i];
        e->soil.smcmax = smcmax[i];
        e->ps.fcr = fcr[i];
    }
    return 0;
}

/* gwet of the last evaluation (EtExtract stores it in ps.gwet). */
void ref_get_gwet(double *gwet)
{
    int i;
    for (i = 0; i < nelem; i++) gwet[i] = g_pihm->elem[i].ps.gwet;
}

/* ---- The Noah land-surface model (src/noah/noah.c, lsm_func.c) ---------
 * The same parameter, state and forcing structs the GPU library takes
 * (include/pihm_noah.h) fill the element records of the model built by
 * ref_build; Noah(), Summary() and NoahHydrol() are the reference's own. */
#define FILL_LAYERS(dst, src, i, n)                                          \
    do {                                                                      \
        int k_;                                                               \
        for (k_ = 0; k_ < MAXLYR; k_++)                                       \
            (dst)[k_] = (k_ < (n)) ? (src)[(size_t)MAXLYR * (i) + k_] : BADVAL; \
    } while (0)

int ref_noah_load(const pihm_noah_params *p, const pihm_noah_state *s, const double *y0)
{
    int i, k;
    if (!g_pihm || p->nelem != nelem) return -1;
    for (i = 0; i < nelem; i++) {
        elem_struct *e = &g_pihm->elem[i];
        const int ns = p->nsoil[i];
        e->ps.nsoil = ns;
        e->ps.nroot = p->nroot[i];
        FILL_LAYERS(e->ps.sldpth, p->sldpth, i, ns);
        FILL_LAYERS(e->ps.rtdis, p->rtdis, i, p->nroot[i]);
        /* DefSldpth's depths below the surface, noah/lsm_func.c:152-156 */
        e->ps.zsoil[0] = -e->ps.sldpth[0];
        for (k = 1; k < ns; k++) e->ps.zsoil[k] = -e->ps.sldpth[k] + e->ps.zsoil[k - 1];
        e->lc.isurban = p->isurban ? p->isurban[i] : 0;
        e->soil.smcmax = p->smcmax[i]; e->soil.smcmin = p->smcmin[i];
        e->soil.smcref = p->smcref[i]; e->soil.smcwlt = p->smcwlt[i];
        e->soil.smcdry = p->smcdry[i]; e->soil.quartz = p->quartz[i];
        e->soil.csoil = p->csoil[i]; e->soil.alpha = p->alpha[i];
        e->soil.beta = p->beta[i]; e->soil.ksatv = p->ksatv[i];
        e->soil.porosity = p->porosity[i]; e->soil.depth = p->depth[i];
        e->topo.area = p->area[i];
        e->lc.shdfac = p->shdfac[i]; e->lc.cmcfactr = p->cmcfactr[i];
        e->lc.laimax = p->laimax[i]; e->lc.laimin = p->laimin[i];
        e->lc.emissmax = p->emissmax[i]; e->lc.emissmin = p->emissmin[i];
        e->lc.albedomax = p->albedomax[i]; e->lc.albedomin = p->albedomin[i];
        e->lc.z0max = p->z0max[i]; e->lc.z0min = p->z0min[i];
        e->lc.snup = p->snup[i]; e->lc.cfactr = p->cfactr[i];
        e->epc.rgl = p->rgl[i]; e->epc.rsmin = p->rsmin[i];
        e->epc.rsmax = p->rsmax[i]; e->epc.topt = p->topt[i]; e->epc.hs = p->hs[i];
        e->ps.sbeta = p->sbeta[i]; e->ps.salp = p->salp[i]; e->ps.frzx = p->frzx[i];
        e->ps.fxexp = p->fxexp[i]; e->ps.czil = p->czil[i]; e->ps.lvcoef = p->lvcoef[i];
        e->ps.zbot = p->zbot[i]; e->ps.tbot = p->tbot[i]; e->ps.zlvl = p->zlvl[i];
        e->ps.zlvl_wind = p->zlvl_wind[i]; e->ps.snoalb = p->snoalb[i];
        FILL_LAYERS(e->ws.smc, s->smc, i, ns);
        FILL_LAYERS(e->ws.sh2o, s->sh2o, i, ns);
        FILL_LAYERS(e->es.stc, s->stc, i, ns);
        e->es.t1 = s->t1[i]; e->ws.cmc = s->cmc[i]; e->ws.sneqv = s->sneqv[i];
        e->ps.snowh = s->snowh[i]; e->ps.sndens = s->sndens[i]; e->ps.ch = s->ch[i];
        e->ps.cm = s->cm[i]; e->ps.snotime1 = s->snotime1[i]; e->ps.albedo = s->albedo[i];
        e->ps.emissi = s->emissi[i]; e->ps.q1 = s->q1[i]; e->ps.ribb = s->ribb[i];
        e->ps.fcr = s->fcr[i];
        e->ps.nwtbl = ns;
        for (k = 0; k < MAXLYR; k++) {
            e->wf.et[k] = 0.0;
            e->wf.runoff2_lyr[k] = 0.0;
            e->wf.smflxv[k] = 0.0;
            e->ps.satdpth[k] = 0.0;
        }
        e->wf.edir = 0.0; e->wf.ett = 0.0; e->wf.ec = 0.0; e->wf.pcpdrp = 0.0;
        e->wf.runoff2 = 0.0; e->wf.runoff3 = 0.0; e->wf.infil = 0.0;
        /* the previous model step's state, for MassBalance */
        e->ws.surf = y0[i]; e->ws.unsat = y0[nelem + i]; e->ws.gw = y0[2 * nelem + i];
        e->ws0 = e->ws;
    }
    return 0;
}

int ref_noah_forcing(const pihm_noah_forcing *f)
{
    int i;
    if (!g_pihm) return -1;
    for (i = 0; i < nelem; i++) {
        elem_struct *e = &g_pihm->elem[i];
        e->wf.prcp = f->prcp[i]; e->es.sfctmp = f->sfctmp[i]; e->ps.rh = f->rh[i];
        e->ps.sfcspd = f->sfcspd[i]; e->ef.soldn = f->soldn[i];
        e->ef.longwave = f->longwave[i]; e->ps.sfcprs = f->sfcprs[i];
        e->ps.proj_lai = f->lai[i];
    }
    return 0;
}

/* Noah() over dt (src/noah/noah.c:3-55) */
int ref_noah_step(double dt)
{
    if (!g_pihm) return -1;
    Noah(g_pihm->elem, dt);
    return 0;
}

/* After a model step ending at y: Summary() (src/update.c:3-99, with its
 * _NOAH_ part) and NoahHydrol() (src/noah/noah.c:57-160).  The fluxes
 * MassBalance reads are the last ref_ode() evaluation's. */
int ref_noah_post(const double *y, double dt)
{
    N_Vector v;
    if (!g_pihm) return -1;
    v = N_VMake_Serial(NumStateVar(), (realtype *)y);
    Summary(g_pihm->elem, g_pihm->river, v, dt);
    N_VDestroy(v);
    NoahHydrol(g_pihm->elem, dt);
    return 0;
}

/* A field of pihm_gpu_noah_get's list (include/pihm_noah.h), reference
 * order; per-layer fields [nelem][MAXLYR] */
int ref_noah_get(int field, double *out)
{
    int i, k;
    if (!g_pihm) return -1;
    for (i = 0; i < nelem; i++) {
        const elem_struct *e = &g_pihm->elem[i];
        const double *lay = NULL;
        double v = 0.0;
        switch (field) {
        case PIHM_NOAH_SMC: lay = e->ws.smc; break;
        case PIHM_NOAH_SH2O: lay = e->ws.sh2o; break;
        case PIHM_NOAH_STC: lay = e->es.stc; break;
        case PIHM_NOAH_ET: lay = e->wf.et; break;
        case PIHM_NOAH_RUNOFF2_LYR: lay = e->wf.runoff2_lyr; break;
        case PIHM_NOAH_SMFLXV: lay = e->wf.smflxv; break;
        case PIHM_NOAH_T1: v = e->es.t1; break;
        case PIHM_NOAH_CMC: v = e->ws.cmc; break;
        case PIHM_NOAH_SNEQV: v = e->ws.sneqv; break;
        case PIHM_NOAH_SNOWH: v = e->ps.snowh; break;
        case PIHM_NOAH_SNDENS: v = e->ps.sndens; break;
        case PIHM_NOAH_CH: v = e->ps.ch; break;
        case PIHM_NOAH_CM: v = e->ps.cm; break;
        case PIHM_NOAH_ALBEDO: v = e->ps.albedo; break;
        case PIHM_NOAH_EMISSI: v = e->ps.emissi; break;
        case PIHM_NOAH_Q1: v = e->ps.q1; break;
        case PIHM_NOAH_FCR: v = e->ps.fcr; break;
        case PIHM_NOAH_EDIR: v = e->wf.edir; break;
        case PIHM_NOAH_EC: v = e->wf.ec; break;
        case PIHM_NOAH_ETT: v = e->wf.ett; break;
        case PIHM_NOAH_ESNOW: v = e->wf.esnow; break;
        case PIHM_NOAH_ETP: v = e->wf.etp; break;
        case PIHM_NOAH_DRIP: v = e->wf.drip; break;
        case PIHM_NOAH_PCPDRP: v = e->wf.pcpdrp; break;
        case PIHM_NOAH_SNOMLT: v = e->wf.snomlt; break;
        case PIHM_NOAH_SSOIL: v = e->ef.ssoil; break;
        case PIHM_NOAH_SHEAT: v = e->ef.sheat; break;
        case PIHM_NOAH_RUNOFF2: v = e->wf.runoff2; break;
        case PIHM_NOAH_RUNOFF3: v = e->wf.runoff3; break;
        case PIHM_NOAH_INFIL: v = e->wf.infil; break;
        case PIHM_NOAH_NWTBL: v = e->ps.nwtbl; break;
        case PIHM_NOAH_SNOTIME1: v = e->ps.snotime1; break;
        case PIHM_NOAH_SNCOVR: v = e->ps.sncovr; break;
        case PIHM_NOAH_BETA: v = e->ps.beta; break;
        case PIHM_NOAH_ETA: v = e->wf.eta; break;
        case PIHM_NOAH_SOILM: v = e->ws.soilm; break;
        default: return -1;
        }
        if (lay) {
            for (k = 0; k < MAXLYR; k++) out[(size_t)MAXLYR * i + k] = (k < e->ps.nsoil) ? lay[k] : 0.0;
        } else {
            out[i] = v;
        }
    }
    return 0;
}
#else
/* Forcing step of src/pihm.c:21-66 for a model loaded by ref_load_example:
 * boundary conditions, meteorological forcing, interception/snow/ET, at model
 * time t (seconds since the epoch, as ctrl.tout). */
int ref_apply_forcing(int t)
{
    if (!g_pihm || !g_have_tables) return -1;
    ApplyBc(&g_pihm->forc, g_pihm->elem, g_pihm->river, t);
    ApplyForc(&g_pihm->forc, g_pihm->elem, t);
    IntcpSnowEt(t, (realtype)g_pihm->ctrl.etstep, g_pihm->elem, &g_pihm->cal);
    return 0;
}

/* The land-surface part of that step alone: ApplyForc and IntcpSnowEt
 * (src/pihm.c:30-66) at time t over `stepsize` seconds. */
int ref_land_step(int t, double stepsize)
{
    if (!g_pihm || !g_have_tables) return -1;
    ApplyForc(&g_pihm->forc, g_pihm->elem, t);
    IntcpSnowEt(t, (realtype)stepsize, g_pihm->elem, &g_pihm->cal);
    return 0;
}

/* Set the element state the land-surface step reads and carries (ws.unsat,
 * ws.gw, ws.cmc, ws.sneqv); a null array leaves that field. */
int ref_land_set_state(const double *unsat, const double *gw, const double *cmc, const double *sneqv)
{
    int i;
    if (!g_pihm) return -1;
    for (i = 0; i < nelem; i++) {
        if (unsat) g_pihm->elem[i].ws.unsat = unsat[i];
        if (gw) g_pihm->elem[i].ws.gw = gw[i];
        if (cmc) g_pihm->elem[i].ws.cmc = cmc[i];
        if (sneqv) g_pihm->elem[i].ws.sneqv = sneqv[i];
    }
    return 0;
}

/* MonthlyLai, MonthlyRl, MonthlyMf (src/forcing.c:532-798) at t for type lc */
void ref_monthly(int t, int lc, double *out3)
{
    out3[0] = MonthlyLai(t, lc);
    out3[1] = MonthlyRl(t, lc);
    out3[2] = MonthlyMf(t);
}

int ref_model_times(int *starttime, int *endtime, int *etstep, int *nstep)
{
    if (!g_pihm || !g_have_tables) return -1;
    *starttime = g_pihm->ctrl.starttime;
    *endtime = g_pihm->ctrl.endtime;
    *etstep = g_pihm->ctrl.etstep;
    *nstep = g_pihm->ctrl.nstep;
    return 0;
}

/* The reference's per-step loop (src/main.c:217-254, src/pihm.c:7-187) on a
 * model built by ref_build: every model step sets the element forcing
 * (uniform pcpdrp/edir/ett of that step, standing in for ApplyForc and
 * IntcpSnowEt), calls SolveCVode (src/ode.c:555), Summary (src/update.c:3)
 * and AdjCVodeMaxStep (src/ode.c:601).  Records the state every `every`
 * steps, the outlet segment's DOWN_CHANL2CHANL flux after every step (the
 * value PIHM prints as rivflx1) and CVODE's counters. */
/* Optional water-balance outputs of ref_run_pihm: a file for the reference's
   own PrintWaterBal and [nsteps][3] (src, snk, storage) at full precision. */
static FILE *g_wb_file = NULL;
static double *g_wb_out = NULL;

int ref_set_water_balance(const char *path, double *out)
{
    if (g_wb_file) fclose(g_wb_file);
    g_wb_file = path ? fopen(path, "w") : NULL;
    g_wb_out = out;
    return (path && !g_wb_file) ? -1 : 0;
}

int ref_close_water_balance(void)
{
    if (g_wb_file) fclose(g_wb_file);
    g_wb_file = NULL;
    g_wb_out = NULL;
    return 0;
}

int ref_run_pihm(double *y, int nsteps, int stepsize, double reltol, double abstol,
                 double initstep, double nncfn, double nnimax, double nnimin, double decr,
                 double incr, double stmin, const double *pcp, const double *edir,
                 const double *ett, int outlet, int every, double *y_out, double *q_out,
                 long *stats)
{
    int n = NumStateVar();
    int i, s;
    N_Vector cv_y = N_VMake_Serial(n, y);
    void *cvode_mem = CVodeCreate(CV_BDF, CV_NEWTON);
    pihm_struct p = g_pihm;
    p->ctrl.stepsize = stepsize;
    p->ctrl.reltol = reltol;
    p->ctrl.abstol = abstol;
    p->ctrl.initstep = initstep;
    p->ctrl.nncfn = nncfn;
    p->ctrl.nnimax = nnimax;
    p->ctrl.nnimin = nnimin;
    p->ctrl.decr = decr;
    p->ctrl.incr = incr;
    p->ctrl.stmin = stmin;
    /* InitVar: ws0 <- initial state (src/initialize.c:576-640) */
    for (i = 0; i < nelem; i++) {
        p->elem[i].ws0.surf = y[i];
        p->elem[i].ws0.unsat = y[i + nelem];
        p->elem[i].ws0.gw = y[i + 2 * nelem];
    }
    SetCVodeParam(p, cvode_mem, cv_y);
    for (s = 0; s < nsteps; s++) {
        int t = 0;
        double pc[1];
        for (i = 0; i < nelem; i++) {
            p->elem[i].wf.pcpdrp = pcp[s];
            p->elem[i].wf.edir = edir[s];
            p->elem[i].wf.ett = ett[s];
        }
        (void)pc;
        SolveCVode(0, &t, (s + 1) * stepsize, 0.0, cvode_mem, cv_y);
        Summary(p->elem, p->river, cv_y, (double)stepsize);
        AdjCVodeMaxStep(cvode_mem, &p->ctrl);
        if (q_out) q_out[s] = p->river[outlet].wf.rivflow[DOWN_CHANL2CHANL];
        if (g_wb_file || g_wb_out) {
            /* the watershed water balance of this step: the reference's own
               PrintWaterBal (src/print.c:337-542, printed with 6 digits) and
               its three sums at full precision, in its summation order */
            double src = 0.0, snk = 0.0, strg = 0.0;
            for (i = 0; i < nelem; i++) {
                p->elem[i].wf.prcp = pcp[s];  /* no interception: prcp = pcpdrp */
                p->elem[i].wf.ec = 0.0;
            }
            if (g_wb_file)
                PrintWaterBal(g_wb_file, (s + 1) * stepsize, 0, stepsize, p->elem, p->river);
            for (i = 0; i < nelem; i++) {
                const elem_struct *e = &p->elem[i];
                src += e->wf.prcp * e->topo.area * stepsize;
                snk += (e->wf.edir + e->wf.ett + e->wf.ec) * e->topo.area * stepsize;
                strg += (e->ws.cmc + e->ws.sneqv + e->ws.surf + (e->ws.unsat + e->ws.gw) * e->soil.porosity) *
                        e->topo.area;
            }
            for (i = 0; i < nriver; i++) {
                const river_struct *r = &p->river[i];
                strg += (r->ws.stage + r->ws.gw * r->matl.porosity) * r->topo.area;
                if (r->down < 0) snk += r->wf.rivflow[DOWN_CHANL2CHANL] * stepsize;
            }
            if (g_wb_out) {
                g_wb_out[3 * s] = src;
                g_wb_out[3 * s + 1] = snk;
                g_wb_out[3 * s + 2] = strg;
            }
        }
        if (y_out && every > 0 && (s + 1) % every == 0)
            memcpy(y_out + (size_t)((s + 1) / every - 1) * n, y, sizeof(double) * n);
    }
    if (stats) {
        long v;
        CVodeGetNumSteps(cvode_mem, &v); stats[0] = v;
        CVodeGetNumRhsEvals(cvode_mem, &v); stats[1] = v;
        CVodeGetNumNonlinSolvIters(cvode_mem, &v); stats[2] = v;
        CVodeGetNumNonlinSolvConvFails(cvode_mem, &v); stats[3] = v;
        CVodeGetNumErrTestFails(cvode_mem, &v); stats[4] = v;
        CVSpilsGetNumLinIters(cvode_mem, &v); stats[5] = v;
        CVSpilsGetNumRhsEvals(cvode_mem, &v); stats[6] = v;
    }
    CVodeFree(&cvode_mem);
    N_VDestroy(cv_y);
    return 0;
}

/* The reference's main loop on a deck loaded by ref_load_example, with its
 * own forcing: from the deck's START, every model step ApplyBc, every
 * LSM_STEP ApplyForc and IntcpSnowEt (src/pihm.c:15-66), then SolveCVode,
 * Summary, AdjCVodeMaxStep (src/pihm.c:86-99, src/main.c:217-254), with the
 * solver controls of the .para file.  y: the initial state (in, reference
 * order) and the final state (out).  Records the state every `every` steps,
 * the outlet segment's DOWN_CHANL2CHANL flux after every step, PrintWaterBal's
 * three sums at full precision after every step (wb_out [nsteps][3], may be
 * null) and CVODE's counters. */
int ref_run_deck(double *y, int nsteps, int outlet, int every, double *y_out, double *q_out, double *wb_out,
                 long *stats)
{
    int n = NumStateVar();
    int i, s;
    N_Vector cv_y;
    void *cvode_mem;
    pihm_struct p = g_pihm;
    if (!p || !g_have_tables) return -1;
    cv_y = N_VMake_Serial(n, y);
    cvode_mem = CVodeCreate(CV_BDF, CV_NEWTON);
    for (i = 0; i < nelem; i++) {
        p->elem[i].ws0.surf = y[i];
        p->elem[i].ws0.unsat = y[i + nelem];
        p->elem[i].ws0.gw = y[i + 2 * nelem];
        p->elem[i].ws.surf = y[i];
        p->elem[i].ws.unsat = y[i + nelem];
        p->elem[i].ws.gw = y[i + 2 * nelem];
    }
    SetCVodeParam(p, cvode_mem, cv_y);
    for (s = 0; s < nsteps; s++) {
        const int t = p->ctrl.starttime + s * p->ctrl.stepsize;
        int tret = t;
        ApplyBc(&p->forc, p->elem, p->river, t);
        if ((t - p->ctrl.starttime) % p->ctrl.etstep == 0) {
            ApplyForc(&p->forc, p->elem, t);
            IntcpSnowEt(t, (realtype)p->ctrl.etstep, p->elem, &p->cal);
        }
        SolveCVode(p->ctrl.starttime, &tret, t + p->ctrl.stepsize, 0.0, cvode_mem, cv_y);
        Summary(p->elem, p->river, cv_y, (realtype)p->ctrl.stepsize);
        AdjCVodeMaxStep(cvode_mem, &p->ctrl);
        if (q_out) q_out[s] = p->river[outlet].wf.rivflow[DOWN_CHANL2CHANL];
        if (wb_out) {
            /* PrintWaterBal's sums (src/print.c:337-542) in its order */
            double src = 0.0, snk = 0.0, strg = 0.0;
            const double dt = (double)p->ctrl.stepsize;
            for (i = 0; i < nelem; i++) {
                const elem_struct *e = &p->elem[i];
                src += e->wf.prcp * e->topo.area * dt;
                snk += (e->wf.edir + e->wf.ett + e->wf.ec) * e->topo.area * dt;
                strg += (e->ws.cmc + e->ws.sneqv + e->ws.surf + (e->ws.unsat + e->ws.gw) * e->soil.porosity) *
                        e->topo.area;
            }
            for (i = 0; i < nriver; i++) {
                const river_struct *r = &p->river[i];
                strg += (r->ws.stage + r->ws.gw * r->matl.porosity) * r->topo.area;
                if (r->down < 0) snk += r->wf.rivflow[DOWN_CHANL2CHANL] * dt;
            }
            wb_out[3 * s] = src;
            wb_out[3 * s + 1] = snk;
            wb_out[3 * s + 2] = strg;
        }
        if (y_out && every > 0 && (s + 1) % every == 0)
            memcpy(y_out + (size_t)((s + 1) / every - 1) * n, y, sizeof(double) * n);
    }
    if (stats) {
        long v;
        CVodeGetNumSteps(cvode_mem, &v); stats[0] = v;
        CVodeGetNumRhsEvals(cvode_mem, &v); stats[1] = v;
        CVodeGetNumNonlinSolvIters(cvode_mem, &v); stats[2] = v;
        CVodeGetNumNonlinSolvConvFails(cvode_mem, &v); stats[3] = v;
        CVodeGetNumErrTestFails(cvode_mem, &v); stats[4] = v;
        CVSpilsGetNumLinIters(cvode_mem, &v); stats[5] = v;
        CVSpilsGetNumRhsEvals(cvode_mem, &v); stats[6] = v;
    }
    CVodeFree(&cvode_mem);
    N_VDestroy(cv_y);
    return 0;
}
#endif /* _NOAH_ */
