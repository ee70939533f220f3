/*
 * Derived from SUNDIALS 2.7.0 (nvector_serial.c). Copyright (c) 2002-2016,
 * Lawrence Livermore National Security; produced at the Lawrence Livermore
 * National Laboratory. Redistributed under the SUNDIALS BSD-3 licence: its
 * full text, conditions and disclaimer are in pihm-cuda_gb300/NOTICE.SUNDIALS.
 *
 * nvector_host.c -- host N_Vector restating the SUNDIALS 2.7 serial N_Vector
 * (cvode/src/nvec_ser/nvector_serial.c:421-1060 of the reference tree):
 * the same case analysis in N_VLinearSum and N_VScale and left-to-right
 * sums, so its results equal the serial vector's bit for bit (checked against
 * tests/golden/nvector_calls.npz).  Test infrastructure only: it lets the
 * integrator of the GPU library (include/pihm_bdf.h) run on the CPU with the
 * right-hand-side restatement, to be compared with the reference's CVODE.
 *
 * Content layout matches the serial vector's (length, own_data, data), so
 * oracle_cvrhs can read it.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#include "pihm_nvector.h"

typedef struct {
    long int length;
    int own_data;
    double *data;
} host_content;

#define HC(v) ((host_content *)(v)->content)
#define HD(v) (HC(v)->data)
#define HL(v) (HC(v)->length)

static N_Vector_ID hv_id(N_Vector v) { (void)v; return SUNDIALS_NVEC_SERIAL; }
static N_Vector hv_clone_empty(N_Vector w);
static N_Vector hv_clone(N_Vector w);
static void hv_destroy(N_Vector v);

static void hv_space(N_Vector v, long int *lrw, long int *liw) { *lrw = HL(v); *liw = 1; }
static double *hv_getptr(N_Vector v) { return HD(v); }
static void hv_setptr(double *d, N_Vector v) { if (HL(v) > 0) HC(v)->data = d; }

static void hv_linearsum(double a, N_Vector x, double b, N_Vector y, N_Vector z)
{
    long i, n = HL(x);
    double *xd = HD(x), *yd = HD(y), *zd = HD(z);
    int test;
    if (b == 1.0 && z == y) {            /* y <- a x + y */
        if (a == 1.0) { for (i = 0; i < n; i++) yd[i] += xd[i]; return; }
        if (a == -1.0) { for (i = 0; i < n; i++) yd[i] -= xd[i]; return; }
        for (i = 0; i < n; i++) yd[i] += a * xd[i];
        return;
    }
    if (a == 1.0 && z == x) {            /* x <- b y + x */
        if (b == 1.0) { for (i = 0; i < n; i++) xd[i] += yd[i]; return; }
        if (b == -1.0) { for (i = 0; i < n; i++) xd[i] -= yd[i]; return; }
        for (i = 0; i < n; i++) xd[i] += b * yd[i];
        return;
    }
    if (a == 1.0 && b == 1.0) { for (i = 0; i < n; i++) zd[i] = xd[i] + yd[i]; return; }
    if ((test = (a == 1.0 && b == -1.0)) || (a == -1.0 && b == 1.0)) {
        double *v1 = test ? yd : xd, *v2 = test ? xd : yd;
        for (i = 0; i < n; i++) zd[i] = v2[i] - v1[i];
        return;
    }
    if ((test = (a == 1.0)) || (b == 1.0)) {
        double c = test ? b : a, *v1 = test ? yd : xd, *v2 = test ? xd : yd;
        for (i = 0; i < n; i++) zd[i] = (c * v1[i]) + v2[i];
        return;
    }
    if ((test = (a == -1.0)) || (b == -1.0)) {
        double c = test ? b : a, *v1 = test ? yd : xd, *v2 = test ? xd : yd;
        for (i = 0; i < n; i++) zd[i] = (c * v1[i]) - v2[i];
        return;
    }
    if (a == b) { for (i = 0; i < n; i++) zd[i] = a * (xd[i] + yd[i]); return; }
    if (a == -b) { for (i = 0; i < n; i++) zd[i] = a * (xd[i] - yd[i]); return; }
    for (i = 0; i < n; i++) zd[i] = (a * xd[i]) + (b * yd[i]);
}

static void hv_const(double c, N_Vector z) { long i; for (i = 0; i < HL(z); i++) HD(z)[i] = c; }
static void hv_prod(N_Vector x, N_Vector y, N_Vector z)
{ long i; for (i = 0; i < HL(x); i++) HD(z)[i] = HD(x)[i] * HD(y)[i]; }
static void hv_div(N_Vector x, N_Vector y, N_Vector z)
{ long i; for (i = 0; i < HL(x); i++) HD(z)[i] = HD(x)[i] / HD(y)[i]; }
static void hv_scale(double c, N_Vector x, N_Vector z)
{
    long i, n = HL(x);
    double *xd = HD(x), *zd = HD(z);
    if (z == x) { for (i = 0; i < n; i++) xd[i] *= c; return; }
    if (c == 1.0) { for (i = 0; i < n; i++) zd[i] = xd[i]; }
    else if (c == -1.0) { for (i = 0; i < n; i++) zd[i] = -xd[i]; }
    else { for (i = 0; i < n; i++) zd[i] = c * xd[i]; }
}
static void hv_abs(N_Vector x, N_Vector z) { long i; for (i = 0; i < HL(x); i++) HD(z)[i] = fabs(HD(x)[i]); }
static void hv_inv(N_Vector x, N_Vector z) { long i; for (i = 0; i < HL(x); i++) HD(z)[i] = 1.0 / HD(x)[i]; }
static void hv_addconst(N_Vector x, double b, N_Vector z)
{ long i; for (i = 0; i < HL(x); i++) HD(z)[i] = HD(x)[i] + b; }
static double hv_dot(N_Vector x, N_Vector y)
{ long i; double s = 0.0; for (i = 0; i < HL(x); i++) s += HD(x)[i] * HD(y)[i]; return s; }
static double hv_maxnorm(N_Vector x)
{ long i; double m = 0.0; for (i = 0; i < HL(x); i++) if (fabs(HD(x)[i]) > m) m = fabs(HD(x)[i]); return m; }
static double hv_wrms(N_Vector x, N_Vector w)
{
    long i; double s = 0.0, p;
    for (i = 0; i < HL(x); i++) { p = HD(x)[i] * HD(w)[i]; s += p * p; }
    return (s / HL(x) <= 0.0) ? 0.0 : sqrt(s / HL(x));
}
static double hv_wrmsmask(N_Vector x, N_Vector w, N_Vector id)
{
    long i; double s = 0.0, p;
    for (i = 0; i < HL(x); i++) if (HD(id)[i] > 0.0) { p = HD(x)[i] * HD(w)[i]; s += p * p; }
    return (s / HL(x) <= 0.0) ? 0.0 : sqrt(s / HL(x));
}
static double hv_min(N_Vector x)
{ long i; double m = HD(x)[0]; for (i = 1; i < HL(x); i++) if (HD(x)[i] < m) m = HD(x)[i]; return m; }
static double hv_wl2(N_Vector x, N_Vector w)
{
    long i; double s = 0.0, p;
    for (i = 0; i < HL(x); i++) { p = HD(x)[i] * HD(w)[i]; s += p * p; }
    return (s <= 0.0) ? 0.0 : sqrt(s);
}
static double hv_l1(N_Vector x)
{ long i; double s = 0.0; for (i = 0; i < HL(x); i++) s += fabs(HD(x)[i]); return s; }
static void hv_compare(double c, N_Vector x, N_Vector z)
{ long i; for (i = 0; i < HL(x); i++) HD(z)[i] = (fabs(HD(x)[i]) >= c) ? 1.0 : 0.0; }
static int hv_invtest(N_Vector x, N_Vector z)
{
    long i; int ok = 1;
    for (i = 0; i < HL(x); i++) { if (HD(x)[i] == 0.0) ok = 0; else HD(z)[i] = 1.0 / HD(x)[i]; }
    return ok;
}
static int hv_constrmask(N_Vector c, N_Vector x, N_Vector m)
{
    long i; int test = 1;
    double *cd = HD(c), *xd = HD(x), *md = HD(m);
    for (i = 0; i < HL(x); i++) {
        md[i] = 0.0;
        if (cd[i] == 0.0) continue;
        if (cd[i] > 1.5 || cd[i] < -1.5) {
            if (xd[i] * cd[i] <= 0.0) { test = 0; md[i] = 1.0; }
            continue;
        }
        if (cd[i] > 0.5 || cd[i] < -0.5)
            if (xd[i] * cd[i] < 0.0) { test = 0; md[i] = 1.0; }
    }
    return test;
}
static double hv_minquotient(N_Vector num, N_Vector den)
{
    long i; int none = 1; double m = DBL_MAX;
    for (i = 0; i < HL(num); i++) {
        if (HD(den)[i] == 0.0) continue;
        if (!none) { double q = HD(num)[i] / HD(den)[i]; if (q < m) m = q; }
        else { m = HD(num)[i] / HD(den)[i]; none = 0; }
    }
    return m;
}

static struct _generic_N_Vector_Ops *hv_ops(void)
{
    struct _generic_N_Vector_Ops *o = calloc(1, sizeof(*o));
    o->nvgetvectorid = hv_id;
    o->nvclone = hv_clone;
    o->nvcloneempty = hv_clone_empty;
    o->nvdestroy = hv_destroy;
    o->nvspace = hv_space;
    o->nvgetarraypointer = hv_getptr;
    o->nvsetarraypointer = hv_setptr;
    o->nvlinearsum = hv_linearsum;
    o->nvconst = hv_const;
    o->nvprod = hv_prod;
    o->nvdiv = hv_div;
    o->nvscale = hv_scale;
    o->nvabs = hv_abs;
    o->nvinv = hv_inv;
    o->nvaddconst = hv_addconst;
    o->nvdotprod = hv_dot;
    o->nvmaxnorm = hv_maxnorm;
    o->nvwrmsnorm = hv_wrms;
    o->nvwrmsnormmask = hv_wrmsmask;
    o->nvmin = hv_min;
    o->nvwl2norm = hv_wl2;
    o->nvl1norm = hv_l1;
    o->nvcompare = hv_compare;
    o->nvinvtest = hv_invtest;
    o->nvconstrmask = hv_constrmask;
    o->nvminquotient = hv_minquotient;
    return o;
}

static N_Vector hv_clone_empty(N_Vector w)
{
    N_Vector v = calloc(1, sizeof(*v));
    host_content *c = calloc(1, sizeof(*c));
    c->length = w ? HL(w) : 0;
    v->content = c;
    v->ops = hv_ops();
    return v;
}

static N_Vector hv_clone(N_Vector w)
{
    N_Vector v = hv_clone_empty(w);
    HC(v)->data = calloc((size_t)(HL(v) > 0 ? HL(v) : 1), sizeof(double));
    HC(v)->own_data = 1;
    return v;
}

static void hv_destroy(N_Vector v)
{
    if (!v) return;
    if (HC(v)->own_data) free(HD(v));
    free(v->content);
    free(v->ops);
    free(v);
}

/* Wrap caller memory (not freed by destroy). */
N_Vector oracle_nv_make(long int length, double *data)
{
    N_Vector v = hv_clone_empty(NULL);
    HC(v)->length = length;
    HC(v)->data = data;
    HC(v)->own_data = 0;
    return v;
}

void oracle_nv_destroy(N_Vector v) { hv_destroy(v); }
