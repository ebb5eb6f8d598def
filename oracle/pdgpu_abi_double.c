/* pdgpu_abi_double.c — a CPU test double of the part of the C ABI
 * (include/pdgpu.h) that PD's side of the boundary (pd_gb300/pd_plugin/ff_gpu.h)
 * calls, backed by the FP64 oracle (pdoracle.c).
 *
 * TEST INFRASTRUCTURE ONLY.  It lets the PD-side C++ components run inside PD
 * on a machine without a GPU (oracle/Makefile plugin-check), so that their
 * marshalling — what they gather from the WorkSpace, the parameters they set,
 * how they add energies and forces back — is checked against PD's own
 * components on the same WorkSpace.  It is never linked into libpdgpu or the
 * product.  With PDGPU_DOUBLE_RECORD=<file> set it also writes every context's
 * description, parameters, last positions and each compute call's result
 * (tests/golden/make_plugin_golden.py turns that into the fixture the GPU
 * replay test feeds to the real library).
 *
 * Record container: per array [u32 name length][name][dtype 'd' | 'i'][u32 ndim]
 * [u64 dims...][little-endian data] (the layout tests/golden/refbin.py reads).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/pdgpu.h"
#include "pdoracle.h"

struct pdgpu_ctx {
    int id, n, nexcl;
    double box[3];
    double *charge, *radius, *epsilon, *mass, *gbR, *gbV, *gbT, *lR, *lP, *lS, *pos;
    int *lU, *excl;
    int has_gb, has_sa, nb_set, gb_set, gb_fast, vac_set;
    pdgpu_nb_params nb, vac;
    pdgpu_gb_params gb;
    pdgpu_list_params lp;
    int ncalls;
    double *last_sasa;
};

static int g_next_id = 0;
static FILE *g_rec = NULL;

static FILE *rec(void) {
    static int opened = 0;
    if (!opened) {
        const char *p = getenv("PDGPU_DOUBLE_RECORD");
        opened = 1;
        if (p && *p) g_rec = fopen(p, "wb");
    }
    return g_rec;
}

static void put(const char *name, char dt, const void *data, int ndim, const unsigned long long *dims) {
    FILE *f = rec();
    if (!f) return;
    unsigned nl = (unsigned)strlen(name), nd = (unsigned)ndim;
    unsigned long long count = 1;
    for (int k = 0; k < ndim; k++) count *= dims[k];
    fwrite(&nl, 4, 1, f);
    fwrite(name, 1, nl, f);
    fwrite(&dt, 1, 1, f);
    fwrite(&nd, 4, 1, f);
    fwrite(dims, 8, (size_t)ndim, f);
    fwrite(data, dt == 'd' ? 8 : 4, (size_t)count, f);
    fflush(f);
}

static void putd(const pdgpu_ctx *c, const char *what, const double *x, unsigned long long n, unsigned long long m) {
    char name[128];
    snprintf(name, sizeof name, "ctx%d_%s", c->id, what);
    unsigned long long dims[2] = {n, m};
    if (x) put(name, 'd', x, m > 1 ? 2 : 1, dims);
}

static void puti(const pdgpu_ctx *c, const char *what, const int *x, unsigned long long n, unsigned long long m) {
    char name[128];
    snprintf(name, sizeof name, "ctx%d_%s", c->id, what);
    unsigned long long dims[2] = {n, m};
    if (x) put(name, 'i', x, m > 1 ? 2 : 1, dims);
}

static double *dup_d(const double *x, size_t n) {
    if (!x) return NULL;
    double *y = (double *)malloc(n * sizeof(double));
    memcpy(y, x, n * sizeof(double));
    return y;
}

static int *dup_i(const int *x, size_t n) {
    if (!x) return NULL;
    int *y = (int *)malloc(n * sizeof(int));
    memcpy(y, x, n * sizeof(int));
    return y;
}

const char *pdgpu_error_string(int status) {
    return status == PDGPU_OK ? "ok" : "pdgpu test double: error";
}

pdgpu_ctx *pdgpu_create(int device, const pdgpu_system_desc *d, int *status) {
    (void)device;
    if (!d || d->nsystems != 1 || !d->natoms || !d->charge || !d->radius || !d->epsilon) {
        if (status) *status = PDGPU_ERR_ARG;
        return NULL;
    }
    pdgpu_ctx *c = (pdgpu_ctx *)calloc(1, sizeof(pdgpu_ctx));
    const size_t n = (size_t)d->natoms[0];
    c->id = g_next_id++;
    c->n = (int)n;
    memcpy(c->box, d->box, sizeof c->box);
    c->charge = dup_d(d->charge, n);
    c->radius = dup_d(d->radius, n);
    c->epsilon = dup_d(d->epsilon, n);
    c->mass = dup_d(d->mass, n);
    c->has_gb = d->gb_radius && d->gb_vj && d->gb_terms123;
    c->gbR = dup_d(d->gb_radius, n);
    c->gbV = dup_d(d->gb_vj, n);
    c->gbT = dup_d(d->gb_terms123, n);
    c->has_sa = d->lcpo_radius && d->lcpo_p && d->lcpo_sigma && d->lcpo_use;
    c->lR = dup_d(d->lcpo_radius, n);
    c->lP = dup_d(d->lcpo_p, 4 * n);
    c->lS = dup_d(d->lcpo_sigma, n);
    c->lU = dup_i(d->lcpo_use, n);
    c->nexcl = d->nexcl;
    c->excl = dup_i(d->excl, 3 * (size_t)d->nexcl);
    c->pos = (double *)calloc(3 * n, sizeof(double));
    c->gb_fast = 1;
    c->last_sasa = (double *)calloc(n, sizeof(double));
    putd(c, "box", c->box, 3, 1);
    putd(c, "charge", c->charge, n, 1);
    putd(c, "radius", c->radius, n, 1);
    putd(c, "epsilon", c->epsilon, n, 1);
    putd(c, "mass", c->mass, n, 1);
    putd(c, "gb_radius", c->gbR, n, 1);
    putd(c, "gb_vj", c->gbV, n, 1);
    putd(c, "gb_terms123", c->gbT, n, 1);
    putd(c, "lcpo_radius", c->lR, n, 1);
    putd(c, "lcpo_p", c->lP, n, 4);
    putd(c, "lcpo_sigma", c->lS, n, 1);
    puti(c, "lcpo_use", c->lU, n, 1);
    if (c->nexcl > 0) puti(c, "excl", c->excl, (unsigned long long)c->nexcl, 3);
    if (status) *status = PDGPU_OK;
    return c;
}

int pdgpu_destroy(pdgpu_ctx *c) {
    if (!c) return PDGPU_ERR_ARG;
    double **p[] = {&c->charge, &c->radius, &c->epsilon, &c->mass, &c->gbR, &c->gbV, &c->gbT,
                    &c->lR, &c->lP, &c->lS, &c->pos, &c->last_sasa};
    for (size_t k = 0; k < sizeof p / sizeof p[0]; k++) free(*p[k]);
    free(c->lU);
    free(c->excl);
    free(c);
    return PDGPU_OK;
}

static void put_nb(const pdgpu_ctx *c, const char *what, const pdgpu_nb_params *p) {
    double v[11] = {p->Cutoff, p->InnerCutoff, p->VdwCutoff, p->VdwInnerCutoff, p->Vdw14Scaling, p->Elec14Scaling,
                    p->Dielectric, p->EnergySwitch, p->ForceSwitch, p->DoVdw, p->DoElec};
    putd(c, what, v, 11, 1);
}

int pdgpu_set_nb_params(pdgpu_ctx *c, const pdgpu_nb_params *p) {
    if (!c || !p) return PDGPU_ERR_ARG;
    c->nb = *p;
    c->nb_set = 1;
    put_nb(c, "nb_params", p);
    return PDGPU_OK;
}

int pdgpu_set_gb_params(pdgpu_ctx *c, const pdgpu_gb_params *p) {
    if (!c || !p) return PDGPU_ERR_ARG;
    c->gb = *p;
    c->gb_set = 1;
    double v[13] = {p->Cutoff, p->InnerCutoff, p->VdwCutoff, p->VdwInnerCutoff, p->Vdw14Scaling, p->Elec14Scaling,
                    p->DielectricSolute, p->DielectricSolvent, p->GbsaStillCutoff, p->ExpApproxThreshold,
                    p->BornRadiusOffset, p->P4, p->P5};
    putd(c, "gb_params", v, 13, 1);
    return PDGPU_OK;
}

int pdgpu_set_gb_mode(pdgpu_ctx *c, int fast_mode, const pdgpu_nb_params *vacuum) {
    if (!c) return PDGPU_ERR_ARG;
    c->gb_fast = fast_mode;
    c->vac_set = vacuum != NULL;
    if (vacuum) {
        c->vac = *vacuum;
        put_nb(c, "gb_vacuum", vacuum);
    }
    double m = fast_mode;
    putd(c, "gb_fast", &m, 1, 1);
    return PDGPU_OK;
}

int pdgpu_set_list_params(pdgpu_ctx *c, const pdgpu_list_params *p) {
    if (!c || !p) return PDGPU_ERR_ARG;
    c->lp = *p;
    double v[2] = {p->Padding, p->check_skin};
    putd(c, "list_params", v, 2, 1);
    return PDGPU_OK;
}

int pdgpu_set_positions(pdgpu_ctx *c, const double *xyz, size_t stride) {
    if (!c || !xyz || stride < 24 || stride % 8) return PDGPU_ERR_ARG;
    for (int i = 0; i < c->n; i++)
        for (int k = 0; k < 3; k++) c->pos[3 * i + k] = xyz[i * (stride / 8) + k];
    putd(c, "pos", c->pos, (unsigned long long)c->n, 3);
    return PDGPU_OK;
}

static double list_radius(const pdgpu_ctx *c) {
    double r = 0;
    if (c->nb_set) r = fmax(r, fmax(c->nb.Cutoff, c->nb.VdwCutoff));
    if (c->gb_set) r = fmax(r, fmax(c->gb.Cutoff, c->gb.VdwCutoff));
    if (c->has_sa) r = fmax(r, 7.0);
    return r + c->lp.Padding;
}

static pdo_nb_params nb_of(const pdgpu_ctx *c, const pdgpu_nb_params *p) {
    pdo_nb_params q;
    memset(&q, 0, sizeof q);
    q.Cutoff = p->Cutoff;
    q.InnerCutoff = p->InnerCutoff;
    q.VdwCutoff = p->VdwCutoff;
    q.VdwInnerCutoff = p->VdwInnerCutoff;
    q.Vdw14Scaling = p->Vdw14Scaling;
    q.Elec14Scaling = p->Elec14Scaling;
    q.Dielectric = p->Dielectric;
    q.EnergySwitch = p->EnergySwitch;
    q.ForceSwitch = p->ForceSwitch;
    q.DoVdw = p->DoVdw;
    q.DoElec = p->DoElec;
    q.ListCutoff = list_radius(c);
    return q;
}

/* the GB object's own FF_NonBonded settings: as set, else its cutoffs with
 * Dielectric 1 and the energy switch (the library's rule, pdgpu.h) */
static pdgpu_nb_params vacuum_of(const pdgpu_ctx *c) {
    if (c->vac_set) return c->vac;
    pdgpu_nb_params p;
    memset(&p, 0, sizeof p);
    p.Cutoff = c->gb.Cutoff;
    p.InnerCutoff = c->gb.InnerCutoff;
    p.VdwCutoff = c->gb.VdwCutoff;
    p.VdwInnerCutoff = c->gb.VdwInnerCutoff;
    p.Vdw14Scaling = c->gb.Vdw14Scaling;
    p.Elec14Scaling = c->gb.Elec14Scaling;
    p.Dielectric = 1.0;
    p.EnergySwitch = 1;
    p.DoVdw = p.DoElec = 1;
    return p;
}

int pdgpu_compute(pdgpu_ctx *c, unsigned what, pdgpu_energies *out, double *f, size_t stride) {
    if (!c || (f && (stride < 24 || stride % 8))) return PDGPU_ERR_ARG;
    const int n = c->n;
    pdo_system s;
    s.natom = n;
    s.pos = c->pos;
    s.charge = c->charge;
    s.radius = c->radius;
    s.epsilon = c->epsilon;
    s.nexcl = c->nexcl;
    s.excl = c->excl;
    memcpy(s.box, c->box, sizeof s.box);
    double *force = (double *)calloc(3 * (size_t)n, sizeof(double));
    pdgpu_energies e;
    memset(&e, 0, sizeof e);
    pdo_energies o;
    if (what & PDGPU_NB) {
        if (!c->nb_set) return PDGPU_ERR_STATE;
        pdo_nb_params p = nb_of(c, &c->nb);
        pdo_nonbonded(&s, &p, 1, &o, force);
        e.vdw += o.vdw;
        e.elec += o.elec;
        e.virial += o.virial;
    }
    if (what & PDGPU_GB) {
        if (!c->has_gb || !c->gb_set) return PDGPU_ERR_STATE;
        pdo_gb_params g;
        memset(&g, 0, sizeof g);
        g.Cutoff = c->gb.Cutoff;
        g.InnerCutoff = c->gb.InnerCutoff;
        g.VdwCutoff = c->gb.VdwCutoff;
        g.VdwInnerCutoff = c->gb.VdwInnerCutoff;
        g.Vdw14Scaling = c->gb.Vdw14Scaling;
        g.Elec14Scaling = c->gb.Elec14Scaling;
        g.DielectricSolute = c->gb.DielectricSolute;
        g.DielectricSolvent = c->gb.DielectricSolvent;
        g.GbsaStillCutoff = c->gb.GbsaStillCutoff;
        g.ExpApproxThreshold = c->gb.ExpApproxThreshold;
        g.BornRadiusOffset = c->gb.BornRadiusOffset;
        g.P4 = c->gb.P4;
        g.P5 = c->gb.P5;
        g.ListCutoff = list_radius(c);
        const int pd_energies = (what & PDGPU_PD_ENERGIES) != 0;
        g.FastMode = (c->gb_fast && !pd_energies) ? 1 : 0;
        if (pd_energies) g.ExpApproxThreshold = -1e300;  /* calcBornEnergy has no threshold */
        pdo_gb_forces(&s, &g, c->gbR, c->gbV, c->gbT, 1, &o, force, NULL);
        e.vdw += o.vdw;
        e.elec += o.elec;
        e.pol += o.pol;
        e.pol_self += o.pol_self;
        e.pol_cross += o.pol_cross;
        if (!g.FastMode) {   /* the vacuum part from the GB object's FF_NonBonded settings */
            pdgpu_nb_params vp = vacuum_of(c);
            pdo_nb_params p = nb_of(c, &vp);
            pdo_nonbonded(&s, &p, 1, &o, force);
            e.vdw += o.vdw;
            e.elec += o.elec;
        }
    }
    if (what & PDGPU_SA) {
        if (!c->has_sa) return PDGPU_ERR_STATE;
        pdo_lcpo_forces(&s, list_radius(c), c->lR, c->lP, c->lS, c->lU, 1, &o, force, c->last_sasa);
        e.surf += o.surf;
    }
    e.epot = e.vdw + e.elec + e.pol + e.surf;
    if (f)
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) f[i * (stride / 8) + k] += force[3 * i + k];
    if (out) *out = e;
    char name[64];
    double w = (double)what;
    snprintf(name, sizeof name, "call%d_what", c->ncalls);
    putd(c, name, &w, 1, 1);
    snprintf(name, sizeof name, "call%d_ene", c->ncalls);
    putd(c, name, &e.epot, 12, 1);
    snprintf(name, sizeof name, "call%d_f", c->ncalls);
    putd(c, name, force, (unsigned long long)n, 3);
    c->ncalls++;
    free(force);
    return PDGPU_OK;
}

int pdgpu_get_sasa(pdgpu_ctx *c, double *sasa) {
    if (!c || !sasa) return PDGPU_ERR_ARG;
    memcpy(sasa, c->last_sasa, (size_t)c->n * sizeof(double));
    return PDGPU_OK;
}
