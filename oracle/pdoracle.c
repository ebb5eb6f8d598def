/* pdoracle.c — FP64 CPU restatement of PD's nonbonded / GB / LCPO / integrator
 * arithmetic.  TEST INFRASTRUCTURE ONLY (checker + timed CPU baseline); the
 * product never links it.  Each function cites the PD file:line it restates
 * (paths inside the PD project).  Loop orders follow PD's (i ascending, list
 * entries in ascending j) so that sums agree with PD to rounding.
 */
#include "pdoracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SQR(x) ((x) * (x))
static const double PI_ = 3.14159265358979323846;

/* PhysicsConst, src/mmlib/forcefields/forcefield.cpp:35-55 */
double pdo_econv_joule(void) {
    const double four_pi_e0 = PI_ * 4.0 * PDO_E0;
    return (PDO_E_CHARGE * PDO_E_CHARGE) / (four_pi_e0 * PDO_ANGSTROM);
}
double pdo_halfeconv(void) {
    const double four_pi_e0 = PI_ * 4.0 * PDO_E0;
    double econv = ((1.0 / PDO_KCAL2J) * PDO_NA * PDO_E_CHARGE * PDO_E_CHARGE) / (four_pi_e0 * PDO_ANGSTROM);
    return econv * 0.5;
}

static int nthreads_eff(int n) {
#ifdef _OPENMP
    return n > 1 ? n : 1;
#else
    (void)n;
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* bond-order lookup: per atom a sorted partner table built from the          */
/* (i, j, bondorder) exclusion list.  Pairs not present have bond order 7,   */
/* which is what PD's list stores for them (neighbourlist.cpp:398-408).      */
/* ------------------------------------------------------------------------ */
typedef struct {
    int *start;  /* natom+1 */
    int *partner;
    int *order;
} bo_table;

static void bo_build(const pdo_system *s, bo_table *t) {
    int n = s->natom;
    t->start = (int *)calloc((size_t)n + 1, sizeof(int));
    t->partner = (int *)malloc(sizeof(int) * (size_t)(2 * s->nexcl + 1));
    t->order = (int *)malloc(sizeof(int) * (size_t)(2 * s->nexcl + 1));
    for (int k = 0; k < s->nexcl; k++) {
        t->start[s->excl[3 * k] + 1]++;
        t->start[s->excl[3 * k + 1] + 1]++;
    }
    for (int i = 0; i < n; i++) t->start[i + 1] += t->start[i];
    int *fill = (int *)calloc((size_t)n, sizeof(int));
    for (int k = 0; k < s->nexcl; k++) {
        int a = s->excl[3 * k], b = s->excl[3 * k + 1], o = s->excl[3 * k + 2];
        int pa = t->start[a] + fill[a]++;
        t->partner[pa] = b; t->order[pa] = o;
        int pb = t->start[b] + fill[b]++;
        t->partner[pb] = a; t->order[pb] = o;
    }
    free(fill);
}
static void bo_free(bo_table *t) { free(t->start); free(t->partner); free(t->order); }
static inline int bo_lookup(const bo_table *t, int i, int j) {
    int best = 7;
    for (int k = t->start[i]; k < t->start[i + 1]; k++)
        if (t->partner[k] == j && t->order[k] < best) best = t->order[k];
    return best;
}

/* minimum image by repeated shifts, as the periodic list build does
 * (neighbourlist.cpp:381-386); infinite space leaves d untouched */
static inline void min_image(const double *box, double *d) {
    for (int c = 0; c < 3; c++) {
        if (box[c] <= 0) continue;
        double h = 0.5 * box[c];
        while (d[c] > h) d[c] -= box[c];
        while (d[c] < -h) d[c] += box[c];
    }
}

/* ------------------------------------------------------------------------ */
/* neighbour list checksums (neighbourlist.cpp:247-333, 336-439)            */
/* ------------------------------------------------------------------------ */
int pdo_list_checksums(const pdo_system *s, double list_cutoff, int32_t *count, int64_t *sumj, int64_t *sumj2) {
    double lim = SQR(list_cutoff);
    for (int i = 0; i < s->natom; i++) {
        int c = 0;
        int64_t a = 0, b = 0;
        for (int j = 0; j < i; j++) {
            double d[3] = {s->pos[3 * j] - s->pos[3 * i], s->pos[3 * j + 1] - s->pos[3 * i + 1],
                           s->pos[3 * j + 2] - s->pos[3 * i + 2]};
            min_image(s->box, d);
            if (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] > lim) continue;
            c++; a += j; b += (int64_t)j * j;
        }
        count[i] = c; sumj[i] = a; sumj2[i] = b;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* LJ + Coulomb                                                              */
/* ------------------------------------------------------------------------ */
typedef struct {
    double sqrcutoff, sqrinner, invSwidth, vdwinvSwidth;
    double sA, sB, sC, sD, sE, fswitch_cutoffV, eshift;
    double invdielectric, econv;
    int elecmode; /* 0 none, 1 normal, 3 energy switch, 4 force switch */
    int dovdw;
} nb_consts;

/* constants and mode selection, nonbonded.cpp:591-637 and dispatch :1222-1246
 * (ForceSwitch wins over EnergySwitch; DDD Levitt mode is never selected) */
static void nb_setup(const pdo_nb_params *p, nb_consts *c) {
    double C = p->Cutoff, I = p->InnerCutoff;
    c->sqrcutoff = C * C;
    c->sqrinner = I * I;
    c->invSwidth = 1.0 / (C - I);
    c->vdwinvSwidth = 1.0 / (p->VdwCutoff - p->VdwInnerCutoff);
    double C2 = C * C, I2 = I * I;
    c->sA = 1.0 / ((C2 - I2) * (C2 - I2) * (C2 - I2));
    c->sB = -(C2 * C2 * C2 - 3.0 * C2 * C2 * I2);
    c->sC = 6.0 * C2 * I2;
    c->sD = -(C2 + I2);
    c->sE = 2.0 / 5.0;
    double innerV = c->sA * (c->sB * (1.0 / I) + c->sC * I + c->sD * I * I * I + c->sE * I * I * I * I * I);
    c->fswitch_cutoffV = c->sA * (c->sB * (1.0 / C) + c->sC * C + c->sD * C * C * C + c->sE * C * C * C * C * C);
    c->eshift = (I < C) ? 1.0 / I + (innerV - c->fswitch_cutoffV) : 0.0;
    c->invdielectric = 1.0 / p->Dielectric;
    c->econv = pdo_econv_joule();
    c->elecmode = 1;
    if (p->EnergySwitch) c->elecmode = 3;
    if (p->ForceSwitch) c->elecmode = 4;
    if (!p->DoElec) c->elecmode = 0;
    c->dovdw = p->DoVdw;
}

/* one listed pair, nonbonded.cpp:715-833; returns 0 when beyond Cutoff */
static inline int nb_pair(const pdo_nb_params *p, const nb_consts *c, double sqrdist, double ri, double rj,
                          double ei, double ej, double qi, double qj, double s_vdw, double s_elec,
                          double *evdw, double *eelec, double *fmag, double *dist_out) {
    if (sqrdist > c->sqrcutoff) return 0;
    double dist = sqrt(sqrdist);
    double invd = 1.0 / dist;
    double vpot = 0, vf = 0, epot = 0, ef = 0;
    if (c->dovdw && dist < p->VdwCutoff) {
        double radiusij = ri + rj;
        double eps = s_vdw * ei * ej;
        double B = SQR(radiusij * invd);
        B = B * B * B;
        double A = B * B;
        vpot = (2.0 * eps) * (0.5 * A - B);
        vf = -(12.0E10 * eps * invd) * (A - B);
        if (dist > p->VdwInnerCutoff) {
            double S = 1.0 - SQR(c->vdwinvSwidth * (dist - p->VdwInnerCutoff));
            double dSdd = -4.0E10 * SQR(c->vdwinvSwidth) * (dist - p->VdwInnerCutoff) * S;
            S = S * S;
            vf = S * vf + vpot * dSdd;
            vpot *= S;
        }
    }
    switch (c->elecmode) {
    case 1:
        epot = c->econv * c->invdielectric * s_elec * (qi * qj) * invd;
        ef = -epot * invd * 1E10;
        break;
    case 3:
        epot = c->econv * c->invdielectric * s_elec * (qi * qj) * invd;
        ef = -epot * invd * 1E10;
        if (dist > p->InnerCutoff) {
            double S = 1.0 - SQR(c->invSwidth * (dist - p->InnerCutoff));
            double dSdd = -4.0E10 * SQR(c->invSwidth) * (dist - p->InnerCutoff) * S;
            S = S * S;
            ef = S * ef + epot * dSdd;
            epot *= S;
        }
        break;
    case 4:
        epot = c->econv * c->invdielectric * s_elec * (qi * qj);
        if (dist > p->InnerCutoff) {
            ef = -1E10 * epot * c->sA * SQR(invd) * SQR(c->sqrcutoff - sqrdist) *
                 (c->sqrcutoff - 3.0 * c->sqrinner + 2.0 * sqrdist);
            epot *= -(c->sA * dist * (c->sB * SQR(invd) + c->sC + c->sD * sqrdist + c->sE * SQR(sqrdist)) -
                      c->fswitch_cutoffV);
        } else {
            ef = -1E10 * epot * SQR(invd);
            epot *= (invd - c->eshift);
        }
        break;
    default:
        break;
    }
    *evdw = vpot;
    *eelec = epot;
    *fmag = vf + ef;
    *dist_out = dist;
    return 1;
}

/* scalar pair law, nonbonded.cpp:400-534 (energy switch / force switch / none;
 * the DDD branch is not reproduced since the force path never selects it) */
void pdo_pair_law(const pdo_nb_params *p, double r, double radiusij, double epsilon, double qi, double qj,
                  double *vdw_pot, double *vdw_force, double *elec_pot, double *elec_force) {
    nb_consts c;
    nb_setup(p, &c);
    *vdw_pot = *vdw_force = *elec_pot = *elec_force = 0;
    double invd = 1.0 / r;
    if (r < p->VdwCutoff) {
        double B = SQR(radiusij * invd);
        B = B * B * B;
        double A = B * B;
        *vdw_pot = (2.0 * epsilon) * (0.5 * A - B);
        *vdw_force = -(12.0E10 * epsilon * invd) * (A - B);
        if (r > p->VdwInnerCutoff) {
            double S = 1.0 - SQR(c.vdwinvSwidth * (r - p->VdwInnerCutoff));
            double dSdd = -4.0E10 * SQR(c.vdwinvSwidth) * (r - p->VdwInnerCutoff) * S;
            S = S * S;
            *vdw_force = S * *vdw_force + *vdw_pot * dSdd;
            *vdw_pot *= S;
        }
    }
    if (r < p->Cutoff) {
        double ev = 0, ef = 0, dummyv = 0;
        pdo_nb_params q = *p;
        q.DoVdw = 0;
        q.DoElec = 1;
        nb_consts c2;
        nb_setup(&q, &c2);
        /* the scalar law's precedence is EnergySwitch first, then ForceSwitch */
        c2.elecmode = p->EnergySwitch ? 3 : (p->ForceSwitch ? 4 : 1);
        nb_pair(&q, &c2, r * r, 0, 0, 0, 0, qi, qj, 0, 1.0, &dummyv, &ev, &ef, &dummyv);
        *elec_pot = ev;
        *elec_force = ef;
    }
}

int pdo_nonbonded(const pdo_system *s, const pdo_nb_params *p, int nthreads, pdo_energies *e, double *force) {
    int n = s->natom;
    nb_consts c;
    nb_setup(p, &c);
    bo_table bt;
    bo_build(s, &bt);
    double tabV[8] = {0, 0, 0, p->Vdw14Scaling, 1, 1, 1, 1};
    double tabE[8] = {0, 0, 0, p->Elec14Scaling, 1, 1, 1, 1};
    double list2 = SQR(p->ListCutoff);
    int nt = nthreads_eff(nthreads);
    double *fbuf = (double *)calloc((size_t)nt * 3 * n, sizeof(double));
    double *ebuf = (double *)calloc((size_t)nt * 3, sizeof(double));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 32) num_threads(nt)
#endif
    for (int i = 0; i < n; i++) {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        double *f = fbuf + (size_t)tid * 3 * n;
        double *eb = ebuf + 3 * tid;
        double fi[3] = {0, 0, 0};
        for (int j = 0; j < i; j++) {
            double d[3] = {s->pos[3 * j] - s->pos[3 * i], s->pos[3 * j + 1] - s->pos[3 * i + 1],
                           s->pos[3 * j + 2] - s->pos[3 * i + 2]};
            min_image(s->box, d);
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (r2 > list2) continue; /* not in the list */
            int bo = bo_lookup(&bt, i, j);
            double ev, ee, fm, dist;
            if (!nb_pair(p, &c, r2, s->radius[i], s->radius[j], s->epsilon[i], s->epsilon[j], s->charge[i],
                         s->charge[j], tabV[bo], tabE[bo], &ev, &ee, &fm, &dist))
                continue;
            eb[0] += ev;
            eb[1] += ee;
            eb[2] += dist * fm * PDO_ANGSTROM;
            double sc = fm / dist;
            for (int k = 0; k < 3; k++) {
                fi[k] += d[k] * sc;
                f[3 * j + k] -= d[k] * sc;
            }
        }
        for (int k = 0; k < 3; k++) f[3 * i + k] += fi[k];
    }
    memset(e, 0, sizeof(*e));
    for (int t = 0; t < nt; t++) {
        e->vdw += ebuf[3 * t];
        e->elec += ebuf[3 * t + 1];
        e->virial += ebuf[3 * t + 2];
        for (int k = 0; k < 3 * n; k++) force[k] += fbuf[(size_t)t * 3 * n + k];
    }
    if (p->VdwCor) { /* nonbonded.cpp:862-874, one constant per atom */
        double v = -0.5 * p->VdwCorDensity * p->VdwCorEpsilon / ((1.0 / PDO_KCAL2J) * PDO_NA) * (8.0 / 3.0) * PI_ *
                   pow(p->VdwCorRadius, 6) / pow(p->VdwCorCutoff, 3);
        e->vdw += v * n;
    }
    e->epot = e->vdw + e->elec;
    free(fbuf);
    free(ebuf);
    bo_free(&bt);
    return 0;
}

/* stored list, neighbourlist.cpp:336-439 */
int pdo_list_build(const pdo_system *s, double list_cutoff, int nthreads, pdo_list *out) {
    int n = s->natom;
    double lim = SQR(list_cutoff);
    int32_t *cnt = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int nt = nthreads_eff(nthreads);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 32) num_threads(nt)
#endif
    for (int i = 0; i < n; i++) {
        int c = 0;
        for (int j = 0; j < i; j++) {
            double d[3] = {s->pos[3 * j] - s->pos[3 * i], s->pos[3 * j + 1] - s->pos[3 * i + 1],
                           s->pos[3 * j + 2] - s->pos[3 * i + 2]};
            min_image(s->box, d);
            if (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] <= lim) c++;
        }
        cnt[i] = c;
    }
    out->natom = n;
    out->start = (int64_t *)malloc(sizeof(int64_t) * ((size_t)n + 1));
    out->start[0] = 0;
    for (int i = 0; i < n; i++) out->start[i + 1] = out->start[i] + cnt[i];
    out->j = (int32_t *)malloc(sizeof(int32_t) * (size_t)(out->start[n] + 1));
    out->shift = (double *)malloc(sizeof(double) * 3 * (size_t)(out->start[n] + 1));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 32) num_threads(nt)
#endif
    for (int i = 0; i < n; i++) {
        int64_t k = out->start[i];
        for (int j = 0; j < i; j++) {
            double d[3] = {s->pos[3 * j] - s->pos[3 * i], s->pos[3 * j + 1] - s->pos[3 * i + 1],
                           s->pos[3 * j + 2] - s->pos[3 * i + 2]};
            double d0[3] = {d[0], d[1], d[2]};
            min_image(s->box, d);
            if (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] > lim) continue;
            out->j[k] = j;
            for (int c = 0; c < 3; c++) out->shift[3 * k + c] = d[c] - d0[c];
            k++;
        }
    }
    free(cnt);
    return 0;
}

void pdo_list_free(pdo_list *l) {
    free(l->start);
    free(l->j);
    free(l->shift);
    l->start = NULL;
    l->j = NULL;
    l->shift = NULL;
}

int pdo_nonbonded_list(const pdo_system *s, const pdo_list *l, const pdo_nb_params *p, int nthreads,
                       pdo_energies *e, double *force) {
    int n = s->natom;
    nb_consts c;
    nb_setup(p, &c);
    bo_table bt;
    bo_build(s, &bt);
    double tabV[8] = {0, 0, 0, p->Vdw14Scaling, 1, 1, 1, 1};
    double tabE[8] = {0, 0, 0, p->Elec14Scaling, 1, 1, 1, 1};
    int nt = nthreads_eff(nthreads);
    double *fbuf = (double *)calloc((size_t)nt * 3 * n, sizeof(double));
    double *ebuf = (double *)calloc((size_t)nt * 3, sizeof(double));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 32) num_threads(nt)
#endif
    for (int i = 0; i < n; i++) {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        double *f = fbuf + (size_t)tid * 3 * n;
        double *eb = ebuf + 3 * tid;
        double fi[3] = {0, 0, 0};
        for (int64_t k = l->start[i]; k < l->start[i + 1]; k++) {
            int j = l->j[k];
            double d[3];
            for (int q = 0; q < 3; q++) d[q] = s->pos[3 * j + q] - s->pos[3 * i + q] + l->shift[3 * k + q];
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            int bo = bo_lookup(&bt, i, j);
            double ev, ee, fm, dist;
            if (!nb_pair(p, &c, r2, s->radius[i], s->radius[j], s->epsilon[i], s->epsilon[j], s->charge[i],
                         s->charge[j], tabV[bo], tabE[bo], &ev, &ee, &fm, &dist))
                continue;
            eb[0] += ev;
            eb[1] += ee;
            eb[2] += dist * fm * PDO_ANGSTROM;
            double sc = fm / dist;
            for (int q = 0; q < 3; q++) {
                fi[q] += d[q] * sc;
                f[3 * j + q] -= d[q] * sc;
            }
        }
        for (int q = 0; q < 3; q++) f[3 * i + q] += fi[q];
    }
    memset(e, 0, sizeof(*e));
    for (int t = 0; t < nt; t++) {
        e->vdw += ebuf[3 * t];
        e->elec += ebuf[3 * t + 1];
        e->virial += ebuf[3 * t + 2];
        for (int k = 0; k < 3 * n; k++) force[k] += fbuf[(size_t)t * 3 * n + k];
    }
    e->epot = e->vdw + e->elec;
    free(fbuf);
    free(ebuf);
    bo_free(&bt);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Generalised Born (Still)                                                 */
/* ------------------------------------------------------------------------ */
static inline double gb_R(double r) { return r <= 0.01 ? 1.15 : r; } /* gbff.cpp:340-341 */

/* gbff.cpp:324-398 */
void pdo_gb_fixed_terms(int natom, const double *gbR, int ncov12, const int *cov12, const double *d12, int ncov13,
                        const int *cov13, const double *d13, const pdo_gb_params *p, double *vj, double *terms123) {
    for (int j = 0; j < natom; j++) {
        double Rj = gb_R(gbR[j]);
        vj[j] = 4.0 * PI_ * Rj * Rj * Rj / 3.0;
    }
    /* subtract half lens volumes of 1-2 partners in the order they are listed */
    for (int k = 0; k < ncov12; k++) {
        int j = cov12[2 * k], kk = cov12[2 * k + 1];
        double Rj = gb_R(gbR[j]), Rk = gb_R(gbR[kk]);
        double rjk = 1.01 * d12[k];
        double hjk = Rj * (1.0 + (Rk * Rk - Rj * Rj - rjk * rjk) / (2.0 * Rj * rjk));
        vj[j] -= PI_ * hjk * hjk * (3 * Rj - hjk) / 3;
    }
    for (int j = 0; j < natom; j++)
        if (vj[j] < 0) vj[j] = 0;
    for (int i = 0; i < natom; i++) terms123[i] = -166.0 / (gb_R(gbR[i]) + p->DielectricOffset + p->P1);
    double *t2 = (double *)calloc((size_t)natom, sizeof(double));
    double *t3 = (double *)calloc((size_t)natom, sizeof(double));
    for (int k = 0; k < ncov12; k++) {
        int i = cov12[2 * k], j = cov12[2 * k + 1];
        t2[i] += p->P2 * vj[j] / (SQR(d12[k]) * SQR(d12[k]));
    }
    for (int k = 0; k < ncov13; k++) {
        int i = cov13[2 * k], j = cov13[2 * k + 1];
        t3[i] += p->P3 * vj[j] / (SQR(d13[k]) * SQR(d13[k]));
    }
    for (int i = 0; i < natom; i++) terms123[i] = terms123[i] + t2[i] + t3[i];
    free(t2);
    free(t3);
}

static inline double sqrdist3(const double *a, const double *b) {
    return SQR(a[0] - b[0]) + SQR(a[1] - b[1]) + SQR(a[2] - b[2]);
}

/* gbff.cpp:432-483: full (shadow) list, plain Euclidean distance */
int pdo_gb_born_radii(const pdo_system *s, const pdo_gb_params *p, const double *gbR, const double *vj,
                      const double *terms123, int nthreads, double *born) {
    int n = s->natom;
    bo_table bt;
    bo_build(s, &bt);
    double invP5 = 1.0 / p->P5;
    double list2 = SQR(p->ListCutoff), still2 = SQR(p->GbsaStillCutoff);
    double halfeconv = pdo_halfeconv();
    int nt = nthreads_eff(nthreads);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
    for (int i = 0; i < n; i++) {
        double Ri = gbR[i];
        double Gpol = terms123[i];
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            double r2 = sqrdist3(s->pos + 3 * i, s->pos + 3 * j);
            if (r2 > list2) continue;
            if (r2 > still2) continue;
            if (bo_lookup(&bt, i, j) <= 2) continue;
            double Rj = gbR[j];
            double rdivR = r2 / SQR(Ri + Rj);
            double CCF = rdivR > invP5 ? 1.0 : SQR(0.5 - 0.5 * cos(rdivR * p->P5 * PI_));
            Gpol += p->P4 * vj[j] * CCF / SQR(r2);
        }
        born[i] = -halfeconv / Gpol + p->BornRadiusOffset;
    }
    bo_free(&bt);
    return 0;
}

/* gbff.cpp:1466-1835 (FastMode); radii from calcBornRadii_PairwiseApprox first (gbff.cpp:185-197).
 * FastMode = 0: calcBornForces (gbff.cpp:1189-1437), the GB part alone: every pair
 * within Cutoff (bonded ones too), the GB term above ExpApproxThreshold and
 * premul q_i q_j / r below it; PD's calcBornEnergy (gbff.cpp:537-596) is that
 * energy with no threshold (ExpApproxThreshold = -inf). */
int pdo_gb_forces(const pdo_system *s, const pdo_gb_params *p, const double *gbR, const double *vj,
                  const double *terms123, int nthreads, pdo_energies *e, double *force, double *born_out) {
    int n = s->natom;
    double *a = (double *)malloc(sizeof(double) * n);
    pdo_gb_born_radii(s, p, gbR, vj, terms123, nthreads, a);
    if (born_out) memcpy(born_out, a, sizeof(double) * n);
    bo_table bt;
    bo_build(s, &bt);
    const double econv = pdo_econv_joule();
    const double premul = -0.5 * econv * (1.0 / p->DielectricSolute - 1.0 / p->DielectricSolvent);
    const double sqrcutoff = SQR(p->Cutoff);
    const double invSwidth = 1.0 / (p->Cutoff - p->InnerCutoff);
    const double vdwinvSwidth = 1.0 / (p->VdwCutoff - p->VdwInnerCutoff);
    const double invdiel = 1.0 / p->DielectricSolute, invsolv = 1.0 / p->DielectricSolvent;
    const double list2 = SQR(p->ListCutoff);
    int nt = nthreads_eff(nthreads);
    /* per-thread accumulators: dE/dx (J/A), dE/da, energies */
    double *dedi = (double *)calloc((size_t)nt * 3 * n, sizeof(double));
    double *deda = (double *)calloc((size_t)nt * n, sizeof(double));
    double *eb = (double *)calloc((size_t)nt * 5, sizeof(double)); /* vdw, elec, pol, cross, self */

    /* loop 1: i > j pairs within Cutoff, gbff.cpp:1546-1746 */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
    for (int i = 0; i < n; i++) {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        double *D = dedi + (size_t)tid * 3 * n;
        double *A = deda + (size_t)tid * n;
        double *E = eb + 5 * tid;
        double ai = a[i], qi = s->charge[i];
        double dedai = 0;
        for (int j = 0; j < i; j++) {
            double dx = s->pos[3 * i] - s->pos[3 * j];
            double dy = s->pos[3 * i + 1] - s->pos[3 * j + 1];
            double dz = s->pos[3 * i + 2] - s->pos[3 * j + 2];
            double srij = dx * dx + dy * dy + dz * dz;
            if (srij > list2) continue;
            if (srij > sqrcutoff) continue;
            int typej = bo_lookup(&bt, i, j);
            double aj = a[j];
            double qiqj = qi * s->charge[j];
            double dist = sqrt(srij);
            double invd = 1.0 / dist;
            double aiaj = ai * aj;
            double uGB = -srij * 0.25 / aiaj;
            double s14 = typej == 3 ? p->Elec14Scaling : 1.0;
            double elec_pot = 0, elec_f = 0;
            if (!p->FastMode) {
                double epol, dedr;
                if (uGB > p->ExpApproxThreshold) {
                    double tGB = exp(uGB);
                    double lGB = srij + tGB * aiaj;
                    epol = premul * qiqj / sqrt(lGB);
                    dedr = -epol * (dist - 0.25 * dist * tGB) / lGB;
                    double dedalpha = -epol * tGB * (1.0 + 0.25 * srij / aiaj) / lGB;
                    if (dist >= p->InnerCutoff) {
                        double S = 1.0 - SQR(invSwidth * (dist - p->InnerCutoff));
                        double dSdd = -4.0 * SQR(invSwidth) * (dist - p->InnerCutoff) * S;
                        S = S * S;
                        dedr = S * dedr + dSdd * epol;
                        dedalpha *= S;
                        epol *= S;
                    }
                    dedai += dedalpha * aj;
                    A[j] += dedalpha * ai;
                } else {
                    epol = premul * qiqj * invd;
                    dedr = -epol * invd;
                    if (dist >= p->InnerCutoff) {
                        double S = 1.0 - SQR(invSwidth * (dist - p->InnerCutoff));
                        double dSdd = -4.0 * SQR(invSwidth) * (dist - p->InnerCutoff) * S;
                        S = S * S;
                        dedr = S * dedr + dSdd * epol;
                        epol *= S;
                    }
                }
                dedr *= 2 * invd;
                D[3 * i] += dedr * dx; D[3 * i + 1] += dedr * dy; D[3 * i + 2] += dedr * dz;
                D[3 * j] -= dedr * dx; D[3 * j + 1] -= dedr * dy; D[3 * j + 2] -= dedr * dz;
                E[2] += 2 * epol;
                E[3] += 2 * epol;
                continue;
            }
            if (uGB > p->ExpApproxThreshold) {
                double tGB = exp(uGB);
                double mGB = tGB * aiaj;
                double lGB = 1 / (srij + mGB);
                double fGB = sqrt(lGB);
                double epol = premul * qiqj * fGB;
                double dedr = -epol * (dist - 0.25 * dist * tGB) * lGB;
                double dedalpha = -epol * tGB * (1.0 - uGB) * lGB;
                if (typej >= 3) {
                    elec_pot = econv * invdiel * s14 * qiqj * invd;
                    elec_f = -elec_pot * invd;
                }
                if (dist >= p->InnerCutoff) {
                    double S = 1.0 - SQR(invSwidth * (dist - p->InnerCutoff));
                    double dSdd = -4.0 * SQR(invSwidth) * (dist - p->InnerCutoff) * S;
                    S = S * S;
                    elec_f = S * elec_f + elec_pot * dSdd;
                    elec_pot *= S;
                    dedr = S * dedr + dSdd * epol;
                    dedalpha *= S;
                    epol *= S;
                }
                dedr *= 2 * invd;
                D[3 * i] += dedr * dx; D[3 * i + 1] += dedr * dy; D[3 * i + 2] += dedr * dz;
                D[3 * j] -= dedr * dx; D[3 * j + 1] -= dedr * dy; D[3 * j + 2] -= dedr * dz;
                E[2] += 2 * epol;
                E[3] += 2 * epol;
                dedai += dedalpha * aj;
                A[j] += dedalpha * ai;
            } else if (typej >= 3) {
                elec_pot = econv * invsolv * s14 * qiqj * invd;
                elec_f = -elec_pot * invd;
                if (dist >= p->InnerCutoff) {
                    double S = 1.0 - SQR(invSwidth * (dist - p->InnerCutoff));
                    double dSdd = -4.0 * SQR(invSwidth) * (dist - p->InnerCutoff) * S;
                    S = S * S;
                    elec_f = S * elec_f + elec_pot * dSdd;
                    elec_pot *= S;
                }
            }
            if (typej >= 3) {
                double s14v = typej == 3 ? p->Vdw14Scaling : 1.0;
                double vdw_f = 0;
                if (dist < p->VdwCutoff) {
                    double rr = SQR(invd * (s->radius[i] + s->radius[j]));
                    double eps = s14v * s->epsilon[i] * s->epsilon[j];
                    double B = rr * rr * rr;
                    double AA = B * B;
                    double vpot = (2.0 * eps) * (0.5 * AA - B);
                    vdw_f = -(12.0 * eps * invd) * (AA - B);
                    if (dist > p->VdwInnerCutoff) {
                        double S = 1.0 - SQR(vdwinvSwidth * (dist - p->VdwInnerCutoff));
                        double dSdd = -4.0 * SQR(vdwinvSwidth) * (dist - p->VdwInnerCutoff) * S;
                        S = S * S;
                        vdw_f = S * vdw_f + vpot * dSdd;
                        vpot *= S;
                    }
                    E[0] += vpot;
                }
                E[1] += elec_pot;
                double fm = (vdw_f + elec_f) * invd;
                D[3 * i] += fm * dx; D[3 * i + 1] += fm * dy; D[3 * i + 2] += fm * dz;
                D[3 * j] -= fm * dx; D[3 * j + 1] -= fm * dy; D[3 * j + 2] -= fm * dz;
            }
        }
        A[i] += dedai;
        double epol = premul * SQR(qi) / ai;
        E[2] += epol;
        E[4] += epol;
        A[i] += -epol / ai;
    }
    /* reduce dE/da over threads */
    double *dedaT = (double *)calloc((size_t)n, sizeof(double));
    for (int t = 0; t < nt; t++)
        for (int i = 0; i < n; i++) dedaT[i] += deda[(size_t)t * n + i];

    /* loop 2: Born-radius chain rule over the full list, gbff.cpp:1768-1825 */
    const double invP5 = 1.0 / p->P5, still2 = SQR(p->GbsaStillCutoff);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
    for (int i = 0; i < n; i++) {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        double *D = dedi + (size_t)tid * 3 * n;
        double Ri = gbR[i];
        double gpi = -SQR(a[i]) / -166.0;
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            double dx = s->pos[3 * j] - s->pos[3 * i];
            double dy = s->pos[3 * j + 1] - s->pos[3 * i + 1];
            double dz = s->pos[3 * j + 2] - s->pos[3 * i + 2];
            double srij = dx * dx + dy * dy + dz * dz;
            if (srij > list2) continue;
            if (srij > still2) continue;
            if (bo_lookup(&bt, i, j) <= 2) continue;
            double Rj = gbR[j];
            double r6 = srij * srij * srij;
            double rdivR = srij / SQR(Ri + Rj);
            double CCF, dCCF;
            if (rdivR > invP5) {
                CCF = 1.0;
                dCCF = 0.0;
            } else {
                double theta = rdivR * p->P5 * PI_;
                double sq = 0.5 - 0.5 * cos(theta);
                CCF = sq * sq;
                dCCF = 2.0 * sq * sin(theta) * theta;
            }
            double dedr = gpi * dedaT[i] * p->P4 * vj[j] * (4.0 * CCF - dCCF) / r6;
            D[3 * i] += dedr * dx; D[3 * i + 1] += dedr * dy; D[3 * i + 2] += dedr * dz;
            D[3 * j] -= dedr * dx; D[3 * j + 1] -= dedr * dy; D[3 * j + 2] -= dedr * dz;
        }
    }
    memset(e, 0, sizeof(*e));
    for (int t = 0; t < nt; t++) {
        e->vdw += eb[5 * t];
        e->elec += eb[5 * t + 1];
        e->pol += eb[5 * t + 2];
        e->pol_cross += eb[5 * t + 3];
        e->pol_self += eb[5 * t + 4];
        for (int k = 0; k < 3 * n; k++) force[k] += dedi[(size_t)t * 3 * n + k] * (-1.0 / PDO_ANGSTROM);
    }
    e->epot = e->vdw + e->elec + e->pol;
    free(a);
    free(dedi);
    free(deda);
    free(dedaT);
    free(eb);
    bo_free(&bt);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* LCPO, lcpo.cpp:640-961 (full recalculation branch)                        */
/* ------------------------------------------------------------------------ */
#define LCPO_NLISTMAX 80 /* lcpo.h:24 */

int pdo_lcpo_forces(const pdo_system *s, double list_cutoff, const double *rad, const double *P, const double *sigma,
                    const int *use, int nthreads, pdo_energies *e, double *force, double *sasa) {
    int n = s->natom;
    int *nl_size = (int *)calloc((size_t)n, sizeof(int));
    int *nl_i = (int *)malloc(sizeof(int) * (size_t)n * LCPO_NLISTMAX);
    double *nl_s = (double *)malloc(sizeof(double) * (size_t)n * LCPO_NLISTMAX);
    double list2 = SQR(list_cutoff);
    const double TwoPI = 2 * PI_;
    /* close-contact lists: pairs j < i of the main list, both atoms in use,
     * overlapping spheres; capped per atom in insertion (= ascending index) order */
    for (int i = 0; i < n; i++) {
        if (!use[i]) continue;
        double ri = rad[i];
        for (int j = 0; j < i; j++) {
            double r2 = sqrdist3(s->pos + 3 * i, s->pos + 3 * j);
            if (r2 > list2) continue;
            if (!use[j]) continue;
            double rj = rad[j];
            if (r2 < SQR(ri + rj)) {
                double d = sqrt(r2);
                double invd = 1 / d;
                double ri2rj2divd2 = 0.5 * (SQR(ri) - SQR(rj)) * invd;
                double sij = TwoPI * ri * (ri - d * 0.5 - ri2rj2divd2);
                double sji = TwoPI * rj * (rj - d * 0.5 + ri2rj2divd2);
                if (nl_size[i] < LCPO_NLISTMAX) {
                    nl_i[i * LCPO_NLISTMAX + nl_size[i]] = j;
                    nl_s[i * LCPO_NLISTMAX + nl_size[i]] = sij;
                    nl_size[i]++;
                }
                if (nl_size[j] < LCPO_NLISTMAX) {
                    nl_i[j * LCPO_NLISTMAX + nl_size[j]] = i;
                    nl_s[j * LCPO_NLISTMAX + nl_size[j]] = sji;
                    nl_size[j]++;
                }
            }
        }
    }
    double epot_cav = 0;
    int nt = nthreads_eff(nthreads);
    double *ecav_t = (double *)calloc((size_t)nt, sizeof(double));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
    for (int i = 0; i < n; i++) {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        double der[3] = {0, 0, 0};
        if (!use[i]) {
            if (sasa) sasa[i] = 0;
            continue;
        }
        const double *pi = s->pos + 3 * i;
        double ri = rad[i];
        double Si = 4.0 * PI_ * ri * ri; /* sphereSurfaceArea, maths.cpp */
        double Si2 = 0, Si3 = 0, Si4 = 0;
        double d2[3] = {0, 0, 0}, d4[3] = {0, 0, 0};
        for (int jj = 0; jj < nl_size[i]; jj++) {
            int ja = nl_i[i * LCPO_NLISTMAX + jj];
            const double *pj = s->pos + 3 * ja;
            double Si2_t = nl_s[i * LCPO_NLISTMAX + jj];
            double Si3_t = 0, Si3ik_t = 0;
            double d = sqrt(sqrdist3(pi, pj));
            double rj = rad[ja];
            double invd = 1 / d;
            double rr = 0.5 * (SQR(ri) - SQR(rj)) * invd;
            double sji = TwoPI * rj * (rj - d * 0.5 + rr);
            rr *= 2.0 * invd;
            double n3[3] = {0, 0, 0}, n4[3] = {0, 0, 0}, n3b[3] = {0, 0, 0}, n4b[3] = {0, 0, 0};
            double dAdd = PI_ * rj * (-rr - 1);
            double ddd[3] = {-(pi[0] - pj[0]) / d, -(pi[1] - pj[1]) / d, -(pi[2] - pj[2]) / d};
            double n2[3] = {dAdd * ddd[0], dAdd * ddd[1], dAdd * ddd[2]};
            dAdd = PI_ * ri * (rr - 1);
            double a2t[3] = {dAdd * ddd[0], dAdd * ddd[1], dAdd * ddd[2]};
            for (int kk = 0; kk < nl_size[ja]; kk++) {
                int ka = nl_i[ja * LCPO_NLISTMAX + kk];
                if (ka == i) continue;
                const double *pk = s->pos + 3 * ka;
                double rk = rad[ka];
                double dik2 = sqrdist3(pi, pk);
                if (SQR(ri + rk) < dik2) continue;
                double dik = sqrt(dik2);
                double invdik = 1 / dik;
                double rrk = (SQR(ri) - SQR(rk)) * SQR(invdik);
                double dA = PI_ * ri * (rrk - 1);
                double dk[3] = {-(pi[0] - pk[0]) * invdik, -(pi[1] - pk[1]) * invdik, -(pi[2] - pk[2]) * invdik};
                double sjk = nl_s[ja * LCPO_NLISTMAX + kk];
                for (int c = 0; c < 3; c++) n3[c] += dA * dk[c];
                dA = PI_ * rk * (-rrk - 1);
                Si3ik_t += PI_ * ri * (2 * ri - dik - dik * rrk);
                for (int c = 0; c < 3; c++) {
                    n3b[c] += dA * dk[c];
                    n4b[c] += sjk * dA * dk[c];
                }
                Si3_t += sjk;
            }
            for (int c = 0; c < 3; c++) {
                n4[c] = sji * n3[c] + n4b[c];
                n3[c] += n3b[c];
                n4[c] += n2[c] * Si3ik_t;
                der[c] += n2[c] * (P[4 * ja + 1] * sigma[ja]) + n3[c] * (P[4 * ja + 2] * sigma[ja]) +
                          n4[c] * (P[4 * ja + 3] * sigma[ja]);
            }
            Si4 += Si3_t * Si2_t;
            Si3 += Si3_t;
            Si2 += Si2_t;
            for (int c = 0; c < 3; c++) {
                d2[c] += a2t[c];
                d4[c] += Si3_t * a2t[c];
            }
        }
        double SAi = P[4 * i] * Si + P[4 * i + 1] * Si2 + P[4 * i + 2] * Si3 + P[4 * i + 3] * Si4;
        for (int c = 0; c < 3; c++) der[c] += d2[c] * (P[4 * i + 1] * sigma[i]) + d4[c] * (P[4 * i + 3] * sigma[i]);
        if (SAi < 0) {
            SAi = 0;
            der[0] = der[1] = der[2] = 0;
        }
        if (sasa) sasa[i] = SAi;
        ecav_t[tid] += SAi * sigma[i];
        for (int c = 0; c < 3; c++) force[3 * i + c] += der[c] * (1 / PDO_ANGSTROM);
    }
    for (int t = 0; t < nt; t++) epot_cav += ecav_t[t];
    memset(e, 0, sizeof(*e));
    e->surf = epot_cav;
    e->epot = epot_cav;
    free(ecav_t);
    free(nl_size);
    free(nl_i);
    free(nl_s);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* integrators                                                               */
/* ------------------------------------------------------------------------ */
/* md.cpp:805-855 (thermostat/barostat are no-ops by default) */
double pdo_vv_step(int natom, double *pos, double *vel, const double *force, const double *mass, double dt) {
    double ekin = 0;
    for (int i = 0; i < natom; i++) {
        double tm = 0.5 * dt / mass[i];
        for (int c = 0; c < 3; c++) vel[3 * i + c] += force[3 * i + c] * tm;
    }
    for (int i = 0; i < natom; i++)
        ekin += 0.5 * mass[i] * (SQR(vel[3 * i]) + SQR(vel[3 * i + 1]) + SQR(vel[3 * i + 2]));
    for (int i = 0; i < natom; i++) {
        double tm = 0.5 * dt / mass[i];
        for (int c = 0; c < 3; c++) {
            double dv = force[3 * i + c] * tm;
            vel[3 * i + c] += dv;
            pos[3 * i + c] += dt * (vel[3 * i + c] + dv) * (1 / PDO_ANGSTROM);
            vel[3 * i + c] += dv;
        }
    }
    return ekin;
}

/* md.cpp:966-1003 */
void pdo_langevin_coeffs(double gamma, double t, double out[6]) {
    double gt = gamma * t;
    double c0, c1, c2, varv, varr, crv;
    if (gt > 0.05) {
        c0 = exp(-gt);
        c1 = (1 - c0) / gt;
        c2 = (1 - c1) / gt;
        double eg = exp(-gt);
        varv = 1.0 - eg * eg;
        varr = 2.0 * gt - 3.0 + (4.0 - eg) * eg;
        crv = SQR(1.0 - eg) / sqrt(varv * varr);
    } else {
        double g2 = gt * gt, g3 = gt * g2, g4 = g2 * g2, g5 = g2 * g3, g6 = g3 * g3, g7 = g3 * g4, g8 = g4 * g4,
               g9 = g4 * g5;
        c0 = 1 - gt + 0.5 * g2 - g3 / 6.0 + g4 / 24.0 - g5 / 120.0 + g6 / 720.0 - g7 / 5040.0 + g8 / 40320.0 -
             g9 / 362880.0;
        c1 = 1 - (0.5 * gt - g2 / 6.0 + g3 / 24.0 - g4 / 120.0 + g5 / 720.0 - g6 / 5040.0 + g7 / 40320.0 -
                  g8 / 362880.0);
        c2 = 0.5 - gt / 6.0 + g2 / 24.0 - g3 / 120.0 + g4 / 720.0 - g5 / 5040.0 + g6 / 40320.0 - g7 / 362880.0;
        varr = 2.0 * g3 / 3.0 - g4 / 2.0 + 7.0 * g5 / 30.0 - g6 / 12.0 + 31.0 * g7 / 1260.0 - g8 / 160.0 +
               127.0 * g9 / 90720.0;
        varv = 2.0 * gt - 2.0 * g2 + 4.0 * g3 / 3.0 - 2.0 * g4 / 3.0 + 4.0 * g5 / 15.0 - 4.0 * g6 / 45.0 +
               8.0 * g7 / 315.0 - 2.0 * g8 / 315.0 + 4.0 * g9 / 2835.0;
        crv = sqrt(3.0) * (0.5 - 3.0 * gt / 16.0 - 17.0 * g2 / 1280.0 + 17.0 * g3 / 6144.0 +
                           40967.0 * g4 / 34406400.0 - 57203.0 * g5 / 275251200.0 - 1429487.0 * g6 / 13212057600.0);
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = varv; out[4] = varr; out[5] = crv;
}

/* md.cpp:923-1063 (gamma*dt >= 1e-5 branch) */
double pdo_langevin_step(int natom, double *pos, double *vel, const double *force, const double *mass, double t,
                         double gamma, double T, const double *noise, int first_step, int last_step) {
    double cf[6];
    pdo_langevin_coeffs(gamma, t, cf);
    double c0 = cf[0], c1 = cf[1], c2 = cf[2], varv = cf[3], varr = cf[4], crv = cf[5];
    double gt = gamma * t;
    if (!first_step) {
        for (int i = 0; i < natom; i++) {
            double tm = t / mass[i];
            for (int c = 0; c < 3; c++) vel[3 * i + c] += (1.0 - c0 / c1) * force[3 * i + c] * tm / gt;
        }
    }
    double ekin = 0;
    for (int i = 0; i < natom; i++)
        ekin += 0.5 * mass[i] * (SQR(vel[3 * i]) + SQR(vel[3 * i + 1]) + SQR(vel[3 * i + 2]));
    if (!last_step) {
        double sq = sqrt(1.0 - SQR(crv));
        for (int i = 0; i < natom; i++) {
            double tm = t / mass[i];
            double kTdivm = PDO_KB * T / mass[i];
            double sigmav = sqrt(kTdivm * varv);
            double sigmar = sqrt(kTdivm * varr) / gamma;
            const double *nz = noise + 6 * i; /* n1x n2y n2x n1z n1y n2z */
            double n1[3] = {nz[0], nz[4], nz[3]}, n2[3] = {nz[2], nz[1], nz[5]};
            for (int c = 0; c < 3; c++) {
                double dvr = sigmav * (crv * n1[c] + sq * n2[c]);
                double drr = sigmar * n1[c];
                double dr = t * (c1 * vel[3 * i + c] + c2 * force[3 * i + c] * tm) + drr;
                double dv = (c0 * c2) * force[3 * i + c] * tm / c1 + dvr;
                pos[3 * i + c] += dr * (1 / PDO_ANGSTROM);
                vel[3 * i + c] = vel[3 * i + c] * c0 + dv;
            }
        }
    }
    return ekin;
}

/* ------------------------------------------------------------------------ */
/* bonded terms, ffbonded.cpp:945-1001 (bonds), 1054-1183 (angles),          */
/* 1270-1470 (dihedrals; impropers use the same law, :1594-1619)             */
/* ------------------------------------------------------------------------ */
static void cross3(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* dihedral with PD's angle convention phi = -atan2(sin, cos) of the
 * (i-a, a-b, b-j) normals; forces from the analytic gradient of phi */
static double dihedral_term(const double *pos, const int *idx, const double *par, double *force) {
    int ti = idx[0], ta = idx[1], tb = idx[2], tj = idx[3], terms = idx[4];
    const double *pi = pos + 3 * ti, *pa = pos + 3 * ta, *pb = pos + 3 * tb, *pj = pos + 3 * tj;
    double v1[3], v2[3], v3[3];
    for (int c = 0; c < 3; c++) { v1[c] = pi[c] - pa[c]; v2[c] = pa[c] - pb[c]; v3[c] = pb[c] - pj[c]; }
    double n1[3], n2[3], n3[3];
    cross3(v1, v2, n1);
    cross3(v2, v3, n2);
    cross3(v2, n1, n3);
    double m1 = sqrt(dot3(n1, n1)), m2 = sqrt(dot3(n2, n2)), m3 = sqrt(dot3(n3, n3));
    double cphi = dot3(n1, n2) / (m1 * m2);
    double sphi = dot3(n3, n2) / (m3 * m2);
    double phi = -atan2(sphi, cphi);
    double E = 0, dEdphi = 0;
    for (int t = 0; t < terms; t++) {
        double k = par[3 * t], nn = par[3 * t + 1], g = par[3 * t + 2];
        if (nn > 0) {
            E += k * (1.0 + cos(nn * phi + g));
            dEdphi += -nn * k * sin(nn * phi + g);
        } else {
            double diff = phi - g;
            if (diff < -PI_) diff += 2.0 * PI_;
            else if (diff > PI_) diff -= 2.0 * PI_;
            E += k * diff * diff;
            dEdphi += 2.0 * k * diff;
        }
    }
    /* gradient of the standard dihedral (F=i-a, G=a-b, H=j-b; Blondel &
     * Karplus 1996), which equals PD's phi for this choice of vectors */
    double F[3], G[3], H[3], A[3], B[3];
    for (int c = 0; c < 3; c++) { F[c] = pi[c] - pa[c]; G[c] = pa[c] - pb[c]; H[c] = pj[c] - pb[c]; }
    cross3(F, G, A);
    cross3(H, G, B);
    double A2 = dot3(A, A), B2 = dot3(B, B), Gm = sqrt(dot3(G, G));
    double FG = dot3(F, G), HG = dot3(H, G);
    for (int c = 0; c < 3; c++) {
        double gi = -Gm / A2 * A[c];
        double gj = Gm / B2 * B[c];
        double ga = Gm / A2 * A[c] + FG / (A2 * Gm) * A[c] - HG / (B2 * Gm) * B[c];
        double gb = -Gm / B2 * B[c] - FG / (A2 * Gm) * A[c] + HG / (B2 * Gm) * B[c];
        double s = -dEdphi * (1.0 / PDO_ANGSTROM);
        force[3 * ti + c] += s * gi;
        force[3 * ta + c] += s * ga;
        force[3 * tb + c] += s * gb;
        force[3 * tj + c] += s * gj;
    }
    return E;
}

int pdo_bonded(int natom, const double *pos, int nbond, const int *bidx, const double *bpar, int nangle,
               const int *aidx, const double *apar, int ntors, const int *tidx, const double *tpar, int nimpr,
               const int *iidx, const double *ipar, double *energy, double *force) {
    (void)natom;
    double eb = 0, ea = 0, et = 0, ei = 0;
    for (int b = 0; b < nbond; b++) {
        int i = bidx[2 * b], j = bidx[2 * b + 1];
        double l = bpar[2 * b], k = bpar[2 * b + 1];
        double v[3] = {pos[3 * i] - pos[3 * j], pos[3 * i + 1] - pos[3 * j + 1], pos[3 * i + 2] - pos[3 * j + 2]};
        double d = sqrt(dot3(v, v));
        double fm = 2 * k * (d - l) / PDO_ANGSTROM;
        eb += k * SQR(d - l);
        for (int c = 0; c < 3; c++) {
            force[3 * i + c] -= v[c] * fm / d;
            force[3 * j + c] += v[c] * fm / d;
        }
    }
    for (int q = 0; q < nangle; q++) {
        int i = aidx[3 * q], a = aidx[3 * q + 1], j = aidx[3 * q + 2];
        double theta0 = apar[2 * q], k = apar[2 * q + 1];
        if (k == 0) continue;
        double u[3], w[3];
        for (int c = 0; c < 3; c++) { u[c] = pos[3 * i + c] - pos[3 * a + c]; w[c] = pos[3 * j + c] - pos[3 * a + c]; }
        double lu = sqrt(dot3(u, u)), lw = sqrt(dot3(w, w));
        double ct = dot3(u, w) / (lu * lw);
        double th = acos(ct);
        double st = sin(th);
        ea += k * SQR(th - theta0);
        double dEdth = 2 * k * (th - theta0) / PDO_ANGSTROM;
        for (int c = 0; c < 3; c++) {
            /* dtheta/dr_i = (cos u^ - w^) / (|u| sin) */
            double gi = (ct * u[c] / lu - w[c] / lw) / (lu * st);
            double gj = (ct * w[c] / lw - u[c] / lu) / (lw * st);
            force[3 * i + c] -= dEdth * gi;
            force[3 * j + c] -= dEdth * gj;
            force[3 * a + c] += dEdth * (gi + gj);
        }
    }
    for (int q = 0; q < ntors; q++) et += dihedral_term(pos, tidx + 5 * q, tpar + 12 * q, force);
    for (int q = 0; q < nimpr; q++) ei += dihedral_term(pos, iidx + 5 * q, ipar + 12 * q, force);
    energy[0] = eb;
    energy[1] = ea;
    energy[2] = et;
    energy[3] = ei;
    return 0;
}
