/*
 * gy_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle; see gy_oracle.h).
 *
 * FP64 CPU restatement of Graphyt's explicit GIMP MPM time step, written from the
 * reference's behaviour, function by function.  Every routine names the reference
 * file:line it follows.  The loop structure is kept where it decides the result or the
 * cost: P2G is the reference's node-centric gather over a 4x4x4 cell window with
 * first-come body slots (Extrapolation.cpp:31-125, 166-286), so the CPU timing taken from
 * this file is a fair stand-in for the reference's OpenMP iterate_CPU.
 *
 * Deliberate, documented deviations from the reference:
 *  - Sort (Extrapolation.cpp:370-503): the reference uses std::sort, whose order among
 *    particles of one cell is unspecified.  Here the order is fixed as (cellID, particle id),
 *    which the GPU body-slot rule uses too.
 *  - Thermal terms (Extrapolation.cpp:281-283, 358-362; TimeIntegration.cpp:50): the
 *    sort moves each particle's temperature gradient with the particle.  The reference's
 *    sort copies one of its three components per slot (Extrapolation.cpp:446, 485), which
 *    corrupts the gradients the P2G right after each sort uses; that copy depends on the
 *    reference's own array order and is not restated.
 *  - 3x3 symmetric eigen-solve (eig3.cpp:258-267, JAMA tred2+tql2) is replaced by a
 *    cyclic Jacobi rotation method; the damaged stress V diag(s') V^T depends only on the
 *    eigenpairs, so the two agree to rounding.
 *  - fixed_grid_bcs (off by default) gives grid_vz & co. a body; the reference's are empty.
 */
#include "gy_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* BCTypes::function values (BoundaryConditions.hpp:6-77), in declaration order. */
enum {
    BC_NONE = 0, BC_GRID_VX = 1, BC_GRID_VY = 2, BC_GRID_VZ = 3, BC_GRID_VX_VY = 11,
    BC_GRID_VX_VZ = 12, BC_GRID_VY_VZ = 13, BC_GRID_VX_VY_VZ = 18,
    BC_MP_VX = 33, BC_MP_VY = 34, BC_MP_VZ = 35, BC_MP_FX = 37, BC_MP_FY = 38, BC_MP_FZ = 39,
    BC_MP_VX_VY = 40, BC_MP_FX_FY = 43, BC_MP_STRESS_XX_YY = 63, BC_MP_VXSIN = 65,
    BC_MP_VYSIN = 66, BC_MP_SYYSIN = 67
};

#define PI_REF 3.14159 /* the reference's literal pi (TimeIntegration.cpp:240, ConstitutiveModels.cpp:247) */

struct gyo {
    int is3D;
    double L[3], h;
    int Nx, Ny, Nz, Nn;
    int Ncx, Ncy, Ncz, Nc;
    int *nidx[3]; /* node index per axis as the reference derives it from positions */

    /* node fields (Nodes.hpp:22-55): COM, body 1, body 2 */
    double *m0, *m1, *m2;
    double *Tn, *Rn; /* node temperature (sum S T m c) and temperature rate (Nodes.hpp:47-48) */
    double *p0, *p1, *p2;
    double *f0, *f1, *f2;
    double *v0, *v1, *v2;
    double *a0, *a1, *a2;
    double *n1, *n2;
    int *body;
    unsigned char *rigid;
    int *nbct;
    double *nbcv;
    int *cells, *ccount;

    /* particle fields (MaterialPoints.hpp:84-137) */
    int N, cap;
    double psep, t;
    double *x, *x0, *u, *v, *gv, *a, *er, *dr, *s, *e, *ep, *eqp, *D, *smax, *m, *rho, *V, *nrm;
    double *T, *gT, *Tr; /* temperature, its gradient, its rate (MaterialPoints.hpp:103-105) */
    double *flaw;        /* scale of the Grady-Kipp activation strain (1: the reference's e_min) */
    int *cell, *mat, *obj, *bct, *pid;
    double *bcv;
    unsigned char *hold;

    int nmat;
    gyo_material *mats;
    gyo_params prm;
    double dt;
    int bad; /* set when a particle key falls outside [0, Nc) */
};

/* ------------------------------------------------------------------------------------ */
/* GIMP basis, Extrapolation.cpp:556-647.  dist = x_node - x_particle, lp = psep/2.       */

double gyo_gimp_shape(double d, double h, double lp)
{
    if (d <= -h - lp) return 0.0;
    if (d <= -h + lp) return (h + lp + d) * (h + lp + d) / (4.0 * h * lp);
    if (d <= -lp) return 1.0 + d / h;
    if (d <= lp) return 1.0 - (d * d + lp * lp) / (2.0 * h * lp);
    if (d <= h - lp) return 1.0 - d / h;
    if (d <= h + lp) return (h + lp - d) * (h + lp - d) / (4.0 * h * lp);
    return 0.0;
}

/* The gradient branch keeps the reference's mix of strict and non-strict bounds
 * (Extrapolation.cpp:613-640) and its sign factor x_p/|x_p| (:642). */
double gyo_gimp_grad(double d, double h, double lp, double xp)
{
    double g = 0.0;
    if (d < -h - lp) g = 0.0;
    else if (-h - lp < d && d < -h + lp) g = (h + lp + d) / (2.0 * h * lp);
    else if (-h + lp <= d && d < -lp) g = 1.0 / h;
    else if (-lp <= d && d < lp) g = -d / (h * lp);
    else if (lp <= d && d < h - lp) g = -1.0 / h;
    else if (h - lp <= d && d <= h + lp) g = -(h + lp - d) / (2.0 * h * lp);
    g = g * xp / fabs(xp);
    return -g;
}

/* ------------------------------------------------------------------------------------ */
/* construction                                                                           */

static double *dalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }
static int *ialloc(size_t n) { return (int *)calloc(n ? n : 1, sizeof(int)); }

gyo *gyo_create(double Lx, double Ly, double Lz, double h, double psep)
{
    /* Nodes::Nodes, Nodes.cpp:8-141: numNodes is rounded, Nx/Ny/Nz truncated (:12, :71-73). */
    double nn = round((1.0 + Lx / h) * (1.0 + Ly / h) * (1.0 + Lz / h));
    int Nx = (int)(1.0 + Lx / h), Ny = (int)(1.0 + Ly / h), Nz = (int)(1.0 + Lz / h);
    if ((double)Nx * Ny * Nz != nn || Nx < 6 || Ny < 6) return NULL;
    gyo *o = (gyo *)calloc(1, sizeof(gyo));
    o->L[0] = Lx; o->L[1] = Ly; o->L[2] = Lz; o->h = h; o->psep = psep;
    o->Nx = Nx; o->Ny = Ny; o->Nz = Nz; o->Nn = Nx * Ny * Nz;
    o->is3D = (Nz > 1);
    o->Ncx = Nx - 1; o->Ncy = Ny - 1; o->Ncz = o->is3D ? Nz - 1 : 1;
    o->Nc = o->Ncx * o->Ncy * o->Ncz;
    int nax[3] = {Nx, Ny, Nz};
    for (int ax = 0; ax < 3; ax++) {
        o->nidx[ax] = ialloc(nax[ax]);
        /* extrapToNodes derives the node's cell from its position (Extrapolation.cpp:43-45);
         * (i*h - 0)/h can round below i, and the window then starts one cell lower. */
        for (int i = 0; i < nax[ax]; i++) {
            double pos = i * h;
            o->nidx[ax][i] = (int)((pos - 0.0) / h);
        }
    }
    size_t Nn = (size_t)o->Nn;
    o->m0 = dalloc(Nn); o->m1 = dalloc(Nn); o->m2 = dalloc(Nn);
    o->Tn = dalloc(Nn); o->Rn = dalloc(Nn);
    o->p0 = dalloc(3 * Nn); o->p1 = dalloc(3 * Nn); o->p2 = dalloc(3 * Nn);
    o->f0 = dalloc(3 * Nn); o->f1 = dalloc(3 * Nn); o->f2 = dalloc(3 * Nn);
    o->v0 = dalloc(3 * Nn); o->v1 = dalloc(3 * Nn); o->v2 = dalloc(3 * Nn);
    o->a0 = dalloc(3 * Nn); o->a1 = dalloc(3 * Nn); o->a2 = dalloc(3 * Nn);
    o->n1 = dalloc(3 * Nn); o->n2 = dalloc(3 * Nn);
    o->body = ialloc(2 * Nn);
    o->rigid = (unsigned char *)calloc(2 * Nn, 1);
    o->nbct = ialloc(Nn);
    o->nbcv = dalloc(4 * Nn);
    o->cells = ialloc(Nn);
    o->ccount = ialloc(Nn);
    for (size_t n = 0; n < 2 * Nn; n++) o->body[n] = -1;
    return o;
}

static void free_particles(gyo *o)
{
    double **d[] = {&o->x, &o->x0, &o->u, &o->v, &o->gv, &o->a, &o->er, &o->dr, &o->s, &o->e,
                    &o->ep, &o->eqp, &o->D, &o->smax, &o->m, &o->rho, &o->V, &o->nrm, &o->bcv,
                    &o->T, &o->gT, &o->Tr, &o->flaw};
    for (size_t i = 0; i < sizeof(d) / sizeof(d[0]); i++) { free(*d[i]); *d[i] = NULL; }
    int **ii[] = {&o->cell, &o->mat, &o->obj, &o->bct, &o->pid};
    for (size_t i = 0; i < sizeof(ii) / sizeof(ii[0]); i++) { free(*ii[i]); *ii[i] = NULL; }
    free(o->hold); o->hold = NULL;
}

void gyo_destroy(gyo *o)
{
    if (!o) return;
    double *d[] = {o->m0, o->m1, o->m2, o->Tn, o->Rn, o->p0, o->p1, o->p2, o->f0, o->f1, o->f2, o->v0,
                   o->v1, o->v2, o->a0, o->a1, o->a2, o->n1, o->n2, o->nbcv};
    for (size_t i = 0; i < sizeof(d) / sizeof(d[0]); i++) free(d[i]);
    free(o->body); free(o->rigid); free(o->nbct); free(o->cells); free(o->ccount);
    for (int ax = 0; ax < 3; ax++) free(o->nidx[ax]);
    free_particles(o);
    free(o->mats);
    free(o);
}

#define GROW(ptr, type, w) ptr = (type *)realloc(ptr, (size_t)cap * (w) * sizeof(type))

int gyo_add_particles(gyo *o, int n, const double *pos, const int *mat, const int *obj)
{
    int N0 = o->N, N1 = o->N + n;
    if (N1 > o->cap) {
        int cap = N1 + N1 / 2 + 16;
        GROW(o->x, double, 3); GROW(o->x0, double, 3); GROW(o->u, double, 3); GROW(o->v, double, 3);
        GROW(o->gv, double, 3); GROW(o->a, double, 3); GROW(o->er, double, 6); GROW(o->dr, double, 1);
        GROW(o->s, double, 6); GROW(o->e, double, 6); GROW(o->ep, double, 6); GROW(o->eqp, double, 1);
        GROW(o->D, double, 1); GROW(o->smax, double, 1); GROW(o->m, double, 1); GROW(o->rho, double, 1);
        GROW(o->V, double, 1); GROW(o->nrm, double, 3); GROW(o->bcv, double, 4);
        GROW(o->T, double, 1); GROW(o->gT, double, 3); GROW(o->Tr, double, 1); GROW(o->flaw, double, 1);
        GROW(o->cell, int, 1); GROW(o->mat, int, 1); GROW(o->obj, int, 1); GROW(o->bct, int, 1);
        GROW(o->pid, int, 1);
        o->hold = (unsigned char *)realloc(o->hold, (size_t)cap);
        o->cap = cap;
    }
    for (int q = 0; q < n; q++) {
        int p = N0 + q;
        for (int k = 0; k < 3; k++) {
            o->x[3 * p + k] = pos[3 * q + k];
            o->x0[3 * p + k] = pos[3 * q + k];
            o->u[3 * p + k] = o->v[3 * p + k] = o->gv[3 * p + k] = o->a[3 * p + k] = 0.0;
            o->nrm[3 * p + k] = 0.0;
            o->gT[3 * p + k] = 0.0;
        }
        o->T[p] = o->Tr[p] = 0.0;
        o->flaw[p] = 1.0;
        for (int k = 0; k < 6; k++) o->er[6 * p + k] = o->s[6 * p + k] = o->e[6 * p + k] = o->ep[6 * p + k] = 0.0;
        for (int k = 0; k < 4; k++) o->bcv[4 * p + k] = 0.0;
        o->dr[p] = o->eqp[p] = o->D[p] = o->smax[p] = o->m[p] = o->rho[p] = o->V[p] = 0.0;
        o->mat[p] = mat ? mat[q] : 0;
        o->obj[p] = obj ? obj[q] : 0;
        o->bct[p] = BC_NONE;
        o->hold[p] = 0;
        o->pid[p] = p;
        /* the initial key has no quarter-cell shift (MaterialPoints.cpp:220-233) */
        int idx = (int)((o->x[3 * p + 0] - 0.0) / o->h);
        int idy = (int)((o->x[3 * p + 1] - 0.0) / o->h);
        int idz = (int)((o->x[3 * p + 2] - 0.0) / o->h);
        o->cell[p] = idx + idy * (o->Nx - 1) + idz * (o->Nx - 1) * (o->Ny - 1);
    }
    o->N = N1;
    return N1;
}

void gyo_set_particle_vel(gyo *o, int p, double vx, double vy, double vz)
{
    o->v[3 * p + 0] = vx; o->v[3 * p + 1] = vy; o->v[3 * p + 2] = vz;
}
void gyo_set_particle_stress(gyo *o, int p, const double *s6)
{
    for (int k = 0; k < 6; k++) o->s[6 * p + k] = s6[k];
}
void gyo_set_particle_damage(gyo *o, int p, double D) { o->D[p] = D; }
void gyo_hold_particle(gyo *o, int p) { o->hold[p] = 1; }
void gyo_set_particle_bc(gyo *o, int p, int type, const double *val, int nval)
{
    o->bct[p] = type;
    for (int i = 0; i < nval && i < 4; i++) o->bcv[4 * p + i] = val[i];
}
void gyo_set_particle_temps(gyo *o, int count, const int *ids, const double *T)
{
    int *at = ialloc((size_t)o->N);
    for (int q = 0; q < o->N; q++) at[o->pid[q]] = q;
    for (int q = 0; q < count; q++)
        if (ids[q] >= 0 && ids[q] < o->N) o->T[at[ids[q]]] = T[q];
    free(at);
}
/* Per-particle scale of the Grady-Kipp activation strain, by particle id: e_min = w (V k)^(-1/m).
 * The reference's deterministic e_min (DamageModels.cpp:102-103) is w = 1, the default; a
 * Weibull draw w = (-ln U)^(1/m) gives the weakest flaw of a Poisson flaw population of
 * density k e^m in the particle's volume. */
void gyo_set_particle_flaws(gyo *o, int count, const int *ids, const double *w)
{
    int *at = ialloc((size_t)o->N);
    for (int q = 0; q < o->N; q++) at[o->pid[q]] = q;
    for (int q = 0; q < count; q++)
        if (ids[q] >= 0 && ids[q] < o->N) o->flaw[at[ids[q]]] = w[q];
    free(at);
}
void gyo_set_node_bc(gyo *o, int n, int type, const double *val, int nval)
{
    o->nbct[n] = type;
    for (int i = 0; i < nval && i < 4; i++) o->nbcv[4 * n + i] = val[i];
}

/* Solver::Solver and Solver::initialize, Solver.cpp:7-69. */
int gyo_init_solver(gyo *o, const gyo_params *prm, int nmat, const gyo_material *mats)
{
    o->prm = *prm;
    o->nmat = nmat;
    free(o->mats);
    o->mats = (gyo_material *)malloc((size_t)(nmat ? nmat : 1) * sizeof(gyo_material));
    memcpy(o->mats, mats, (size_t)nmat * sizeof(gyo_material));
    double maxK = 1.0, minrho = 1e15;
    for (int i = 0; i < nmat; i++) {
        if (mats[i].bulkMod > maxK) maxK = mats[i].bulkMod;
        if (mats[i].density < minrho) minrho = mats[i].density;
    }
    o->dt = prm->CFL * (o->h / sqrt(maxK / minrho));
    for (int p = 0; p < o->N; p++) {
        int mid = o->mat[p];
        if (mid < 0 || mid >= nmat) return -1;
        o->rho[p] = mats[mid].density;
        if (prm->is3D) {
            o->V[p] = o->psep * o->psep * o->psep;
            o->m[p] = o->rho[p] * o->V[p];
            if (mats[mid].isRigid) o->m[p] = 1.0;
        } else {
            o->V[p] = o->psep * o->psep; /* per unit depth; no rigid override in 2D */
            o->m[p] = o->rho[p] * o->V[p];
        }
    }
    return 0;
}

double gyo_get_dt(const gyo *o) { return o->dt; }
void gyo_set_dt(gyo *o, double dt) { o->dt = dt; }
void gyo_set_params(gyo *o, const gyo_params *prm) { o->prm = *prm; }

/* ------------------------------------------------------------------------------------ */
/* (a) sort, Extrapolation.cpp:370-503 -- order fixed as (cellID, pid)                    */

#define PERM(arr, type, w)                                                              \
    do {                                                                                \
        type *tmp_ = (type *)malloc((size_t)N * (w) * sizeof(type));                   \
        for (int i_ = 0; i_ < N; i_++)                                                  \
            for (int k_ = 0; k_ < (w); k_++) tmp_[(size_t)i_ * (w) + k_] = arr[(size_t)order[i_] * (w) + k_]; \
        free(arr);                                                                      \
        arr = tmp_;                                                                     \
    } while (0)

static void sort_particles(gyo *o)
{
    int N = o->N, Nc = o->Nc;
    memset(o->ccount, 0, sizeof(int) * (size_t)o->Nn);
    for (int p = 0; p < N; p++) {
        int g = o->cell[p];
        if (g >= Nc) { o->bad = 1; return; }
        if (g >= 0) o->ccount[g]++;
    }
    /* counting sort over (cell, pid): walk particles in pid order, bucket by cell */
    int *at = ialloc(N), *order = ialloc(N), *start = ialloc((size_t)Nc + 1);
    for (int p = 0; p < N; p++) at[o->pid[p]] = p;
    int nneg = 0;
    for (int p = 0; p < N; p++)
        if (o->cell[p] < 0) nneg++;
    start[0] = nneg;
    for (int c = 0; c < Nc; c++) start[c + 1] = start[c] + o->ccount[c];
    int negpos = 0;
    for (int q = 0; q < N; q++) {
        int p = at[q];
        int g = o->cell[p];
        if (g < 0) order[negpos++] = p;
        else order[start[g]++] = p;
    }
    free(at); free(start);
    /* permute every array the reference permutes (Extrapolation.cpp:406-491); the rate
     * arrays are rebuilt each step and stay in place, as in the reference */
    PERM(o->x, double, 3); PERM(o->x0, double, 3); PERM(o->u, double, 3); PERM(o->v, double, 3);
    PERM(o->gv, double, 3); PERM(o->s, double, 6); PERM(o->e, double, 6); PERM(o->ep, double, 6);
    PERM(o->eqp, double, 1); PERM(o->D, double, 1); PERM(o->smax, double, 1); PERM(o->m, double, 1);
    PERM(o->rho, double, 1); PERM(o->obj, int, 1); PERM(o->V, double, 1); PERM(o->nrm, double, 3);
    PERM(o->bcv, double, 4); PERM(o->mat, int, 1); PERM(o->cell, int, 1); PERM(o->hold, unsigned char, 1);
    PERM(o->bct, int, 1); PERM(o->pid, int, 1); PERM(o->T, double, 1); PERM(o->gT, double, 3);
    PERM(o->flaw, double, 1);
    o->cap = N;
    free(order);
    /* cell start table: exclusive scan with cells[0] = 0 (Extrapolation.cpp:494-501) */
    int cur = 0;
    o->cells[0] = 0;
    for (int c = 1; c < Nc; c++) {
        cur += o->ccount[c - 1];
        o->cells[c] = cur;
    }
}

/* ------------------------------------------------------------------------------------ */
/* node reset, Grid.cpp:797-860; particle rate reset, TimeIntegration.cpp:145-161         */

static void reset_nodes(gyo *o)
{
    size_t Nn = (size_t)o->Nn;
    memset(o->m0, 0, Nn * 8); memset(o->m1, 0, Nn * 8); memset(o->m2, 0, Nn * 8);
    memset(o->Tn, 0, Nn * 8); memset(o->Rn, 0, Nn * 8);
    double *z3[] = {o->p0, o->p1, o->p2, o->f0, o->f1, o->f2, o->v0, o->v1, o->v2,
                    o->a0, o->a1, o->a2, o->n1, o->n2};
    for (size_t i = 0; i < sizeof(z3) / sizeof(z3[0]); i++) memset(z3[i], 0, 3 * Nn * 8);
    for (size_t n = 0; n < 2 * Nn; n++) { o->body[n] = -1; o->rigid[n] = 0; }
}

static void reset_rates(gyo *o)
{
    for (int p = 0; p < o->N; p++) {
        o->dr[p] = 0.0;
        o->Tr[p] = 0.0;
        for (int k = 0; k < 3; k++) { o->a[3 * p + k] = 0.0; o->gv[3 * p + k] = 0.0; }
        for (int k = 0; k < 6; k++) o->er[6 * p + k] = 0.0;
    }
}

/* ------------------------------------------------------------------------------------ */
/* (b) P2G: node-centric gather, Extrapolation.cpp:31-125 and 166-286                     */

static void p2g_pair(gyo *o, int mp, int n, const double *np)
{
    const double h = o->h, lp = 0.5 * o->psep;
    const double *xp = o->x + 3 * mp;
    double sx = gyo_gimp_shape(np[0] - xp[0], h, lp);
    double sy = gyo_gimp_shape(np[1] - xp[1], h, lp);
    double sz = gyo_gimp_shape(np[2] - xp[2], h, lp);
    double gx = gyo_gimp_grad(np[0] - xp[0], h, lp, xp[0]);
    double gy = gyo_gimp_grad(np[1] - xp[1], h, lp, xp[1]);
    double gz = gyo_gimp_grad(np[2] - xp[2], h, lp, xp[2]);
    double mass = o->m[mp];
    int mid = o->mat[mp], ob = o->obj[mp];
    int isRigid = o->mats[mid].isRigid;
    if (isRigid) mass = 1.0;
    if (!o->is3D) { sz = 1.0; gz = 0.0; }
    const double *s = o->s + 6 * mp, *vel = o->v + 3 * mp;
    const double *g = o->prm.gravity;
    double rho = o->rho[mp], vol = o->V[mp];

    /* first-come body slots, even for zero weight (Extrapolation.cpp:191-208) */
    int *b = o->body + 2 * n;
    unsigned char *rg = o->rigid + 2 * n;
    if (b[0] == -1) b[0] = ob;
    if (b[1] == -1 && b[0] != ob) b[1] = ob;
    if (isRigid && !rg[0] && b[0] == ob) rg[0] = 1;
    else if (isRigid && !rg[1] && b[1] == ob) rg[1] = 1;

    double w = sx * sy * sz;
    double fx = (mass / rho) * ((gx * sy * sz * s[0]) + (gy * sx * sz * s[3]) + (gz * sx * sy * s[5]));
    double fy = (mass / rho) * ((gx * sy * sz * s[3]) + (gy * sx * sz * s[1]) + (gz * sx * sy * s[4]));
    double fz = (mass / rho) * ((gx * sy * sz * s[5]) + (gy * sx * sz * s[4]) + (gz * sx * sy * s[2]));
    double *mb = NULL, *pb = NULL, *fb = NULL, *nb = NULL;
    if (b[0] == ob) { mb = o->m1 + n; pb = o->p1 + 3 * n; fb = o->f1 + 3 * n; nb = o->n1 + 3 * n; }
    else if (b[1] == ob) { mb = o->m2 + n; pb = o->p2 + 3 * n; fb = o->f2 + 3 * n; nb = o->n2 + 3 * n; }
    if (mb) {
        *mb += w * mass;
        pb[0] += w * mass * vel[0];
        pb[1] += w * mass * vel[1];
        pb[2] += w * mass * vel[2];
        fb[0] -= fx; fb[1] -= fy; fb[2] -= fz;
        if (!isRigid) {
            fb[0] += w * mass * g[0];
            fb[1] += w * mass * g[1];
            fb[2] += w * mass * g[2];
        }
        nb[0] += (gx * sy * sz * vol);
        nb[1] += (sx * gy * sz * vol);
        nb[2] += (sx * sy * gz * vol);
    }
    /* centre-of-mass fields: gravity always added (Extrapolation.cpp:265-278) */
    o->m0[n] += w * mass;
    o->p0[3 * n + 0] += w * mass * vel[0];
    o->p0[3 * n + 1] += w * mass * vel[1];
    o->p0[3 * n + 2] += w * mass * vel[2];
    o->f0[3 * n + 0] -= fx; o->f0[3 * n + 1] -= fy; o->f0[3 * n + 2] -= fz;
    o->f0[3 * n + 0] += w * mass * g[0];
    o->f0[3 * n + 1] += w * mass * g[1];
    o->f0[3 * n + 2] += w * mass * g[2];
    /* thermal (Extrapolation.cpp:280-283): node temperature sum S T m c, not normalised;
     * the rate from the particle's temperature gradient of the previous G2P */
    const gyo_material *M = &o->mats[mid];
    const double *gT = o->gT + 3 * mp;
    o->Tn[n] += w * o->T[mp] * mass * M->specificHeatCapacity;
    o->Rn[n] -= (mass / rho) * M->thermalConductivity *
                ((gx * sy * sz * gT[0]) + (sx * gy * sz * gT[1]) + (sx * sy * gz * gT[2]));
}

static void p2g(gyo *o)
{
    const int Nx = o->Nx, Ny = o->Ny, Ncx = o->Ncx, Ncy = o->Ncy, Nc = o->Nc;
    const int kmin = o->is3D ? -2 : 0, kmax = o->is3D ? 2 : 1;
#pragma omp parallel for schedule(dynamic, 64)
    for (int n = 0; n < o->Nn; n++) {
        int i = n % Nx, j = (n / Nx) % Ny, k = n / (Nx * Ny);
        double np[3] = {i * o->h, j * o->h, k * o->h};
        int cx = o->nidx[0][i], cy = o->nidx[1][j], cz = o->is3D ? o->nidx[2][k] : 0;
        for (int kk = kmin; kk < kmax; kk++)
            for (int jj = -2; jj < 2; jj++)
                for (int ii = -2; ii < 2; ii++) {
                    int c = (cx + ii) + (cy + jj) * Ncx + (cz + kk) * Ncx * Ncy;
                    if (c >= Nc || c < 0) continue;
                    int p0 = o->cells[c], np_ = o->ccount[c];
                    for (int mp = p0; mp < p0 + np_; mp++) p2g_pair(o, mp, n, np);
                }
    }
}

/* ------------------------------------------------------------------------------------ */
/* (c) grid: BCs (Grid.cpp:862-1094), periodic fold (Grid.cpp:310-795), nodal solve       */
/*     (Grid.cpp:9-245) with the friction helper (Grid.cpp:247-308)                        */

static void set_vel_component(gyo *o, int n, int ax, double val)
{
    o->v1[3 * n + ax] = val; o->a1[3 * n + ax] = 0.0;
    o->v2[3 * n + ax] = val; o->a2[3 * n + ax] = 0.0;
    o->v0[3 * n + ax] = val; o->a0[3 * n + ax] = 0.0;
}

static void grid_bc(gyo *o)
{
    for (int n = 0; n < o->Nn; n++) {
        const double *val = o->nbcv + 4 * n;
        switch (o->nbct[n]) {
        case BC_GRID_VX: set_vel_component(o, n, 0, val[0]); break;
        case BC_GRID_VY: set_vel_component(o, n, 1, val[0]); break;
        case BC_GRID_VX_VY: set_vel_component(o, n, 0, val[0]); set_vel_component(o, n, 1, val[1]); break;
        case BC_GRID_VZ:
            if (o->prm.fixed_grid_bcs) set_vel_component(o, n, 2, val[0]);
            break;
        case BC_GRID_VX_VZ:
            if (o->prm.fixed_grid_bcs) { set_vel_component(o, n, 0, val[0]); set_vel_component(o, n, 2, val[1]); }
            break;
        case BC_GRID_VY_VZ:
            if (o->prm.fixed_grid_bcs) { set_vel_component(o, n, 1, val[0]); set_vel_component(o, n, 2, val[1]); }
            break;
        case BC_GRID_VX_VY_VZ:
            if (o->prm.fixed_grid_bcs) {
                set_vel_component(o, n, 0, val[0]); set_vel_component(o, n, 1, val[1]);
                set_vel_component(o, n, 2, val[2]);
            }
            break;
        default: break; /* every other node BC has an empty body in the reference */
        }
    }
}

static void fold_pair(gyo *o, int a, int b)
{
    double *sc[] = {o->m0, o->m1, o->m2};
    for (int f = 0; f < 3; f++) { double s = sc[f][a] + sc[f][b]; sc[f][a] = s; sc[f][b] = s; }
    double *vc[] = {o->p0, o->p1, o->p2, o->f0, o->f1, o->f2};
    for (int f = 0; f < 6; f++)
        for (int k = 0; k < 3; k++) {
            double s = vc[f][3 * a + k] + vc[f][3 * b + k];
            vc[f][3 * a + k] = s; vc[f][3 * b + k] = s;
        }
}

static void periodic_fold(gyo *o)
{
    const int Nx = o->Nx, Ny = o->Ny, Nz = o->Nz;
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < Nz; k++)
            for (int j = 0; j < Ny; j++) fold_pair(o, i + j * Nx + k * Nx * Ny, (Nx - 3 + i) + j * Nx + k * Nx * Ny);
    for (int j = 0; j < 3; j++)
        for (int k = 0; k < Nz; k++)
            for (int i = 0; i < Nx; i++) fold_pair(o, i + j * Nx + k * Nx * Ny, i + (Ny - 3 + j) * Nx + k * Nx * Ny);
    if (o->is3D)
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < Ny; j++)
                for (int i = 0; i < Nx; i++) fold_pair(o, i + j * Nx + k * Nx * Ny, i + j * Nx + (Nz - 3 + k) * Nx * Ny);
}

/* calculateColoumbFrictionContactNormals, Grid.cpp:247-308: only contact_normals is used
 * by the caller (the friction outputs are discarded there). */
static void friction_normals(const double *rv, const double *nrm, double mu, double *cn)
{
    double om[3];
    om[0] = rv[1] * nrm[2] - rv[2] * nrm[1];
    om[1] = rv[0] * nrm[2] - rv[2] * nrm[0];
    om[2] = rv[0] * nrm[1] - rv[1] * nrm[0];
    double mag = sqrt(om[0] * om[0] + om[1] * om[1] + om[2] * om[2]) + 0.001;
    om[0] /= mag; om[1] /= mag; om[2] /= mag;
    double mu0 = mag / (rv[0] * nrm[0] + rv[1] * nrm[1] + rv[2] * nrm[2]) + 0.001;
    double on[3];
    on[0] = om[2] * nrm[1] - om[1] * nrm[2];
    on[1] = om[2] * nrm[0] - om[0] * nrm[2];
    on[2] = om[1] * nrm[0] - om[0] * nrm[1];
    if (mu0 < mu) mu = mu0;
    cn[0] = nrm[0] + on[0] * mu;
    cn[1] = nrm[1] + on[1] * mu;
    cn[2] = nrm[2] + on[2] * mu;
}

static void body_update(double m, const double *p, const double *f, double *v, double *a, double dt, int step)
{
    for (int k = 0; k < 3; k++) { v[k] = p[k] / m; a[k] = f[k] / m; }
    for (int k = 0; k < 3; k++) v[k] += (step == 1) ? a[k] * 0.5 * dt : a[k] * dt;
}

static void nodal_solve(gyo *o, int step)
{
    const double dt = o->dt;
#pragma omp parallel for schedule(static)
    for (int n = 0; n < o->Nn; n++) {
        if (o->m0[n] == 0.0) continue;
        double *v0 = o->v0 + 3 * n, *n1 = o->n1 + 3 * n, *n2 = o->n2 + 3 * n;
        for (int k = 0; k < 3; k++) v0[k] = o->p0[3 * n + k] / o->m0[n];
        double mag1 = sqrt(n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2]);
        if (mag1 > 1e-8) { n1[0] /= mag1; n1[1] /= mag1; n1[2] /= mag1; }
        else { n1[0] = n1[1] = n1[2] = 0.0; }
        /* body 2's own normal is overwritten by -n1 (Grid.cpp:45-47) */
        n2[0] = -n1[0]; n2[1] = -n1[1]; n2[2] = -n1[2];
        double m1 = o->m1[n], m2 = o->m2[n];
        const double *p1 = o->p1 + 3 * n, *p2 = o->p2 + 3 * n, *f1 = o->f1 + 3 * n, *f2 = o->f2 + 3 * n;
        double *v1 = o->v1 + 3 * n, *v2 = o->v2 + 3 * n, *a1 = o->a1 + 3 * n, *a2 = o->a2 + 3 * n;
        if (o->body[2 * n + 1] != -1) {
            double ap1 = 0.0, ap2 = 0.0, rv1[3] = {0, 0, 0}, rv2[3] = {0, 0, 0};
            if (m1 != 0.0) {
                for (int k = 0; k < 3; k++) rv1[k] = (p1[k] / m1) - v0[k];
                ap1 = rv1[0] * n1[0] + rv1[1] * n1[1] + rv1[2] * n1[2];
            }
            if (m2 != 0.0) {
                for (int k = 0; k < 3; k++) rv2[k] = (p2[k] / m2) - v0[k];
                ap2 = rv2[0] * n2[0] + rv2[1] * n2[1] + rv2[2] * n2[2];
            }
            if (ap1 > 0.01 || ap2 > 0.01) {
                if (o->rigid[2 * n + 0]) {
                    if (m1 != 0.0) {
                        for (int k = 0; k < 3; k++) v1[k] = p1[k] / m1;
                        if (m2 != 0.0)
                            for (int k = 0; k < 3; k++) v2[k] = p2[k] / m2 - (p2[k] - m2 * v1[k]) / m2;
                    }
                } else if (o->rigid[2 * n + 1]) {
                    if (m2 != 0.0) {
                        for (int k = 0; k < 3; k++) v2[k] = p2[k] / m2;
                        if (m1 != 0.0)
                            for (int k = 0; k < 3; k++) v1[k] = p1[k] / m1 - (p1[k] - m1 * v2[k]) / m1;
                    }
                } else {
                    if (m1 != 0.0) {
                        double cn[3];
                        friction_normals(rv1, n1, o->prm.mu, cn);
                        for (int k = 0; k < 3; k++) {
                            v1[k] = (p1[k] / m1) - ap1 * cn[k];
                            a1[k] = (f1[k] / m1) - (ap1 * cn[k]) / dt;
                        }
                        for (int k = 0; k < 3; k++) v1[k] += (step == 1) ? a1[k] * 0.5 * dt : a1[k] * dt;
                    }
                    if (m2 != 0.0) {
                        double cn[3];
                        friction_normals(rv2, n2, o->prm.mu, cn);
                        for (int k = 0; k < 3; k++) {
                            v2[k] = (p2[k] / m2) - ap2 * cn[k];
                            a2[k] = (f2[k] / m2) - (ap2 * cn[k]) / dt;
                        }
                        for (int k = 0; k < 3; k++) v2[k] += (step == 1) ? a2[k] * 0.5 * dt : a2[k] * dt;
                    }
                }
            } else {
                if (m1 != 0.0) body_update(m1, p1, f1, v1, a1, dt, step);
                if (m2 != 0.0) body_update(m2, p2, f2, v2, a2, dt, step);
            }
        } else {
            if (m1 != 0.0) body_update(m1, p1, f1, v1, a1, dt, step);
        }
    }
}

/* ------------------------------------------------------------------------------------ */
/* (d) G2P, Extrapolation.cpp:127-163 (stencil :649-708) and 288-367                      */

static void g2p(gyo *o)
{
    const int Nx = o->Nx, Ny = o->Ny, Nn = o->Nn;
    const double h = o->h, lp = 0.5 * o->psep, ps2 = o->psep / 2;
#pragma omp parallel for schedule(static)
    for (int mp = 0; mp < o->N; mp++) {
        const double *xp = o->x + 3 * mp;
        o->nrm[3 * mp + 0] = o->nrm[3 * mp + 1] = o->nrm[3 * mp + 2] = 0.0;
        int ix = (int)((xp[0] - ps2 - 0.0) / h);
        int iy = (int)((xp[1] - ps2 - 0.0) / h);
        int iz = o->is3D ? (int)((xp[2] - ps2 - 0.0) / h) : 0;
        int kn = o->is3D ? 3 : 1;
        int ob = o->obj[mp];
        double rho = o->rho[mp];
        double *acc = o->a + 3 * mp, *gv = o->gv + 3 * mp, *er = o->er + 6 * mp, *nr = o->nrm + 3 * mp;
        double *gT = o->gT + 3 * mp;
        gT[0] = gT[1] = gT[2] = 0.0; /* Extrapolation.cpp:132-134 */
        for (int k = 0; k < kn; k++)
            for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++) {
                    int n = (ix + i) + (iy + j) * Nx + (iz + k) * Nx * Ny;
                    if (n >= Nn || n < 0) n = 0; /* out-of-range stencil entries read node 0 */
                    if (o->m0[n] == 0.0) continue;
                    int ni = n % Nx, nj = (n / Nx) % Ny, nk = n / (Nx * Ny);
                    double np[3] = {ni * h, nj * h, nk * h};
                    double sx = gyo_gimp_shape(np[0] - xp[0], h, lp);
                    double sy = gyo_gimp_shape(np[1] - xp[1], h, lp);
                    double sz = gyo_gimp_shape(np[2] - xp[2], h, lp);
                    double gx = gyo_gimp_grad(np[0] - xp[0], h, lp, xp[0]);
                    double gy = gyo_gimp_grad(np[1] - xp[1], h, lp, xp[1]);
                    double gz = gyo_gimp_grad(np[2] - xp[2], h, lp, xp[2]);
                    if (!o->is3D) { sz = 1.0; gz = 0.0; }
                    /* thermal, every node with mass, whatever its bodies (Extrapolation.cpp:358-362) */
                    gT[0] += (gx * sy * sz) * o->Tn[n];
                    gT[1] += (sx * gy * sz) * o->Tn[n];
                    gT[2] += (sx * sy * gz) * o->Tn[n];
                    o->Tr[mp] += sx * sy * sz * o->Rn[n];
                    const double *vb, *ab, *nb;
                    if (o->body[2 * n + 0] == ob) { vb = o->v1 + 3 * n; ab = o->a1 + 3 * n; nb = o->n1 + 3 * n; }
                    else if (o->body[2 * n + 1] == ob) { vb = o->v2 + 3 * n; ab = o->a2 + 3 * n; nb = o->n2 + 3 * n; }
                    else continue; /* a third body sees nothing from this node */
                    double w = sx * sy * sz;
                    o->dr[mp] -= rho * ((gx * sy * sz * vb[0]) + (gy * sz * sx * vb[1]) + (gz * sx * sy * vb[2]));
                    acc[0] += w * ab[0]; acc[1] += w * ab[1]; acc[2] += w * ab[2];
                    gv[0] += w * vb[0]; gv[1] += w * vb[1]; gv[2] += w * vb[2];
                    er[0] += (gx * sy * sz * vb[0]);
                    er[1] += (gy * sx * sz * vb[1]);
                    er[2] += (gz * sx * sy * vb[2]);
                    er[3] += 0.5 * (gx * sy * sz * vb[1] + gy * sx * sz * vb[0]);
                    er[4] += 0.5 * (gy * sx * sz * vb[2] + gz * sx * sy * vb[1]);
                    er[5] += 0.5 * (gx * sy * sz * vb[2] + gz * sx * sy * vb[0]);
                    nr[0] += w * nb[0]; nr[1] += w * nb[1]; nr[2] += w * nb[2];
                }
    }
}

/* ------------------------------------------------------------------------------------ */
/* particle BCs, TimeIntegration.cpp:177-296                                              */

static void particle_bc(gyo *o)
{
    for (int p = 0; p < o->N; p++) {
        const double *val = o->bcv + 4 * p;
        double *v = o->v + 3 * p, *a = o->a + 3 * p, *gv = o->gv + 3 * p, *s = o->s + 6 * p;
        double m = o->m[p];
        switch (o->bct[p]) {
        case BC_MP_VX: v[0] = val[0]; break;
        case BC_MP_VY: v[0] = 0.0; v[1] = val[0]; v[2] = 0.0; break;
        case BC_MP_VZ: v[0] = 0.0; v[1] = 0.0; v[2] = val[0]; break;
        case BC_MP_VX_VY: v[0] = val[0]; v[1] = val[1]; v[2] = 0.0; break;
        case BC_MP_VXSIN: v[0] = val[0] * sin(2.0 * PI_REF * val[1] * o->t); break;
        case BC_MP_VYSIN:
            v[1] = val[0] * sin(2.0 * PI_REF * val[1] * o->t);
            gv[1] = 0.0; a[1] = 0.0;
            break;
        case BC_MP_SYYSIN:
            s[1] = val[0] * sin(2.0 * PI_REF * val[1] * o->t);
            v[0] = v[1] = v[2] = 0.0; gv[0] = gv[1] = gv[2] = 0.0;
            break;
        case BC_MP_FX: a[0] += val[0] / m; break;
        case BC_MP_FY: a[0] = 0.0; a[1] += val[0] / m; break;
        case BC_MP_FZ: a[2] += val[0] / m; break;
        case BC_MP_FX_FY: a[0] += val[0] / m; a[1] += val[1] / m; break;
        case BC_MP_STRESS_XX_YY: s[0] = val[0]; s[1] = val[1]; break;
        default: break;
        }
    }
}

/* ------------------------------------------------------------------------------------ */
/* constitutive models, ConstitutiveModels.cpp                                            */

/* elastic, ConstitutiveModels.cpp:3-30 (1/3 written as 0.3333) */
static void elastic(gyo *o, int mp, const gyo_material *M, double dt)
{
    const double *r = o->er + 6 * mp;
    double *s = o->s + 6 * mp;
    double vol = 0.3333 * (r[0] + r[1] + r[2]);
    double dev[6] = {r[0] - vol, r[1] - vol, r[2] - vol, r[3], r[4], r[5]};
    double G = M->shearMod, K = M->bulkMod;
    s[0] += (2.0 * G * dev[0] + 3.0 * K * vol) * dt;
    s[1] += (2.0 * G * dev[1] + 3.0 * K * vol) * dt;
    s[2] += (2.0 * G * dev[2] + 3.0 * K * vol) * dt;
    s[3] += (2.0 * G * dev[3]) * dt;
    s[4] += (2.0 * G * dev[4]) * dt;
    s[5] += (2.0 * G * dev[5]) * dt;
}

/* Newtonian liquid, ConstitutiveModels.cpp:33-64 (1/3 as 0.33333; viscous term times dt) */
static void newtonian(gyo *o, int mp, const gyo_material *M, double dt, double mu_eff)
{
    const double *r = o->er + 6 * mp, *e = o->e + 6 * mp;
    double *s = o->s + 6 * mp;
    double vol = 0.33333 * (r[0] + r[1] + r[2]);
    double P = M->bulkMod * (e[0] + e[1] + e[2]);
    double dev[6] = {r[0] - vol, r[1] - vol, r[2] - vol, r[3], r[4], r[5]};
    double mu = mu_eff;
    s[0] = P + mu * (2. - (2. / 3.)) * (dev[0]) * dt;
    s[1] = P + mu * (2. - (2. / 3.)) * (dev[1]) * dt;
    s[3] = 2.0 * mu * (dev[3]) * dt;
    if (o->is3D) {
        s[2] = P + mu * (2. - (2. / 3.)) * (dev[2]) * dt;
        s[4] = 2.0 * mu * (dev[4]) * dt;
        s[5] = 2.0 * mu * (dev[5]) * dt;
    }
}

/* turbulent liquid, ConstitutiveModels.cpp:66-126.  The turbulence flag lives in damage;
 * the deviatoric rates are taken before the volumetric part is formed (:77-82), so the
 * normal stresses use the raw normal strain rates. */
static void turbulent(gyo *o, int mp, const gyo_material *M, double dt)
{
    const double *r = o->er + 6 * mp, *v = o->v + 3 * mp, *e = o->e + 6 * mp;
    double *s = o->s + 6 * mp;
    double mu = M->viscosity;
    if (o->D[mp] == 1) mu = M->viscosity / 2.0;
    double KE = 0.5 * o->m[mp] * ((v[0] * v[0]) + (v[1] * v[1]) + (v[2] * v[2]));
    double VE = 0.5 * M->viscosity * (r[3] * r[3] + r[4] * r[4] + r[5] * r[5]);
    double crit = KE - VE - M->turbStress;
    if (crit > 0) o->D[mp] = 1.0;
    if (crit <= 0) { o->D[mp] = 0.0; mu = M->viscosity; }
    double P = M->bulkMod * (e[0] + e[1] + e[2]);
    s[0] = P + mu * (2. - (2. / 3.)) * (r[0]) * dt;
    s[1] = P + mu * (2. - (2. / 3.)) * (r[1]) * dt;
    s[3] = 2.0 * mu * (r[3]) * dt;
    if (o->is3D) {
        s[2] = P + mu * (2. - (2. / 3.)) * (r[2]) * dt;
        s[4] = 2.0 * mu * (r[4]) * dt;
        s[5] = 2.0 * mu * (r[5]) * dt;
    }
}

/* von Mises perfect plasticity, ConstitutiveModels.cpp:131-234 (1/3 as 0.33) */
static void perfect_plastic(gyo *o, int mp, const gyo_material *M, double dt)
{
    const double *r = o->er + 6 * mp;
    double *s = o->s + 6 * mp;
    double G = M->shearMod, K = M->bulkMod, Y = M->yieldStress;
    double vol = 0.33 * (r[0] + r[1] + r[2]);
    double dev[6] = {r[0] - vol, r[1] - vol, r[2] - vol, r[3], r[4], r[5]};
    double tr[6] = {0, 0, 0, 0, 0, 0};
    tr[0] = s[0] + (2 * G * dev[0] + 3 * K * vol) * dt;
    tr[1] = s[1] + (2 * G * dev[1] + 3 * K * vol) * dt;
    if (o->is3D) {
        tr[2] = s[2] + (2 * G * dev[2] + 3 * K * vol) * dt;
        tr[4] = s[4] + (2 * G * dev[4]) * dt;
        tr[5] = s[5] + (2 * G * dev[5]) * dt;
    }
    tr[3] = s[3] + (2 * G * dev[3]) * dt;
    double q = sqrt(0.5 * (tr[0] - tr[1]) * (tr[0] - tr[1]) + 0.5 * (tr[1] - tr[2]) * (tr[1] - tr[2]) +
                    0.5 * (tr[2] - tr[0]) * (tr[2] - tr[0]) + tr[3] * tr[3] + tr[4] * tr[4] + tr[5] * tr[5]);
    if (q > Y) {
        double dL = (q - Y) / (3.0 * G);
        double c = dL * (0.5 / q);
        double pr[6];
        pr[0] = c * (2.0 * tr[0] - tr[1] - tr[2]);
        pr[1] = c * (2.0 * tr[1] - tr[2] - tr[0]);
        pr[2] = c * (2.0 * tr[2] - tr[0] - tr[1]);
        pr[3] = c * (6.0 * tr[3]);
        pr[4] = c * (6.0 * tr[4]);
        pr[5] = c * (6.0 * tr[5]);
        o->eqp[mp] += dt * sqrt(0.5 * (pr[0] - pr[1]) * (pr[0] - pr[1]) + 0.5 * (pr[1] - pr[2]) * (pr[1] - pr[2]) +
                                0.5 * (pr[2] - pr[0]) * (pr[2] - pr[0]) + pr[3] * pr[3] + pr[4] * pr[4] + pr[5] * pr[5]);
        for (int k = 0; k < 6; k++) o->ep[6 * mp + k] += pr[k];
        double el[6];
        for (int k = 0; k < 6; k++) el[k] = r[k] - (pr[k] / dt);
        double d2[6] = {el[0] - vol, el[1] - vol, el[2] - vol, el[3], el[4], el[5]};
        s[0] += (2.0 * G * d2[0] + 3.0 * K * vol) * dt;
        s[1] += (2.0 * G * d2[1] + 3.0 * K * vol) * dt;
        s[3] += (2.0 * G * d2[3]) * dt;
        if (o->is3D) {
            s[2] += (2.0 * G * d2[2] + 3.0 * K * vol) * dt;
            s[4] += (2.0 * G * d2[4]) * dt;
            s[5] += (2.0 * G * d2[5]) * dt;
        }
    } else {
        for (int k = 0; k < 6; k++) s[k] = tr[k];
    }
}

/* Drucker-Prager with linear cohesion softening, ConstitutiveModels.cpp:238-428.  The
 * Newton-Raphson loops are kept as written (tolerance 1e-8, 200-iteration cap). */
static void drucker_prager(gyo *o, int mp, const gyo_material *M, double dt)
{
    const double *r = o->er + 6 * mp;
    double *s = o->s + 6 * mp;
    double G = M->shearMod, K = M->bulkMod, c = M->cohesion;
    double phi = M->phi * PI_REF / 180.0, psi = M->psi * PI_REF / 180.0;
    double ecr = M->criticalStrain;
    int isDamage = M->isDamage;
    double vol = 0.3333 * (r[0] + r[1] + r[2]);
    double dev[6] = {r[0] - vol, r[1] - vol, r[2] - vol, r[3], r[4], r[5]};
    double tr[6];
    tr[0] = s[0] + (2.0 * G * dev[0] + 3.0 * K * vol) * dt;
    tr[1] = s[1] + (2.0 * G * dev[1] + 3.0 * K * vol) * dt;
    tr[2] = s[2] + (2.0 * G * dev[2] + 3.0 * K * vol) * dt;
    tr[3] = s[3] + (2.0 * G * dev[3]) * dt;
    tr[4] = s[4] + (2.0 * G * dev[4]) * dt;
    tr[5] = s[5] + (2.0 * G * dev[5]) * dt;
    double I1 = (1.0 / 3.0) * (tr[0] + tr[1] + tr[2]); /* mean stress */
    double sxx = tr[0] - I1, syy = tr[1] - I1, szz = tr[2] - I1, sxy = tr[3], syz = tr[4], sxz = tr[5];
    double J2 = 0.5 * (sxx * sxx + syy * syy + szz * szz + 2.0 * sxy * sxy + 2.0 * syz * syz + 2.0 * sxz * sxz);
    double eta = 6.0 * sin(phi) / (sqrt(3.0) * (3.0 - sin(phi)));
    double xi = 6.0 * cos(phi) / (sqrt(3.0) * (3.0 - sin(phi)));
    double etab = (phi == psi) ? eta : 6.0 * sin(psi) / (sqrt(3.0) * (3.0 - sin(psi)));
    double F = sqrt(J2) + eta * I1 - xi * c;
    int yield = isDamage ? (F > 0.0 && I1 < 0.0) : (F > 0.0);
    if (!yield) {
        for (int k = 0; k < 6; k++) s[k] = tr[k];
        return;
    }
    int it = 0;
    double err = 1.0, dL = 0.0, dLn = 10.0;
    double eq = o->eqp[mp];
    while (err > 1e-8) {
        it++;
        double cv = c - (eq + (xi * dL)) * (c / ecr);
        double dc = -c / ecr;
        if (cv < c / 10.0) { cv = c / 10.0; dc = 0.0; }
        double Fp = sqrt(J2) - G * dL + eta * (I1 - etab * K * dL) - xi * cv;
        double dFp = -G - K * eta * etab - xi * xi * dc;
        dLn = dL - (Fp / dFp);
        err = fabs(Fp / cv);
        dL = dLn;
        if (it > 200) break;
    }
    double Gapex = sqrt(J2) - G * dL;
    if (Gapex < 0.0 && !isDamage) {
        it = 0;
        err = 1.0;
        double de = 0.0;
        while (err > 1e-8) {
            it++;
            double cv = c - (eq + ((xi / eta) * de)) * (c / ecr);
            double dc = -c / ecr;
            if (cv < c / 10.0) { cv = c / 10.0; dc = 0.0; }
            double Gp = cv * (xi / etab) - I1 + K * de;
            double dGp = (xi / eta) * dc * (xi / etab) + K;
            de = de - (Gp / dGp);
            err = fabs(Gp / cv);
            if (it > 200) break;
        }
        if (de < 0.0) {
            de = 0.0;
        } else {
            s[0] = I1 - K * de; s[1] = I1 - K * de; s[3] = 0.0;
            s[2] = I1 - K * de; s[4] = 0.0; s[5] = 0.0;
            o->eqp[mp] += de * (xi / eta);
            o->ep[6 * mp + 0] += de * (etab / 3.0);
            o->ep[6 * mp + 1] += de * (etab / 3.0);
            o->ep[6 * mp + 2] += de * (etab / 3.0);
        }
    } else {
        double f = (1.0 - (G * dL / sqrt(J2)));
        double pm = (I1 - K * etab * dL);
        s[0] = f * sxx + pm; s[1] = f * syy + pm; s[3] = f * sxy;
        s[2] = f * szz + pm; s[4] = f * syz; s[5] = f * sxz;
        o->eqp[mp] += dL * xi;
        o->ep[6 * mp + 0] += dL * ((0.5 / J2) * sxx + etab / 3.0);
        o->ep[6 * mp + 1] += dL * ((0.5 / J2) * syy + etab / 3.0);
        o->ep[6 * mp + 2] += dL * ((0.5 / J2) * szz + etab / 3.0);
        o->ep[6 * mp + 3] += dL * (0.5 / J2) * sxy;
        o->ep[6 * mp + 4] += dL * (0.5 / J2) * syz;
        o->ep[6 * mp + 5] += dL * (0.5 / J2) * sxz;
    }
}

/* ------------------------------------------------------------------------------------ */
/* symmetric 3x3 eigen-solve (cyclic Jacobi); stands in for eig3.cpp:258-267              */

int gyo_sym_eigen(const double *a9, double *V9, double *d3)
{
    double A[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) A[i][j] = a9[3 * i + j];
    int sweep;
    for (sweep = 0; sweep < 64; sweep++) {
        double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
        double diag = fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]);
        if (off == 0.0 || off <= 1e-300 || off < 1e-18 * diag) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                double apq = A[p][q];
                if (apq == 0.0) continue;
                double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; k++) { /* A <- A J */
                    double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - s * akq;
                    A[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) { /* A <- J^T A */
                    double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - s * aqk;
                    A[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; k++) {
                    double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
    }
    /* ascending eigenvalues, eigenvectors in columns (the reference's output convention) */
    int idx[3] = {0, 1, 2};
    for (int i = 0; i < 2; i++)
        for (int j = i + 1; j < 3; j++)
            if (A[idx[j]][idx[j]] < A[idx[i]][idx[i]]) { int t = idx[i]; idx[i] = idx[j]; idx[j] = t; }
    for (int c = 0; c < 3; c++) {
        d3[c] = A[idx[c]][idx[c]];
        for (int r = 0; r < 3; r++) V9[3 * r + c] = V[r][idx[c]];
    }
    return sweep;
}

/* Grady-Kipp damage, DamageModels.cpp:3-152 */
static void grady_kipp(gyo *o, int mp, const gyo_material *M, double dt)
{
    double Cg = M->Cg, mm = M->damageM, k = M->damageK, G = M->shearMod, K = M->bulkMod;
    double *s6 = o->s + 6 * mp;
    double alpha = (8.0 * PI_REF * Cg * Cg * Cg * k) / (((mm + 1.0) * (mm + 2.0) * (mm + 3.0)));
    if (!o->is3D) {
        double st[4] = {s6[0], s6[1], s6[3], s6[2]};
        double th;
        if (fabs(st[0] - st[1]) < 1e-5) th = PI_REF / 4.0;
        else th = 0.5 * atan(2.0 * st[2] / (st[0] - st[1]));
        double c = cos(th), s = sin(th);
        double s1 = st[0] * c * c + st[1] * s * s + 2.0 * c * s * st[2];
        double s2 = st[0] * s * s + st[1] * c * c - 2.0 * c * s * st[2];
        double smx = s1 > s2 ? s1 : s2;
        if (smx < 0.0) smx = 0.0;
        o->smax[mp] = smx;
        if (smx > 1e-3) {
            double eff = smx / (K + (4.0 * G / 3.0));
            double vol = o->m[mp] / o->rho[mp];
            double emin = o->flaw[mp] * pow(vol * k, -1.0 / mm);
            if (eff > emin) {
                double rate = ((mm + 3.0) / 3.0) * pow(alpha, 1.0 / 3.0) * pow(eff, mm / 3.0);
                o->D[mp] = pow(pow(o->D[mp], 1.0 / 3.0) + (dt * rate), 3.0);
                if (o->D[mp] > 1.0) o->D[mp] = 1.0;
                if (s1 > 0.0) s1 = (1.0 - o->D[mp]) * s1;
                if (s2 > 0.0) s2 = (1.0 - o->D[mp]) * s2;
                st[0] = s1 * c * c + s2 * s * s;
                st[1] = s1 * s * s + s2 * c * c;
                st[2] = (s1 - s2) * c * s;
                st[3] = 0.0;
            }
        }
        if (o->D[mp] == 1.0) {
            if (s1 > 0.0) s1 = (1.0 - o->D[mp]) * s1;
            if (s2 > 0.0) s2 = (1.0 - o->D[mp]) * s2;
            st[0] = s1 * c * c + s2 * s * s;
            st[1] = s1 * s * s + s2 * c * c;
            st[2] = (s1 - s2) * c * s;
            st[3] = 0.0;
        }
        s6[0] = st[0]; s6[1] = st[1]; s6[2] = st[3]; s6[3] = st[2];
        return;
    }
    double A[9] = {s6[0], s6[3], s6[5], s6[3], s6[1], s6[4], s6[5], s6[4], s6[2]};
    /* the gate is a signed component sum, not a norm (DamageModels.cpp:82) */
    double chk = fabs(A[0] + A[4] + A[8] + A[1] + A[5] + A[2]);
    if (!(chk > 1e-3)) return;
    double Vv[9], d[3];
    gyo_sym_eigen(A, Vv, d);
    double s1 = d[0], s2 = d[1], s3 = d[2];
    double smx = s3 > 0.0 ? s3 : 0.0;
    if (s2 > smx) smx = s2;
    if (s1 > smx) smx = s1;
    o->smax[mp] = smx;
    if (smx > 1e-3) {
        double eff = smx / (K + 4.0 * G / 3.0);
        double vol = o->m[mp] / o->rho[mp];
        double emin = o->flaw[mp] * pow(vol * k, -1.0 / mm);
        if (eff > emin) {
            double rate = ((mm + 3.0) / 3.0) * pow(alpha, 1.0 / 3.0) * pow(eff, mm / 3.0);
            o->D[mp] = pow(pow(o->D[mp], 1.0 / 3.0) + (dt * rate), 3.0);
            if (o->D[mp] > 1.0) o->D[mp] = 1.0;
            if (s1 > 0.0) s1 = (1.0 - o->D[mp]) * s1;
            if (s2 > 0.0) s2 = (1.0 - o->D[mp]) * s2;
            if (s3 > 0.0) s3 = (1.0 - o->D[mp]) * s3;
        }
    }
    /* stress rebuilt from the principal values: V diag(s) V^T (DamageModels.cpp:124-148) */
    double dg[3] = {s1, s2, s3};
    double T[3][3], R[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) T[i][j] = dg[i] * Vv[3 * j + i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) R[i][j] = Vv[3 * i + 0] * T[0][j] + Vv[3 * i + 1] * T[1][j] + Vv[3 * i + 2] * T[2][j];
    s6[0] = R[0][0]; s6[1] = R[1][1]; s6[2] = R[2][2];
    s6[3] = R[0][1]; s6[4] = R[1][2]; s6[5] = R[0][2];
}

/* ------------------------------------------------------------------------------------ */
/* particle update, TimeIntegration.cpp:11-117, with dispatch :120-143 and :165-173       */

static void update_particles(gyo *o)
{
    const double dt = o->dt, h = o->h;
    const int Ncx = o->Nx - 1, Ncy = o->Ny - 1;
    const double Lx = o->L[0] - 2 * h, Ly = o->L[1] - 2 * h, Lz = o->L[2] - 2 * h;
#pragma omp parallel for schedule(static)
    for (int p = 0; p < o->N; p++) {
        double *x = o->x + 3 * p, *v = o->v + 3 * p;
        o->rho[p] += o->dr[p] * dt;
        o->V[p] = o->m[p] / o->rho[p];
        double c = o->prm.damping;
        if (!o->hold[p]) {
            v[0] = v[0] + (o->a[3 * p + 0] - c * v[0]) * dt;
            v[1] = v[1] + (o->a[3 * p + 1] - c * v[1]) * dt;
            if (o->is3D) v[2] = v[2] + (o->a[3 * p + 2] - c * v[2]) * dt;
            x[0] += o->gv[3 * p + 0] * dt;
            x[1] += o->gv[3 * p + 1] * dt;
            if (o->is3D) x[2] += o->gv[3 * p + 2] * dt;
        }
        for (int k = 0; k < 3; k++) o->u[3 * p + k] = x[k] - o->x0[3 * p + k];
        o->T[p] += o->Tr[p] * dt; /* TimeIntegration.cpp:49-50 */
        for (int k = 0; k < 6; k++) o->e[6 * p + k] += o->er[6 * p + k] * dt;
        const gyo_material *M = &o->mats[o->mat[p]];
        if (!M->isRigid) {
            switch (M->model) {
            case 1: elastic(o, p, M, dt); break;
            case 2: newtonian(o, p, M, dt, M->viscosity); break;
            case 3: perfect_plastic(o, p, M, dt); break;
            case 4: drucker_prager(o, p, M, dt); break;
            case 5: turbulent(o, p, M, dt); break;
            default: break;
            }
            if (M->isDamage && M->damageModel == 1) grady_kipp(o, p, M, dt);
        }
        /* periodic wrap with period L - 2h (TimeIntegration.cpp:80-108) */
        if (x[0] > Lx) x[0] = 1.0 * h + fmod((x[0] + Lx), Lx);
        if (x[0] < 1 * h) x[0] += Lx - 1.0 * h;
        if (x[1] > Ly) x[1] = 1.0 * h + fmod((x[1] + Ly), Ly);
        if (x[1] < 1 * h) x[1] += Ly - 1.0 * h;
        if (o->is3D) {
            if (x[2] > Lz) x[2] = 1.0 * h + fmod((x[2] + Lz), Lz);
            if (x[2] < 1 * h) x[2] += Lz - 1.0 * h;
        }
        /* binning key with the quarter-cell shift (TimeIntegration.cpp:110-115) */
        int idx = (int)((x[0] - 0.0 - 0.25 * h) / h);
        int idy = (int)((x[1] - 0.0 - 0.25 * h) / h);
        int idz = (int)((x[2] - 0.0 - 0.25 * h) / h);
        o->cell[p] = idx + idy * Ncx + idz * Ncx * Ncy;
    }
}

/* ------------------------------------------------------------------------------------ */
/* iterate_CPU, Solver.cpp:86-292                                                         */

int gyo_step(gyo *o, double t, int step)
{
    if (o->bad) return -1;
    if ((step % 10 == 0) || (step == 1)) {
        sort_particles(o);
        if (o->bad) return -1;
    }
    reset_nodes(o);
    reset_rates(o);
    p2g(o);
    grid_bc(o);        /* phase 1 */
    periodic_fold(o);
    nodal_solve(o, step);
    grid_bc(o);        /* phase 2 */
    g2p(o);
    grid_bc(o);        /* phase 3: node fields only */
    particle_bc(o);    /* phase 4 */
    update_particles(o);
    particle_bc(o);    /* phase 5 */
    o->t = t;
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* field access                                                                           */

int gyo_num_particles(const gyo *o) { return o->N; }
int gyo_num_nodes(const gyo *o) { return o->Nn; }
void gyo_dims(const gyo *o, int *nxyz) { nxyz[0] = o->Nx; nxyz[1] = o->Ny; nxyz[2] = o->Nz; }

static const int pwidth[GYO_P_NFIELDS] = {3, 3, 3, 3, 3, 3, 6, 6, 6, 6, 1, 1, 1, 1, 1, 1, 3, 1, 1, 3};
int gyo_particle_width(int f) { return (f >= 0 && f < GYO_P_NFIELDS) ? pwidth[f] : 0; }
int gyo_node_width(int f)
{
    switch (f) {
    case GYO_N_MASS: case GYO_N_MASS1: case GYO_N_MASS2: case GYO_N_TEMP: case GYO_N_TEMPRATE: return 1;
    default: return (f > GYO_N_MASS2 && f <= GYO_N_NORMAL2) ? 3 : 0;
    }
}

int gyo_get_particle_field(const gyo *o, int f, double *out)
{
    const double *src[GYO_P_NFIELDS] = {o->x, o->x0, o->u, o->v, o->gv, o->a, o->er, o->s, o->e, o->ep,
                                        o->eqp, o->D, o->smax, o->m, o->rho, o->V, o->nrm, o->dr,
                                        o->T, o->gT};
    int w = gyo_particle_width(f);
    if (!w) return -1;
    memcpy(out, src[f], sizeof(double) * (size_t)w * (size_t)o->N);
    return 0;
}

int gyo_get_particle_ifield(const gyo *o, int f, int *out)
{
    const int *src = f == GYO_PI_CELL ? o->cell : f == GYO_PI_MAT ? o->mat : f == GYO_PI_OBJ ? o->obj : f == GYO_PI_PID ? o->pid : NULL;
    if (!src) return -1;
    memcpy(out, src, sizeof(int) * (size_t)o->N);
    return 0;
}

int gyo_get_node_field(const gyo *o, int f, double *out)
{
    const double *src[] = {o->m0, o->m1, o->m2, o->p0, o->p1, o->p2, o->f0, o->f1, o->f2,
                           o->v0, o->v1, o->v2, o->a1, o->a2, o->n1, o->n2, o->Tn, o->Rn};
    int w = gyo_node_width(f);
    if (!w) return -1;
    memcpy(out, src[f], sizeof(double) * (size_t)w * (size_t)o->Nn);
    return 0;
}

int gyo_get_node_ifield(const gyo *o, int f, int *out)
{
    size_t Nn = (size_t)o->Nn;
    switch (f) {
    case GYO_NI_BODY: memcpy(out, o->body, sizeof(int) * 2 * Nn); return 0;
    case GYO_NI_RIGID: for (size_t i = 0; i < 2 * Nn; i++) out[i] = o->rigid[i]; return 0;
    case GYO_NI_CELLS: memcpy(out, o->cells, sizeof(int) * Nn); return 0;
    case GYO_NI_CELLCOUNT: memcpy(out, o->ccount, sizeof(int) * Nn); return 0;
    default: return -1;
    }
}
