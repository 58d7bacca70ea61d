/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A C-ABI driver around the reference's own classes and free functions, compiled together
 * with the unmodified reference sources into oracle/_ref/libgyref.so by oracle/Makefile.
 * It pins the FP64 restatement in gy_oracle.c against the reference itself and times the
 * reference step as the CPU baseline.  The entry points mirror gy_oracle.h (prefix gyr_).
 *
 * Two step modes:
 *   literal (mode 0)  Solver::iterate_CPU as shipped (Solver.cpp:86-292), std::sort included.
 *   harness (mode 1)  the same phase sequence composed from the reference's free functions,
 *                     with the sort replaced by a (cellID, particle id) counting sort and,
 *                     when fixed_grid_bcs is set, working grid_vz / vx_vz / vy_vz / vx_vy_vz
 *                     BCs applied right after each enforceGridBC call.
 */
#include "Solver.hpp"
#include "Extrapolation.hpp"
#include "Grid.hpp"
#include "TimeIntegration.hpp"

#include <algorithm>
#include <cstring>
#include <vector>

#include "gy_oracle.h"

static int pwidth(int f)
{
    static const int w[GYO_P_NFIELDS] = {3, 3, 3, 3, 3, 3, 6, 6, 6, 6, 1, 1, 1, 1, 1, 1, 3, 1, 1, 3};
    return (f >= 0 && f < GYO_P_NFIELDS) ? w[f] : 0;
}
static int nwidth(int f)
{
    return (f == GYO_N_MASS || f == GYO_N_MASS1 || f == GYO_N_MASS2 || f == GYO_N_TEMP || f == GYO_N_TEMPRATE) ? 1 : 3;
}

struct gyr {
    Nodes *nds;
    MaterialPoints *mpts;
    Parameters *prm;
    Solver *solver;
    std::vector<int> pid;
    int fixed_grid_bcs;
};

/* the permutation applied to every array sortParticlesByCellID_CPU moves
 * (Extrapolation.cpp:406-491), in the reference's own containers */
template <class V> static void permute(V &a, const std::vector<int> &order, int w)
{
    V t(a.size());
    for (size_t i = 0; i < order.size(); i++)
        for (int k = 0; k < w; k++) t[i * w + k] = a[(size_t)order[i] * w + k];
    for (size_t i = order.size() * w; i < a.size(); i++) t[i] = a[i];
    a.swap(t);
}

extern "C" {

gyr *gyr_create(double Lx, double Ly, double Lz, double h, double psep)
{
    std::vector<double> L = {Lx, Ly, Lz};
    gyr *r = new gyr();
    r->nds = new Nodes(L, h);
    r->mpts = new MaterialPoints(r->nds);
    r->mpts->psep = psep;
    r->prm = nullptr;
    r->solver = nullptr;
    r->fixed_grid_bcs = 0;
    return r;
}

void gyr_destroy(gyr *r)
{
    if (!r) return;
    delete r->solver;
    delete r->prm;
    delete r->mpts;
    /* Nodes arrays are allocated with new[] and never released by the reference */
    delete r->nds;
    delete r;
}

int gyr_add_particles(gyr *r, int n, const double *pos, const int *mat, const int *obj)
{
    int base = r->mpts->numParticles;
    for (int q = 0; q < n; q++) r->mpts->add(base + q, pos[3 * q + 0], pos[3 * q + 1], pos[3 * q + 2]);
    r->mpts->numParticles = base + n;
    for (int q = 0; q < n; q++) {
        int p = base + q;
        r->mpts->material[p] = mat ? mat[q] : 0;
        r->mpts->materialtemp[p] = r->mpts->material[p];
        r->mpts->objID[p] = obj ? obj[q] : 0;
        r->mpts->objIDtemp[p] = r->mpts->objID[p];
        r->pid.push_back(p);
    }
    return r->mpts->numParticles;
}

void gyr_set_particle_vel(gyr *r, int p, double vx, double vy, double vz) { r->mpts->setVel(p, vx, vy, vz); }
void gyr_set_particle_temps(gyr *r, int count, const int *ids, const double *T)
{
    std::vector<int> at(r->pid.size());
    for (size_t q = 0; q < r->pid.size(); q++) at[r->pid[q]] = (int)q;
    for (int q = 0; q < count; q++)
        if (ids[q] >= 0 && ids[q] < (int)at.size()) r->mpts->setTemp(at[ids[q]], T[q]);
}
void gyr_set_particle_stress(gyr *r, int p, const double *s)
{
    r->mpts->setStress(p, s[0], s[1], s[2], s[3], s[4], s[5]);
}
void gyr_set_particle_damage(gyr *r, int p, double D) { r->mpts->setDamage(p, D); }
void gyr_hold_particle(gyr *r, int p) { r->mpts->holdParticle(p); }
void gyr_set_particle_bc(gyr *r, int p, int type, const double *val, int nval)
{
    r->mpts->setBC(p, (BCTypes::function)type, std::vector<double>(val, val + nval));
}
void gyr_set_node_bc(gyr *r, int n, int type, const double *val, int nval)
{
    r->nds->setBC(n, (BCTypes::function)type, std::vector<double>(val, val + nval));
}

int gyr_init_solver(gyr *r, const gyo_params *p, int nmat, const gyo_material *mats)
{
    r->prm = new Parameters(p->tmax, p->is3D != 0);
    r->prm->setGravity(p->gravity[0], p->gravity[1], p->gravity[2]);
    r->prm->setDampingCoef(p->damping);
    r->prm->setCFL(p->CFL);
    r->prm->setFriction(p->mu);
    r->prm->dt = 0.0;
    r->fixed_grid_bcs = p->fixed_grid_bcs;
    std::vector<MaterialModels> mv;
    for (int i = 0; i < nmat; i++) {
        MaterialModels m;
        const gyo_material &g = mats[i];
        m.setBulkMod(g.bulkMod); m.setShearMod(g.shearMod); m.setDensity(g.density);
        m.setIsRigid(g.isRigid != 0); m.setViscosity(g.viscosity);
        m.setThermalConductivity(g.thermalConductivity); m.setSpecificHeatCapacity(g.specificHeatCapacity);
        m.setYieldStress(g.yieldStress); m.setCohesion(g.cohesion); m.setCriticalStrain(g.criticalStrain);
        m.setFrictionAngle(g.phi); m.setDilatancyAngle(g.psi); m.setIsDamage(g.isDamage != 0);
        m.setDamageModel(g.damageModel); m.setCrackSpeed(g.Cg); m.setDamageM(g.damageM);
        m.setDamageK(g.damageK); m.setTurbulentStress(g.turbStress); m.setModel(g.model);
        mv.push_back(m);
    }
    r->solver = new Solver(r->nds, r->mpts, r->prm, mv);
    return 0;
}

double gyr_get_dt(const gyr *r) { return r->solver->dt; }
void gyr_set_dt(gyr *r, double dt) { r->solver->setDt(dt); }
void gyr_set_params(gyr *r, const gyo_params *p)
{
    r->prm->setGravity(p->gravity[0], p->gravity[1], p->gravity[2]);
    r->prm->setDampingCoef(p->damping);
    r->prm->setCFL(p->CFL);
    r->prm->setFriction(p->mu);
    r->fixed_grid_bcs = p->fixed_grid_bcs;
}

static void harness_sort(gyr *r)
{
    MaterialPoints *m = r->mpts;
    Nodes *nds = r->nds;
    int N = m->numParticles;
    int Ncx = nds->Nx - 1, Ncy = nds->Ny - 1, Ncz = r->prm->is3D ? nds->Nz - 1 : 1;
    int Nc = Ncx * Ncy * Ncz;
    for (int g = 0; g < Nc; g++) nds->cell_pcount[g] = 0;
    for (int p = 0; p < N; p++)
        if (m->cellID[p] >= 0) nds->cell_pcount[m->cellID[p]]++;
    std::vector<int> order(N);
    for (int p = 0; p < N; p++) order[p] = p;
    const std::vector<int> &pid = r->pid;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (m->cellID[a] != m->cellID[b]) return m->cellID[a] < m->cellID[b];
        return pid[a] < pid[b];
    });
    permute(m->position, order, 3); permute(m->pos0, order, 3); permute(m->displacement, order, 3);
    permute(m->velocity, order, 3); permute(m->Gvelocity, order, 3); permute(m->stress, order, 6);
    permute(m->strain, order, 6); permute(m->plastic_strain, order, 6); permute(m->acc_plastic_strain, order, 1);
    permute(m->damage, order, 1); permute(m->smax, order, 1); permute(m->mass, order, 1);
    permute(m->density, order, 1); permute(m->objID, order, 1); permute(m->volume, order, 1);
    permute(m->normals, order, 3); permute(m->temperature, order, 1); permute(m->BCVAL, order, 4);
    permute(m->temperatureGrad, order, 3);  /* with its particle (the reference's sort garbles it) */
    permute(m->material, order, 1); permute(m->cellID, order, 1); permute(m->hold, order, 1);
    permute(m->BCTYPE, order, 1); permute(r->pid, order, 1);
    int cur = 0;
    nds->cells[0] = 0;
    for (int i = 1; i < Nc; i++) {
        cur += nds->cell_pcount[i - 1];
        nds->cells[i] = cur;
    }
}

/* working z-velocity node BCs for harness mode (the reference bodies are empty) */
static void fixed_z_bcs(gyr *r)
{
    Nodes *nds = r->nds;
    for (int n = 0; n < nds->numNodes; n++) {
        int t = nds->BCTYPE[n];
        const double *val = nds->BCVAL + 4 * n;
        auto setc = [&](int ax, double v) {
            nds->velocity_body1[3 * n + ax] = v; nds->acceleration_body1[3 * n + ax] = 0.0;
            nds->velocity_body2[3 * n + ax] = v; nds->acceleration_body2[3 * n + ax] = 0.0;
            nds->velocity[3 * n + ax] = v; nds->acceleration[3 * n + ax] = 0.0;
        };
        if (t == BCTypes::grid_vz) setc(2, val[0]);
        else if (t == BCTypes::grid_vx_vz) { setc(0, val[0]); setc(2, val[1]); }
        else if (t == BCTypes::grid_vy_vz) { setc(1, val[0]); setc(2, val[1]); }
        else if (t == BCTypes::grid_vx_vy_vz) { setc(0, val[0]); setc(1, val[1]); setc(2, val[2]); }
    }
}

int gyr_step(gyr *r, double t, int step, int mode)
{
    MaterialPoints *mpts = r->mpts;
    Nodes *nds = r->nds;
    Parameters *P = r->prm;
    Solver *S = r->solver;
    if (mode == 0) {
        bool sorts = (step % 10 == 0) || (step == 1);
        S->iterate_CPU(t, step, P);
        if (sorts) {
            std::vector<int> np(mpts->numParticles);
            for (int i = 0; i < mpts->numParticles; i++) np[i] = r->pid[mpts->pidx[i]];
            r->pid.swap(np);
        }
        return 0;
    }
    if ((step % 10 == 0) || (step == 1)) harness_sort(r);
#pragma omp parallel for
    for (int n = 0; n < nds->numNodes; n++) resetNode(nds, n);
#pragma omp parallel for
    for (int p = 0; p < mpts->numParticles; p++) resetMaterialPointRates(mpts, p);
#pragma omp parallel for schedule(dynamic, 64)
    for (int n = 0; n < nds->numNodes; n++) extrapToNodes(P, mpts, nds, &S->materials, n);
    for (int n = 0; n < nds->numNodes; n++) enforceGridBC(nds, 1, n);
    if (r->fixed_grid_bcs) fixed_z_bcs(r);
    collectPeriodicContributions(P, nds);
#pragma omp parallel for
    for (int n = 0; n < nds->numNodes; n++) solveNodalEquations(P, nds, S->dt, step, n);
    for (int n = 0; n < nds->numNodes; n++) enforceGridBC(nds, 2, n);
    if (r->fixed_grid_bcs) fixed_z_bcs(r);
#pragma omp parallel for
    for (int p = 0; p < mpts->numParticles; p++) extrapToMatPoints(P, mpts, nds, &S->materials, p);
    for (int n = 0; n < nds->numNodes; n++) enforceGridBC(nds, 3, n);
    if (r->fixed_grid_bcs) fixed_z_bcs(r);
    for (int p = 0; p < mpts->numParticles; p++) enforceMatPointBC(mpts, 4, p);
#pragma omp parallel for
    for (int p = 0; p < mpts->numParticles; p++) updateMatPoint(P, mpts, nds, S->dt, &S->materials, p);
    for (int p = 0; p < mpts->numParticles; p++) enforceMatPointBC(mpts, 5, p);
    nds->t = t;
    mpts->t = t;
    return 0;
}

int gyr_num_particles(const gyr *r) { return r->mpts->numParticles; }
int gyr_num_nodes(const gyr *r) { return r->nds->numNodes; }
void gyr_dims(const gyr *r, int *nxyz) { nxyz[0] = r->nds->Nx; nxyz[1] = r->nds->Ny; nxyz[2] = r->nds->Nz; }

int gyr_get_particle_field(const gyr *r, int f, double *out)
{
    MaterialPoints *m = r->mpts;
    int N = m->numParticles;
    const double *src = nullptr;
    int w = pwidth(f);
    switch (f) {
    case GYO_P_POS: src = m->position.data(); break;
    case GYO_P_POS0: src = m->pos0.data(); break;
    case GYO_P_DISP: src = m->displacement.data(); break;
    case GYO_P_VEL: src = m->velocity.data(); break;
    case GYO_P_GVEL: src = m->Gvelocity.data(); break;
    case GYO_P_ACC: src = m->acceleration.data(); break;
    case GYO_P_STRAINRATE: src = m->strainRate.data(); break;
    case GYO_P_STRESS: src = m->stress.data(); break;
    case GYO_P_STRAIN: src = m->strain.data(); break;
    case GYO_P_PSTRAIN: src = m->plastic_strain.data(); break;
    case GYO_P_EQPS: src = m->acc_plastic_strain.data(); break;
    case GYO_P_DAMAGE: src = m->damage.data(); break;
    case GYO_P_SMAX: src = m->smax.data(); break;
    case GYO_P_MASS: src = m->mass.data(); break;
    case GYO_P_DENSITY: src = m->density.data(); break;
    case GYO_P_VOLUME: src = m->volume.data(); break;
    case GYO_P_NORMALS: src = m->normals.data(); break;
    case GYO_P_DENSITYRATE: src = m->densityRate.data(); break;
    case GYO_P_TEMP: src = m->temperature.data(); break;
    case GYO_P_TEMPGRAD: src = m->temperatureGrad.data(); break;
    default: return -1;
    }
    std::memcpy(out, src, sizeof(double) * (size_t)w * (size_t)N);
    return 0;
}

int gyr_get_particle_ifield(const gyr *r, int f, int *out)
{
    MaterialPoints *m = r->mpts;
    int N = m->numParticles;
    const int *src = nullptr;
    switch (f) {
    case GYO_PI_CELL: src = m->cellID.data(); break;
    case GYO_PI_MAT: src = m->material.data(); break;
    case GYO_PI_OBJ: src = m->objID.data(); break;
    case GYO_PI_PID: src = r->pid.data(); break;
    default: return -1;
    }
    std::memcpy(out, src, sizeof(int) * (size_t)N);
    return 0;
}

int gyr_get_node_field(const gyr *r, int f, double *out)
{
    Nodes *n = r->nds;
    const double *src = nullptr;
    switch (f) {
    case GYO_N_MASS: src = n->mass; break;
    case GYO_N_MASS1: src = n->mass_body1; break;
    case GYO_N_MASS2: src = n->mass_body2; break;
    case GYO_N_MOM: src = n->momentum; break;
    case GYO_N_MOM1: src = n->momentum_body1; break;
    case GYO_N_MOM2: src = n->momentum_body2; break;
    case GYO_N_FORCE: src = n->force; break;
    case GYO_N_FORCE1: src = n->force_body1; break;
    case GYO_N_FORCE2: src = n->force_body2; break;
    case GYO_N_VEL: src = n->velocity; break;
    case GYO_N_VEL1: src = n->velocity_body1; break;
    case GYO_N_VEL2: src = n->velocity_body2; break;
    case GYO_N_ACC1: src = n->acceleration_body1; break;
    case GYO_N_ACC2: src = n->acceleration_body2; break;
    case GYO_N_NORMAL1: src = n->normals_body1; break;
    case GYO_N_NORMAL2: src = n->normals_body2; break;
    case GYO_N_TEMP: src = n->temperature; break;
    case GYO_N_TEMPRATE: src = n->temperatureRate; break;
    default: return -1;
    }
    std::memcpy(out, src, sizeof(double) * (size_t)nwidth(f) * (size_t)n->numNodes);
    return 0;
}

int gyr_get_node_ifield(const gyr *r, int f, int *out)
{
    Nodes *n = r->nds;
    size_t Nn = (size_t)n->numNodes;
    switch (f) {
    case GYO_NI_BODY: std::memcpy(out, n->bodyID, sizeof(int) * 2 * Nn); return 0;
    case GYO_NI_RIGID: for (size_t i = 0; i < 2 * Nn; i++) out[i] = n->hasRigid[i] ? 1 : 0; return 0;
    case GYO_NI_CELLS: std::memcpy(out, n->cells, sizeof(int) * Nn); return 0;
    case GYO_NI_CELLCOUNT: std::memcpy(out, n->cell_pcount, sizeof(int) * Nn); return 0;
    default: return -1;
    }
}

} /* extern "C" */
