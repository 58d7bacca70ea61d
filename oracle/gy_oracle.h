/*
 * gy_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU oracle for Graphyt's explicit GIMP MPM step: an FP64 restatement, written from
 * scratch, of Solver::iterate_CPU (Solver.cpp:86-292) and every function it calls.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load this
 * library.  It checks results and is never the product: the GPU path does not link it.
 */
#ifndef GY_ORACLE_H
#define GY_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* One material, field for field the MaterialModels class (MaterialModels.hpp:29-47).
 * The layout is mirrored by ctypes in oracle/oracle.py. */
typedef struct gyo_material {
    double bulkMod, shearMod, density, viscosity, thermalConductivity, specificHeatCapacity;
    double yieldStress, cohesion, criticalStrain, phi, psi, Cg, damageM, damageK, turbStress;
    int isRigid, isDamage, damageModel, model;
} gyo_material;

/* Global parameters (Parameters.hpp:25-31) plus one oracle switch:
 * fixed_grid_bcs = 1 makes grid_vz / grid_vx_vz / grid_vy_vz / grid_vx_vy_vz act on the
 * nodes (in the reference they dispatch to empty bodies, Grid.cpp:872-873, 1032-1052). */
typedef struct gyo_params {
    double gravity[3];
    double damping;
    double mu;
    double CFL;
    double tmax;
    int is3D;
    int fixed_grid_bcs;
} gyo_params;

typedef struct gyo gyo;

/* Nodes(L, cellsize) (Nodes.cpp:8-141).  Returns NULL when Nx*Ny*Nz != numNodes. */
gyo *gyo_create(double Lx, double Ly, double Lz, double cellsize, double psep);
void gyo_destroy(gyo *o);

/* MaterialPoints::add for n particles (MaterialPoints.cpp:95-235) followed by the
 * material / objectID int fields (MaterialPoints.cpp:32-54). */
int gyo_add_particles(gyo *o, int n, const double *pos3, const int *mat, const int *obj);

/* Per-particle setters (MaterialPoints.cpp:88-93, 302-340) and Nodes::setBC (Nodes.cpp:155-163). */
void gyo_set_particle_vel(gyo *o, int p, double vx, double vy, double vz);
void gyo_set_particle_stress(gyo *o, int p, const double *s6);
void gyo_set_particle_damage(gyo *o, int p, double D);
void gyo_hold_particle(gyo *o, int p);
void gyo_set_particle_bc(gyo *o, int p, int type, const double *val, int nval);
void gyo_set_node_bc(gyo *o, int n, int type, const double *val, int nval);
/* MaterialPoints::setTemp (MaterialPoints.cpp:319-322) for `count` particles given by their
 * original index; valid before and between steps. */
void gyo_set_particle_temps(gyo *o, int count, const int *ids, const double *T);
/* Per-particle scale w of the Grady-Kipp activation strain, e_min = w (V k)^(-1/m), by particle
 * id (default 1, the reference's DamageModels.cpp:102-103).  No reference counterpart. */
void gyo_set_particle_flaws(gyo *o, int count, const int *ids, const double *w);

/* Solver(nds, mpts, params, materials): dt from CFL and initialize() (Solver.cpp:7-69). */
int gyo_init_solver(gyo *o, const gyo_params *prm, int nmat, const gyo_material *mats);
double gyo_get_dt(const gyo *o);
void gyo_set_dt(gyo *o, double dt);
void gyo_set_params(gyo *o, const gyo_params *prm);

/* One explicit step, iterate_CPU(t, step) (Solver.cpp:86-292).  Returns 0, or -1 when a
 * particle left the cell range the reference can index. */
int gyo_step(gyo *o, double t, int step);

/* Field access.  Particle arrays are in the oracle's current (sorted) order; pid gives
 * each slot's original particle index. */
enum gyo_pfield {
    GYO_P_POS = 0, GYO_P_POS0, GYO_P_DISP, GYO_P_VEL, GYO_P_GVEL, GYO_P_ACC, GYO_P_STRAINRATE,
    GYO_P_STRESS, GYO_P_STRAIN, GYO_P_PSTRAIN, GYO_P_EQPS, GYO_P_DAMAGE, GYO_P_SMAX, GYO_P_MASS,
    GYO_P_DENSITY, GYO_P_VOLUME, GYO_P_NORMALS, GYO_P_DENSITYRATE, GYO_P_TEMP, GYO_P_TEMPGRAD,
    GYO_P_NFIELDS
};
enum gyo_pifield { GYO_PI_CELL = 0, GYO_PI_MAT, GYO_PI_OBJ, GYO_PI_PID };
enum gyo_nfield {
    GYO_N_MASS = 0, GYO_N_MASS1, GYO_N_MASS2, GYO_N_MOM, GYO_N_MOM1, GYO_N_MOM2, GYO_N_FORCE,
    GYO_N_FORCE1, GYO_N_FORCE2, GYO_N_VEL, GYO_N_VEL1, GYO_N_VEL2, GYO_N_ACC1, GYO_N_ACC2,
    GYO_N_NORMAL1, GYO_N_NORMAL2, GYO_N_TEMP, GYO_N_TEMPRATE
};
enum gyo_nifield { GYO_NI_BODY = 0, GYO_NI_RIGID, GYO_NI_CELLS, GYO_NI_CELLCOUNT };

int gyo_num_particles(const gyo *o);
int gyo_num_nodes(const gyo *o);
void gyo_dims(const gyo *o, int *nxyz);
int gyo_particle_width(int field);
int gyo_node_width(int field);
int gyo_get_particle_field(const gyo *o, int field, double *out);
int gyo_get_particle_ifield(const gyo *o, int field, int *out);
int gyo_get_node_field(const gyo *o, int field, double *out);
int gyo_get_node_ifield(const gyo *o, int field, int *out);

/* Single-function entry points for known-answer tests. */
double gyo_gimp_shape(double dist, double cellsize, double lp);
double gyo_gimp_grad(double dist, double cellsize, double lp, double xp);
int gyo_sym_eigen(const double *a9, double *vec9, double *val3);

#ifdef __cplusplus
}
#endif
#endif
