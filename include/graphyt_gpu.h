/*
 * graphyt_gpu.h -- C ABI of the GB300 explicit GIMP MPM step (libgraphyt_gpu.so).
 *
 * One handle holds one simulation: a uniform background grid (the reference's Nodes), a
 * particle set (MaterialPoints), a material table (std::vector<MaterialModels>), the global
 * Parameters and the Solver's dt.  Particle and grid state live on one GPU in SoA layout
 * from gy_initialize() on; gy_step() advances one explicit step on the handle's CUDA stream
 * without a host sync; downloads sync.
 *
 * Conventions
 *   - Plain pointers and sizes only; every host array is caller-owned and only read or
 *     written during the call.
 *   - Every call returns gy_status (0 = GY_OK).  On error, gy_last_error(h) describes it.
 *   - Calls on one handle are not re-entrant; different handles are independent.
 *   - Particle arrays are exchanged in insertion order (particle i is the i-th particle
 *     given to gy_add_particles), whatever order the device currently keeps them in.
 *
 * Each entry point names the reference interface it replaces (file:line in the reference
 * tree).  The reference has no GPU path: its Solver::iterate_GPU (Solver.cpp:293-302) is a
 * stub, so gy_step is the first GPU implementation of iterate_CPU (Solver.cpp:86-292).
 */
#ifndef GRAPHYT_GPU_H
#define GRAPHYT_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GY_ABI_VERSION 4

typedef int gy_status;
enum {
    GY_OK = 0,
    GY_ERR_ARG = -1,         /* invalid argument or handle */
    GY_ERR_CUDA = -2,        /* a CUDA call failed (message in gy_last_error) */
    GY_ERR_STATE = -3,       /* call out of order (e.g. gy_step before gy_initialize) */
    GY_ERR_RANGE = -4,       /* a particle left the grid the reference can index */
    GY_ERR_UNSUPPORTED = -5, /* input the GPU path does not implement */
    GY_ERR_NONFINITE = -6,   /* a NaN or Inf appeared in particle state */
    GY_ERR_NOMEM = -7        /* device allocation failed */
};

typedef struct gy_solver gy_solver;

/* Background grid, Nodes::Nodes(std::vector<double> L, double cellsize) (Nodes.cpp:8-141),
 * plus MaterialPoints::psep (MaterialPoints.hpp:82).  L[2] == 0 selects a 2D grid. */
typedef struct gy_grid_desc {
    double L[3];
    double cellsize;
    double psep;
} gy_grid_desc;

/* One material, MaterialModels (MaterialModels.hpp:5-48); field order is part of the ABI. */
typedef struct gy_material {
    double bulkMod, shearMod, density, viscosity, thermalConductivity, specificHeatCapacity;
    double yieldStress, cohesion, criticalStrain, phi, psi, Cg, damageM, damageK, turbStress;
    int isRigid, isDamage, damageModel, model;
} gy_material;

/* Parameters (Parameters.hpp:16-32) plus one switch: fixed_grid_bcs = 1 gives
 * grid_vz / grid_vx_vz / grid_vy_vz / grid_vx_vy_vz a body (empty in the reference,
 * Grid.cpp:872-873, 1032-1052); 0 keeps the reference's behaviour. */
typedef struct gy_params {
    double gravity[3];
    double damping;
    double mu;
    double CFL;
    double tmax;
    int is3D;
    int fixed_grid_bcs;
} gy_params;

/* Tuning knobs that change speed, never results beyond summation order. */
typedef struct gy_options {
    int sort_every;     /* reorder particle state by cell every n steps (>= 1) */
    int full_sort;      /* 1: every sort is a full radix sort; 0: after the first, an incremental
                           re-sort of the particles that changed cell (same permutation) */
    int use_graph;      /* 1 (default): each step replays a captured CUDA graph of its kernels,
                           the step's scalars reaching the device in one small copy; 0: the
                           kernels are launched one by one */
    int track_normals;  /* 1: keep per-particle contact normals (getNormalsArr) */
    int check_finite;   /* 1: flag NaN/Inf in particle state every step */
    int keep_node_fields; /* 1: keep centre-of-mass node velocity/force for node getters */
    int p2g_lanes;      /* P2G (with or without heat conduction): lanes per run of equal cell, 3 (default:
                           each lane sums a z-plane of nine stencil nodes) or 9 (each lane a
                           column of three x nodes).  Multi-body problems without tracked
                           normals: 3 sends the segments of one deformable object whose node
                           tile holds that body only through the 3-lane kernel and the rest
                           through the body-slot kernel; 9 sends every segment through the
                           body-slot kernel.  Same sums, different speed */
} gy_options;

/* FP64 conservation sums and counters, Solver.cpp:264-289's printout made a struct. */
typedef struct gy_stats {
    double mass;           /* sum m_p */
    double momentum[3];    /* sum m_p v_p */
    double kinetic;        /* sum 0.5 m_p |v_p|^2 */
    double strain_energy;  /* sum 0.5 V_p sigma_p : eps_p */
    int64_t active_nodes;  /* nodes with nonzero mass after the last P2G */
    int64_t steps;         /* steps taken by this handle */
    int64_t status_flags;  /* device error bits (range / nonfinite) */
} gy_stats;

/* Particle fields for gy_get_particles / gy_set_particles (double, insertion order).
 * Widths: POS 3, POS0 3, DISP 3, VEL 3, STRESS 6, STRAIN 6, PSTRAIN 6, EQPS 1, DAMAGE 1,
 * SMAX 1, MASS 1, DENSITY 1, VOLUME 1, NORMALS 3, TEMP 1, TEMPGRAD 3.  Stress/strain order
 * xx yy zz xy yz xz.  TEMP / TEMPGRAD: getTemperatureArr (MaterialPoints.cpp:265) and the
 * particle temperature gradient of the last G2P (Extrapolation.cpp:358-361). */
enum gy_pfield {
    GY_P_POS = 0, GY_P_POS0, GY_P_DISP, GY_P_VEL, GY_P_STRESS, GY_P_STRAIN, GY_P_PSTRAIN,
    GY_P_EQPS, GY_P_DAMAGE, GY_P_SMAX, GY_P_MASS, GY_P_DENSITY, GY_P_VOLUME, GY_P_NORMALS,
    GY_P_TEMP, GY_P_TEMPGRAD,
    GY_P_NFIELDS
};
/* Integer particle fields: CELLID (the reference's binning key, TimeIntegration.cpp:110-115),
 * MATERIAL, OBJECT, DEVICE_SLOT (where the device keeps the particle now). */
enum gy_pifield { GY_PI_CELLID = 0, GY_PI_MATERIAL, GY_PI_OBJECT, GY_PI_DEVICE_SLOT };
/* Node fields (double, node order i + j*Nx + k*Nx*Ny): MASS 1 (centre of mass), VEL 3
 * (centre-of-mass velocity), FORCE 3, VEL1 3 / ACC1 3 (body-1 field after the solve).
 * VEL and FORCE need gy_options.keep_node_fields = 1 during the step. */
enum gy_nfield { GY_N_MASS = 0, GY_N_VEL, GY_N_FORCE, GY_N_VEL1, GY_N_ACC1, GY_N_NFIELDS };

/* ---------------------------------------------------------------------------------------- */

/* Library ABI version (GY_ABI_VERSION). */
int gy_abi_version(void);

/* Nodes::Nodes (Nodes.cpp:8-141) + MaterialPoints::MaterialPoints (MaterialPoints.cpp:10-17).
 * device < 0 uses the current device.  Rejects grids where the reference's truncated
 * Nx*Ny*Nz differs from its rounded numNodes (Nodes.cpp:12, 71-73). */
gy_status gy_create(const gy_grid_desc *grid, int device, gy_solver **out);

/* Releases every device and host resource of the handle. */
gy_status gy_destroy(gy_solver *h);

/* Message for the last failed call on this handle (never NULL). */
const char *gy_last_error(const gy_solver *h);

/* Grid size: nxyz[3] = Nx, Ny, Nz; numNodes = Nx*Ny*Nz (Nodes.cpp:12, 71-73). */
gy_status gy_grid_dims(const gy_solver *h, int *nxyz, int64_t *num_nodes);

/* MaterialPoints::addPyckGeom + addPyckIntField("material"/"objectID")
 * (MaterialPoints.cpp:24-54, add() at :95-235).  mat/obj may be NULL (zeros).  Appends. */
gy_status gy_add_particles(gy_solver *h, int64_t n, const double *pos3, const int *mat, const int *obj);

/* MaterialPoints::setVel (MaterialPoints.cpp:302-306), setStress (:312-319), setDamage
 * (:308-310), holdParticle (:336-340), setBC (:88-93), for many particles at once.
 * idx lists insertion indices; values are per listed particle. */
gy_status gy_set_particle_vel(gy_solver *h, int64_t count, const int64_t *idx, const double *vel3);
gy_status gy_set_particle_stress(gy_solver *h, int64_t count, const int64_t *idx, const double *s6);
gy_status gy_set_particle_damage(gy_solver *h, int64_t count, const int64_t *idx, const double *d);
gy_status gy_hold_particles(gy_solver *h, int64_t count, const int64_t *idx);
gy_status gy_set_particle_bc(gy_solver *h, int64_t count, const int64_t *idx, const int *type, const double *val4);

/* Per-particle scale w > 0 of the Grady-Kipp activation strain, e_min = w (V k)^(-1/m), for
 * many particles (before gy_initialize).  The reference computes the deterministic
 * e_min = (V k)^(-1/m) (DamageModels.cpp:102-103), which is w = 1, every particle's default;
 * a per-particle Weibull draw w = (-ln U)^(1/m) gives each particle the activation strain of
 * the weakest flaw of a Poisson flaw population k e^m in its volume.  No reference
 * counterpart (the reference has no per-particle flaw field). */
gy_status gy_set_particle_flaw(gy_solver *h, int64_t count, const int64_t *idx, const double *w);

/* MaterialPoints::setTemp (MaterialPoints.cpp:319-322) for many particles.  Unlike the other
 * setters it also works between steps (the reference's scripts reset temperatures every step,
 * Examples/thermalTest.py:110-117).  The heat conduction terms of the step run once any
 * temperature is nonzero. */
gy_status gy_set_particle_temp(gy_solver *h, int64_t count, const int64_t *idx, const double *T);

/* Nodes::setBC (Nodes.cpp:155-163) for many nodes: node index, BCTypes value, 4 values. */
gy_status gy_set_node_bc(gy_solver *h, int64_t count, const int64_t *nodes, const int *type, const double *val4);

/* Solver::Solver (Solver.cpp:7-37): stores the materials and parameters, sets dt =
 * CFL*h/sqrt(maxK/minRho) and runs initialize() (Solver.cpp:40-69); uploads all state.
 * Up to 4096 materials and 16 distinct objectIDs (GY_ERR_UNSUPPORTED beyond). */
gy_status gy_initialize(gy_solver *h, const gy_material *mats, int nmat, const gy_params *prm);

/* Solver::setDt (Solver.cpp:70-73) and the dt attribute (Solver.i:17). */
gy_status gy_set_dt(gy_solver *h, double dt);
gy_status gy_get_dt(const gy_solver *h, double *dt);

/* The Parameters* passed to every iterate call (gravity, damping, friction may change). */
gy_status gy_set_params(gy_solver *h, const gy_params *prm);

gy_status gy_set_options(gy_solver *h, const gy_options *opt);
gy_status gy_get_options(const gy_solver *h, gy_options *opt);

/* Solver::iterate_GPU(double t, int step, Parameters*) -- the GPU counterpart of
 * iterate_CPU (Solver.cpp:86-292).  Enqueues one step on the handle's stream and returns
 * without waiting.  step selects the reference's step-dependent rules (half dt at step 1,
 * Grid.cpp:126-131); t is the time stored for the next step's sine-ramped particle BCs. */
gy_status gy_step(gy_solver *h, double t, int step);

/* Solver::iterate_CPU_steps (Solver.cpp:75-84) on the GPU: nsteps steps from step0/t0,
 * t advancing by dt.  use_graph overrides gy_options.use_graph for these steps. */
gy_status gy_steps(gy_solver *h, double t0, int step0, int nsteps, int use_graph);

/* Waits for all queued work, then reports device error flags (GY_ERR_RANGE /
 * GY_ERR_NONFINITE) raised since the last gy_sync. */
gy_status gy_sync(gy_solver *h);

/* The handle's CUDA stream (a cudaStream_t), for callers that time or order work. */
void *gy_stream(gy_solver *h);

/* Particle getters (MaterialPoints.cpp:238-273) and setters; count must equal n*width. */
gy_status gy_num_particles(const gy_solver *h, int64_t *n);
gy_status gy_get_particles(gy_solver *h, int field, double *out, int64_t count);
gy_status gy_get_particles_int(gy_solver *h, int field, int *out, int64_t count);
/* Node getters (Nodes.cpp:147-153): getMassArr, getVelArr, getForceArr and body-1 fields. */
gy_status gy_get_nodes(gy_solver *h, int field, double *out, int64_t count);

/* Stable sort of n non-negative keys on the device, the counting sort the step uses:
 * perm_out[i] = index of the i-th key in ascending order, ties in input order.  Host
 * arrays; for testing the sort against a CPU stable sort. */
gy_status gy_sort_keys(const int *keys, int64_t n, int *perm_out, int device);

/* The incremental re-sort the step uses after its first sort (no counterpart in the
 * reference, whose Extrapolation.cpp:370-503 sorts from scratch).  prev_sorted[i] is the key
 * particle i had at the last sort, in that sort's order (non-decreasing); keys[i] is its key
 * now.  Result: the stable ascending order of keys, equal to gy_sort_keys(keys).  Host arrays;
 * GY_ERR_ARG if prev_sorted is not non-decreasing or a key is negative. */
gy_status gy_resort_keys(const int *keys, const int *prev_sorted, int64_t n, int *perm_out, int *sorted_out,
                         int device);

/* Checkpoint / resume of the device state.  The reference has no checkpoint: its only
 * output, Serialise (MaterialPoints.cpp:341-364), writes lossy %f CSV with no reader.
 * gy_state_size gives the byte size of a snapshot; gy_state_save copies the particle state
 * (and the body-slot table of multi-body problems) into a caller buffer after the queued
 * work finishes; gy_state_load restores it into a handle built from the same model (same
 * grid, particle count, materials and options).  The step index is the caller's, so a
 * resumed run keeps the reference's step-dependent rules (sort cadence, half dt at step 1). */
gy_status gy_state_size(const gy_solver *h, int64_t *bytes);
gy_status gy_state_save(gy_solver *h, void *buf, int64_t bytes);
gy_status gy_state_load(gy_solver *h, const void *buf, int64_t bytes);

/* Allocation-free form of gy_sort_keys.  It has no counterpart in the reference.  Some
 * callers cannot call cudaMalloc or cudaFree at the point where they sort: a host framework
 * that owns all device memory through its own pool and forbids other allocations, or a
 * step loop that cannot absorb the device-wide synchronisation cudaFree implies.  This
 * entry point sorts device-resident keys with the same stable radix sort, taking its
 * scratch from a fixed array compiled into the library instead of allocating it.
 *   d_keys      n device ints, non-negative and below 2^key_bits (1 <= key_bits <= 31)
 *   d_perm_out  n device ints: index of the i-th key in ascending order, ties in input order
 *   stream      a cudaStream_t (NULL = legacy default stream); the call only enqueues work
 * Limit: n <= GY_SORT_STATIC_MAX; larger n returns GY_ERR_ARG before any GPU work.  The
 * scratch (4.47 MB, 4.27 MiB) is held on every GPU that loads the library until the process
 * exits.  The first call on a device looks the scratch's device address up once, on the
 * calling thread's current device; make that first call before any stream capture.  The
 * address is kept for the process: a cudaDeviceReset replaces the device's primary context
 * and leaves it stale, so do not reset a device this entry point has run on.  The status
 * reports this call's own launches; an error left by earlier work stays pending.  All
 * calls share the one scratch array: calls whose work overlaps on the GPU (two streams, or
 * two host threads) race and corrupt each other's results; order them on one stream. */
#define GY_SORT_STATIC_MAX 262144
gy_status gy_sort_keys_static(const int *d_keys, int64_t n, int key_bits, int *d_perm_out, void *stream);

/* FP64 conservation sums over the particles (waits for queued work). */
gy_status gy_get_stats(gy_solver *h, gy_stats *out);

/* Phase timing with CUDA events on the handle's stream, recorded around every phase of
 * every step while on, without host syncs.  gy_get_phase_times waits, returns the summed
 * milliseconds per phase since timing was switched on -- [0] sort+permute, [1] P2G,
 * [2] fold+solve, [3] G2P+update, [4] total -- with the number of timed steps, and resets. */
gy_status gy_set_phase_timing(gy_solver *h, int on);
gy_status gy_get_phase_times(gy_solver *h, float *ms5, int64_t *steps);

/* Device time of nsteps consecutive steps (as gy_steps), from CUDA events recorded on the
 * handle's stream before the first and after the last step. */
gy_status gy_time_steps(gy_solver *h, double t0, int step0, int nsteps, float *ms);

/* Tensor-core GEMM, C[M x N] = A[M x K] * B[N x K]^T: BF16 row-major A and B (K contiguous),
 * FP32 row-major C, all in device memory; 16 <= N <= 256 and 16 <= K <= 256, both multiples of
 * 16.  tcgen05 MMAs from shared memory into tensor memory, one 128-row tile per CTA.  No
 * reference counterpart: the building block of the learned constitutive surrogate's kernels,
 * exposed so it can be checked on its own.  d_status (may be null) receives bit 4 if a
 * tensor-core wait gave up.  Only enqueues work on stream. */
gy_status gy_tc_gemm_bf16(const uint16_t *d_A, const uint16_t *d_B, float *d_C, int M, int N, int K, int *d_status,
                          void *stream);

/* Self-check of the bounded waits (no reference counterpart): one block waits on an mbarrier
 * that nothing completes, gives up after the library's poll limit (a fraction of a second),
 * sets bit 4 in d_status and writes the wait's duration in ns to d_elapsed_ns -- the path every
 * tensor-core wait takes when its arrival is lost, so a lost arrival ends the kernel with a
 * status instead of a hang.  Only enqueues work on stream. */
gy_status gy_tc_wait_check(int *d_status, unsigned long long *d_elapsed_ns, void *stream);

/* ---- learned Drucker-Prager surrogate (no reference counterpart) --------------------------
 * A 16 -> 64 -> 64 -> 7 MLP with SiLU in one packed FP32 parameter vector of
 * gy_mlp_param_count() floats: W1 [16][64], b1 [64], W2 [64][64], b2 [64], W3 [64][7], b3 [7]
 * (y = x W + b, weights input-major), then the input mean [16] and std [16] and the output
 * mean [7] and std [7] (x_n = (x - mean) / std, y = y_n std + mean).  The kernels run it in
 * BF16 on the tensor cores (tcgen05 MMAs, FP32 accumulation in tensor memory) over tiles of
 * 128 rows. */
int64_t gy_mlp_param_count(void);

/* Y [n][7] = MLP(X [n][16]), raw FP32 rows in device memory; only enqueues work on stream.
 * d_status (may be null) receives bit 4 if a tensor-core wait gave up. */
gy_status gy_mlp_forward(const float *d_params, const float *d_X, int64_t n, float *d_Y, int *d_status, void *stream);

/* Gradient of the mean squared error over rows [0, n) (n a multiple of 128), normalised
 * targets: d_grad [gy_mlp_param_count()] and d_loss [1] receive += (zero them first).  The
 * training kernel's own pass (BF16 tensor-core forward, backward and weight gradients), for
 * checking it. */
gy_status gy_mlp_grad(const float *d_params, const float *d_X, const float *d_T, int64_t n, float *d_grad,
                      float *d_loss, int *d_status, void *stream);

/* Train the MLP in place: steps Adam steps (lr, betas 0.9 / 0.999) on batches of `batch` rows
 * (a multiple of 128) drawn with replacement from X [n][16] -> T [n][7] by a hash of (seed,
 * step, row); the loss is the mean squared error of the normalised outputs.  init != 0 first
 * sets the normalisation from the data and draws the weights (seeded).  Each step is one
 * tensor-core kernel over the batch plus one Adam kernel, replayed from a CUDA graph; the call
 * allocates its optimizer state and returns after the last step with its loss in *loss_out. */
gy_status gy_mlp_train(float *d_params, const float *d_X, const float *d_T, int64_t n, int steps, int batch, float lr,
                       uint64_t seed, int init, float *loss_out, int *d_status, void *stream);

/* The surrogate in the step (Drucker-Prager materials, 3D).  Logging: while on, the exact
 * return mapping records, for yielding particles whose (insertion index + step) is a multiple
 * of `every`, the MLP input (strain increment 6, previous stress 6, accumulated plastic
 * strain, damage, cohesion, friction angle in degrees) and target (stress minus the elastic
 * trial stress 6, plastic strain increment), up to cap records (later ones are dropped).
 * gy_dp_surrogate_train trains the handle's surrogate on the logged records (normalisation and
 * weights from scratch).  With the surrogate on, a yielding particle without a BC takes the
 * MLP's return (stress = trial + predicted correction) when the yield function there is
 * within tol x cohesion of zero and the predicted increment is not negative, else the exact
 * return mapping (ConstitutiveModels.cpp:238-429); damage stays exact.  counts: predictions
 * kept and fallbacks since the surrogate parameters were first set. */
gy_status gy_dp_log_begin(gy_solver *h, int64_t cap, int every);
gy_status gy_dp_log_end(gy_solver *h);
gy_status gy_dp_log_count(gy_solver *h, int64_t *count);
gy_status gy_dp_log_read(gy_solver *h, float *x16, float *y7, int64_t max_records);
gy_status gy_dp_surrogate_train(gy_solver *h, int steps, int batch, float lr, uint64_t seed, float *loss_out);
gy_status gy_set_dp_surrogate(gy_solver *h, const float *params, int on, float tol);
gy_status gy_get_dp_surrogate(gy_solver *h, float *params);
gy_status gy_dp_surrogate_counts(gy_solver *h, int64_t *kept, int64_t *fallback);

/* Number of kernels this library has launched in the process so far. */
int64_t gy_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif /* GRAPHYT_GPU_H */
