// gy_common.cuh -- device-side layout, constants and the GIMP basis of the GB300 MPM step.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gy {

// ---------------------------------------------------------------------------------------
// Particle state: one SoA slab of 4-byte lanes, field f of particle i at slab[f*cap + i].
// Positions are an integer cell key plus an FP32 offset per axis: x/h = c + o with
// o in [lp/h, 1 + lp/h), c the cell of the particle's first GIMP node (the stencil base
// getGIMPNodes computes, Extrapolation.cpp:658-660).
enum PField : int {
    PF_OX = 0, PF_OY, PF_OZ,          // offsets within the base cell (cell units)
    PF_VX, PF_VY, PF_VZ,              // velocity
    PF_S0, PF_S1, PF_S2, PF_S3, PF_S4, PF_S5,  // stress xx yy zz xy yz xz
    PF_E0, PF_E1, PF_E2, PF_E3, PF_E4, PF_E5,  // strain
    PF_RHO,                           // density
    PF_MASS,                          // mass (1 for rigid particles, Solver.cpp:51-54)
    PF_KEY,                           // int: block-major cell key (encode_key)
    PF_INFO,                          // int: packed material / object slot / BC / flags
    PF_PID,                           // int: insertion index
    PF_EQPS,                          // accumulated plastic strain
    PF_EP0, PF_EP1, PF_EP2, PF_EP3, PF_EP4, PF_EP5,  // plastic strain
    PF_DMG,                           // damage
    PF_SMAX,                          // max principal stress seen by Grady-Kipp
    PF_NX, PF_NY, PF_NZ,              // contact normals (kept only when tracked)
    PF_COUNT
};

// PF_INFO bit layout
constexpr uint32_t INFO_MAT_MASK = 0xFFFu;         // bits 0-11  material index
constexpr int INFO_OBJ_SHIFT = 12;                 // bits 12-15 object slot (dense, < MAX_BODIES)
constexpr int INFO_BC_SHIFT = 16;                  // bits 16-23 BCTypes value (< 256)
constexpr uint32_t INFO_HOLD = 1u << 24;           // holdParticle
constexpr uint32_t INFO_RIGID = 1u << 25;          // material is rigid
constexpr uint32_t INFO_INIT_VOL = 1u << 26;       // volume still psep^d (no update yet)

__host__ __device__ inline int info_mat(uint32_t i) { return int(i & INFO_MAT_MASK); }
__host__ __device__ inline int info_obj(uint32_t i) { return int((i >> INFO_OBJ_SHIFT) & 0xFu); }
__host__ __device__ inline int info_bc(uint32_t i) { return int((i >> INFO_BC_SHIFT) & 0xFFu); }

// BCTypes::function values (BoundaryConditions.hpp:6-77) the step acts on.
enum BCType : int {
    BC_NONE = 0, BC_GRID_VX = 1, BC_GRID_VY = 2, BC_GRID_VZ = 3, BC_GRID_VX_VY = 11,
    BC_GRID_VX_VZ = 12, BC_GRID_VY_VZ = 13, BC_GRID_VX_VY_VZ = 18,
    BC_MP_VX = 33, BC_MP_VY = 34, BC_MP_VZ = 35, BC_MP_FX = 37, BC_MP_FY = 38, BC_MP_FZ = 39,
    BC_MP_VX_VY = 40, BC_MP_FX_FY = 43, BC_MP_STRESS_XX_YY = 63, BC_MP_VXSIN = 65,
    BC_MP_VYSIN = 66, BC_MP_SYYSIN = 67
};

// Material table (MaterialModels.hpp:29-47), FP32 where the step computes in FP32;
// Grady-Kipp factors precomputed in FP64 on the host.
struct DevMaterial {
    float K, G, rho0, viscosity, yield, cohesion, crit_strain;
    float eta, xi, eta_bar;     // Drucker-Prager cone constants from phi, psi
    float gk_m, gk_rate_coef;   // Grady-Kipp m and ((m+3)/3) * alpha^(1/3)
    float gk_logk;              // log(k) for e_min = (V k)^(-1/m)
    float turb_stress;
    float k_th, c_th;           // thermal conductivity, specific heat capacity
    float phi_deg;              // friction angle in degrees (an input of the learned surrogate)
    int model, rigid, damage, damage_model;
};
constexpr int MAX_MATERIALS = 4096;  // a batch of independent instances carries one per instance
constexpr int MAX_BODIES = 16;

// Grid geometry and per-step scalars, passed by value to every kernel.
struct GridGeom {
    int nx, ny, nz;           // nodes per axis
    int ncx, ncy, ncz;        // cells per axis (ncz = 1 in 2D)
    int nbx, nby, nbz;        // 4x4x4 cell blocks per axis (nbz = 1 in 2D)
    int nnbx, nnby, nnbz;     // 4x4x4 node blocks per axis
    long long nnb;            // node blocks
    unsigned long long div_nbx, div_nby;  // ceil(2^39 / nbx), ceil(2^39 / nby): exact n / d for n < 2^25
    long long nn;             // nodes
    long long nc;             // cells
    float h, inv_h;           // cell size
    float lp;                 // GIMP half-width psep/2 in cell units
    float inv_l, inv_2l, inv_4l;  // 1/lp, 1/(2 lp), 1/(4 lp)
    int is3d;
    // periodic particle wrap (TimeIntegration.cpp:80-108) in cell units:
    // X > wrap_hi[a] -> X += shift; X < 1 -> X -= shift, shift = 1 - (L/h - 2)
    float wrap_hi[3];
    int wrap_shift_int[3];
    float wrap_shift_frac[3];
};

struct StepScalars {
    float dt;
    float dt_node;            // dt, or 0.5*dt at step 1 (Grid.cpp:126-131)
    float gravity[3];
    float damping;
    float mu;
    float t_bc;               // time seen by the sine BCs (set at the end of the previous step)
    int fixed_grid_bcs;
    int multi_body;
    float init_volume;        // psep^3 (psep^2 in 2D): volume before the first update
    int step;                 // the step index (sampling of logged Drucker-Prager returns)
};

// ---------------------------------------------------------------------------------------
// GIMP basis (Extrapolation.cpp:556-647) along one axis, in cell units.
// With offset u = x/h - c in [l, 1+l) the particle's three stencil nodes sit at
// d_k = k - u (node minus particle).  S is the shape value, G the gradient with respect
// to the particle coordinate in 1/cell units (the reference returns -dS/d(dist) for
// positive coordinates, :642-644).  The pieces follow from the reference's piecewise
// definition restricted to the three stencil nodes:
//   u <  1-l: node 0 and 1 on the linear pieces, node 2 outside the support;
//   u >= 1-l: q = u-(1-l) in [0, 2l): node 0 and 2 on the quadratic end pieces, node 1
//             on the central parabola.
__device__ __forceinline__ void gimp_axis(float u, const GridGeom &g, float S[3], float G[3])
{
    const float l = g.lp;
    if (u < 1.0f - l) {
        S[0] = 1.0f - u; S[1] = u;    S[2] = 0.0f;
        G[0] = -1.0f;    G[1] = 1.0f; G[2] = 0.0f;
    } else {
        const float q = u - (1.0f - l);
        const float a = 2.0f * l - q;          // = 1 + l - u
        const float d1 = 1.0f - u;
        S[0] = a * a * g.inv_4l;
        S[1] = 1.0f - (d1 * d1 + l * l) * g.inv_2l;
        S[2] = q * q * g.inv_4l;
        G[0] = -a * g.inv_2l;
        G[1] = d1 * g.inv_l;
        G[2] = q * g.inv_2l;
    }
}

// Cell keys are block-major: 4x4x4 cell blocks in x-fastest order, cells x-fastest inside
// a block, key = block * 64 + (lz*4 + ly)*4 + lx.  Sorting by key groups each block's
// particles contiguously, which the tiled P2G needs.
constexpr int CB = 4;           // cells per block edge
constexpr int CB_SHIFT = 6;     // log2(CB^3)

__host__ __device__ __forceinline__ int encode_key(int ci, int cj, int ck, const GridGeom &g)
{
    const int blk = ((ck >> 2) * g.nby + (cj >> 2)) * g.nbx + (ci >> 2);
    return (blk << CB_SHIFT) | ((ck & 3) << 4) | ((cj & 3) << 2) | (ci & 3);
}

// n / d by multiply-shift with M = ceil(2^39 / d): the error n (M - 2^39/d) / 2^39 stays
// below 2^-14 for n < 2^25, smaller than the 1/d gap to the next integer for d < 2^14, and
// n * M < 2^64.
__host__ __device__ __forceinline__ int fast_div(int n, unsigned long long M)
{
    return (int)(((unsigned long long)(unsigned)n * M) >> 39);
}

__host__ __device__ __forceinline__ void decode_block(int blk, const GridGeom &g, int &bx, int &by, int &bz)
{
    const int t = fast_div(blk, g.div_nbx);
    bx = blk - t * g.nbx;
    bz = fast_div(t, g.div_nby);
    by = t - bz * g.nby;
}

__host__ __device__ __forceinline__ void decode_key(int key, const GridGeom &g, int &ci, int &cj, int &ck)
{
    int bx, by, bz;
    decode_block(key >> CB_SHIFT, g, bx, by, bz);
    ci = (bx << 2) | (key & 3);
    cj = (by << 2) | ((key >> 2) & 3);
    ck = (bz << 2) | ((key >> 4) & 3);
}

__host__ __device__ __forceinline__ long long node_block(int i, int j, int k, const GridGeom &g)
{
    return ((long long)(k >> 2) * g.nnby + (j >> 2)) * g.nnbx + (i >> 2);
}

// grids hold fewer than 2^31 nodes (checked at creation), so 32-bit index math suffices
__device__ __forceinline__ int node_index(int i, int j, int k, const GridGeom &g)
{
    return i + (j + k * g.ny) * g.nx;
}

// device error bits
// Programmatic dependent launch (the re-sort's chain of short kernels): a kernel first lets
// the next kernel of its stream start launching (once all of this grid's CTAs are resident)
// and then waits until its own predecessor has completed and its writes are visible.
// Launched without the attribute, both instructions return at once.
__device__ __forceinline__ void pdl_prologue()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

constexpr int ERR_RANGE = 1;
constexpr int ERR_NONFINITE = 2;
constexpr int ERR_TC_TIMEOUT = 4;  // a tensor-core wait gave up (gy_tc.cuh)

}  // namespace gy
