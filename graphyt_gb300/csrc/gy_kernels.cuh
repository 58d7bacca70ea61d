// gy_kernels.cuh -- launch interface between the host runtime (gy_api.cu) and the kernels.
#pragma once

#include <utility>

#include "gy_common.cuh"

namespace gy {

// Device view of one particle slab.
struct PView {
    float *base;
    long long cap;
    __device__ __forceinline__ float &f(int field, long long i) const { return base[(long long)field * cap + i]; }
    __device__ __forceinline__ int &ii(int field, long long i) const
    {
        return reinterpret_cast<int *>(base)[(long long)field * cap + i];
    }
};

// Single-body node buffers.  Accumulators (P2G target, zeroed by the solve):
//   acc0 = (m, px, py, pz), acc1 = (fx, fy, fz, -).
// Solved fields (read by G2P): gv = (m, v1x, v1y, v1z), ga = (a1x, a1y, a1z, -).
// Multi-body adds per-slot accumulators and solved fields.
struct NodeBufs {
    float4 *acc0, *acc1;
    float4 *gv, *ga;
    float4 *out_com;        // optional (vcom, -) for node getters
    float4 *out_force;      // optional COM force for node getters
    const unsigned char *bc_type;
    const float4 *bc_val;
    // multi-body
    float4 *bacc0[2], *bacc1[2];  // per body slot: (m, p), (f, -)
    float4 *bnrm[2];              // per body slot: (n, -)
    float4 *bgv[2], *bga[2];      // solved per slot: (m, v), (a, -); slot 0's are gv / ga
    float4 *nrm_out[2];           // normalised slot normals (only when normals are tracked)
    int2 *body;                   // body slot objects (dense ids) or -1
    int *flags;                   // active 4x4x4 node blocks (set by P2G / fold, cleared by the solve)
    int *active_list;             // node blocks marked this step, in marking order
    int *active_n;                // length of active_list
    unsigned char *has_rigid;     // bit0: slot 0 rigid, bit1: slot 1 rigid
    int *active_count;            // nodes with mass (stats)
    int *block_body;              // per 4x4x4 cell block: the one body of its 6x6x6 node tile, -1 none, -2 more
    int *nblk_two;                // per 4x4x4 node block: 1 if one of its nodes holds two bodies
};

// Hooks of the learned Drucker-Prager surrogate into the step (every pointer null when off).
// Logging: the exact return mapping records, for particles that yield and whose
// (insertion index + step) is a multiple of log_every, the MLP input (strain increment,
// previous stress, plastic strain, damage, cohesion, friction angle) and target (stress
// minus the elastic trial stress, plastic strain increment).  Deferral: a yielding particle
// without a BC goes to the pending list (slot and strain increment) with its stress left at
// the previous value; the surrogate pass finishes its return mapping and damage.
struct DpHooks {
    float *log_x, *log_y;         // [log_cap][16], [log_cap][7]
    unsigned int *log_n;          // records claimed (those past log_cap are dropped)
    unsigned int log_cap;
    int log_every;
    float4 *pend;                 // [pend_cap][2]: (slot bits, de0, de1, de2), (de3, de4, de5, -)
    unsigned int *pend_n;
    unsigned int pend_cap;
};

struct StepArgs {
    GridGeom g;
    const StepScalars *sc;   // per-step scalars in device memory (one small copy per step)
    int multi_body;          // host-side launch choice, fixed per handle
    const DevMaterial *mats;
    const float4 *pbc_val;   // particle BC values by pid
    const float *flaw;       // Grady-Kipp activation strain scale by pid, or null (every scale 1)
    int *status;
    double *stats;           // STATS_SLOTS x 8 conservation partials written by G2P, or null
    DpHooks dp;              // learned-surrogate logging / deferral (zero when off)
    unsigned *mover_mask;    // G2P flags the slots whose key changed, one bit per slot (or null),
    int *mover_cnt;          //   with the flagged count per 32 slots, for the next re-sort
};

// partials of the conservation sums (mass, momentum, kinetic and strain energy); the host
// adds the slots
constexpr int STATS_SLOTS = 16;

// launch with programmatic stream serialization (the kernel starts with pdl_prologue), so the
// launch of a kernel overlaps the tail of the one before it in the stream or graph
template <typename... P, typename... A>
inline cudaError_t launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, cudaStream_t s, A &&... args)
{
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t c{};
    c.gridDim = grid;
    c.blockDim = block;
    c.dynamicSmemBytes = 0;
    c.stream = s;
    c.attrs = at;
    c.numAttrs = 1;
    return cudaLaunchKernelEx(&c, kernel, std::forward<A>(args)...);
}

// keeps the first failure of a sequence of launches (err may be null)
inline void keep_first(cudaError_t *err, cudaError_t e)
{
    if (err && e != cudaSuccess && *err == cudaSuccess) *err = e;
}

// process-wide count of kernel launches (for the benchmark's launch accounting)
void note_launch(int k);
long long launch_count();

// launchers (gy_kernels.cu)
// therm / tnode non-null: the single-body kernel also sums the heat conduction node fields
// (multi-body problems run launch_thermal_p2g instead).  lanes: lanes per run of equal cell in
// the single-body kernel without heat conduction, 3 (z-plane lanes) or 9 (x-column lanes).
void launch_p2g(const PView &p, const int *perm, const int *skey, long long n, const int *seg_start,
                const int *nseg, int persist_grid, const NodeBufs &nb, const StepArgs &a, cudaStream_t s,
                const float4 *therm = nullptr, float2 *tnode = nullptr, int lanes = 3, int *defer = nullptr,
                int *ndefer = nullptr);
void launch_fold(const NodeBufs &nb, const StepArgs &a, cudaStream_t s);
void launch_block_body(const NodeBufs &nb, const GridGeom &g, cudaStream_t s);
void launch_solve(const NodeBufs &nb, const StepArgs &a, bool keep_node_fields, cudaStream_t s);
// therm / tnode non-null: the single-body kernel also runs the heat conduction G2P and the
// temperature update (multi-body problems run launch_thermal_g2p instead)
void launch_g2p_update(const PView &src, const PView &dst, const int *perm, const int *skey, long long n,
                       const int *seg_start, const int *nseg, int g2p_grid, const NodeBufs &nb, const StepArgs &a,
                       bool track_normals, bool check_finite, bool has_dp, cudaStream_t s, float4 *therm = nullptr,
                       const float2 *tnode = nullptr);
int g2p_blocks_per_sm(bool has_dp);
int p2g_blocks_per_sm();
// the learned surrogate's pass over the particles G2P deferred (gy_mlp.cu)
void launch_dp_surrogate(const PView &P, const float4 *pend, const unsigned int *pend_n, unsigned int cap,
                         const DevMaterial *mats, const float *prm, const StepScalars *scp, const float *flaw, float tol,
                         unsigned long long *counts, int *status, cudaStream_t s);
void launch_body_tables(const PView &p, long long n, const StepArgs &a, int *cell_min, int nbody,
                        const int *refkeys, cudaStream_t s);
void launch_body_assign(const NodeBufs &nb, const StepArgs &a, const int *cell_min, int nbody,
                        const int *nidx_x, const int *nidx_y, const int *nidx_z, cudaStream_t s);
void launch_stats(const PView &p, long long n, double *out8, cudaStream_t s);
void launch_gather_slab(const float *src, float *dst, const int *perm, long long n, long long cap, int nfields,
                        cudaStream_t s);

// heat conduction (gy_thermal.cu): therm = (T, grad T) per insertion index, tnode = (T, rate)
void launch_thermal_p2g(const PView &p, const float4 *therm, const int *perm, const int *skey, long long n,
                        const int *seg_start, const int *nseg, float2 *tnode, const StepArgs &a, cudaStream_t s);
void launch_thermal_g2p(const PView &p, float4 *therm, const int *perm, const int *skey, long long n,
                        const int *seg_start, const int *nseg, const float2 *tnode, const NodeBufs &nb,
                        const StepArgs &a, cudaStream_t s);
void launch_thermal_clear(const NodeBufs &nb, const StepArgs &a, float2 *tnode, cudaStream_t s);
void launch_thermal_set(float4 *therm, const int *ids, const float *T, int count, long long n, cudaStream_t s);

// sort (gy_sort.cu): stable LSD radix sort of (key, index) pairs
struct SortScratch {
    int *keys[2], *vals[2];
    int *hist;          // 2 * 256 * nblocks
    int *scan_tmp;      // scan workspace
    long long cap;
    int nblocks_cap;
};
size_t sort_scratch_bytes(long long n);

// Incremental re-sort (gy_resort.cu): scratch, zeroed once at allocation.
struct ResortScratch {
    unsigned *wmask;
    int *wcnt, *wpref, *wscan_tmp;
    int *bkey, *bidx, *gap, *bslot;       // the movers in slot order
    unsigned long long *stage;            // the movers grouped by key bucket, as (key, slot) words
    int *tval;                            // a buffer of the fallback sort
    int *gapcnt, *gwcnt, *gwpref, *gscan_tmp;
    int *big;                             // a bucket too crowded to rank by counting
    int *mlast;                           // the last re-sort's mover count
    long long cap, ngw;
};
size_t resort_scratch_ints(long long cap);
void resort_bind(ResortScratch &rs, int *mem, long long cap);
void resort_keys(const int *key, const int *prev_skey, int *skey_out, int *perm_out, long long n, int key_bits,
                 ResortScratch &rs, cudaStream_t s, bool mask_ready = false, const int *blk_first = nullptr);
// err (may be null) receives the first launch failure of the sort's kernels
const int *sort_pairs(const int *keys_in, int *perm_out, long long n, int key_bits, SortScratch &ws, cudaStream_t s,
                      cudaError_t *err = nullptr);
// nseg must be zero on entry; clear0..2 (may be null): counters the kernel zeroes on the way;
// blk_first (may be null, one int per cell block): each non-empty block's first position
void launch_block_heads(const int *skey, long long n, int *seg_start, int *nseg, cudaStream_t s,
                        int *clear0 = nullptr, int *clear1 = nullptr, int *clear2 = nullptr,
                        int *blk_first = nullptr);
void exclusive_scan_int(const int *in, int *out, long long n, int *tmp, cudaStream_t s, cudaError_t *err = nullptr);

// exclusive scan of ints: tiles of SCAN_TILE, scanned recursively over the tile sums
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// ints of scratch exclusive_scan_int needs for n elements (constant-evaluable, so fixed
// scratch sizes can be checked at compile time)
constexpr size_t scan_tmp_ints(long long n)
{
    size_t total = 0;
    long long m = n;
    while (m > SCAN_TILE) {
        m = (m + SCAN_TILE - 1) / SCAN_TILE;
        total += (size_t)m * 2 + 32;
    }
    return total + 64;
}

}  // namespace gy
