// gy_kernels.cu -- the GB300 kernels of one explicit GIMP MPM step.
//
// Data flow of a step (single body, the fast path):
//   sort      stable counting sort of the particle cell keys (gy_sort.cu) -> perm, plus the
//             list of non-empty 4x4x4 cell blocks ("segments");
//   fold      periodic node-layer fold of the accumulated P2G fields (Grid.cpp:310-795);
//   P2G       one CTA per segment: particles of a run of equal cell are summed in registers
//             (nine lanes per run, a lane per x column of three stencil nodes) into a
//             shared-memory node tile, flushed with vector reductions (Extrapolation.cpp:
//             166-286); multi-body problems keep the centre-of-mass and both body-slot
//             fields in the tile (a lane per stencil node);
//   solve     nodal momentum update + grid BCs over the active 4x4x4 node blocks only
//             (Grid.cpp:9-245, 862-1094); it also clears the accumulators it read;
//   G2P       one CTA per segment over a shared-memory tile of the solved nodes, a thread
//             per particle in sorted order: G2P (Extrapolation.cpp:127-163, 288-367), particle
//             BCs (TimeIntegration.cpp:177-296), update + constitutive + damage + wrap
//             (TimeIntegration.cpp:11-117), the state written to the other slab in sorted
//             order, with the momentum and energy sums of that state.
//
// P2G is a particle-centric scatter: the reference gathers per node over a 4x4x4 cell
// window (Extrapolation.cpp:31-125), but a particle contributes exactly to the nodes of its
// GIMP support, so scattering over its 3x3x3 stencil sums the same terms.
#include <algorithm>
#include <atomic>
#include <cstdio>

#include "gy_kernels.cuh"
#include "gy_physics.cuh"

namespace gy {

static std::atomic<long long> g_launches{0};
void note_launch(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------------------------------
// helpers

__device__ __forceinline__ void red_add4(float4 *a, float x, float y, float z, float w)
{
    // one vector reduction request for four floats into global memory (sm_90+)
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(a), "f"(x), "f"(y), "f"(z), "f"(w)
                 : "memory");
}

// 4-byte asynchronous global -> shared copy (no register holds the value in flight)
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Mark the node's 4x4x4 block active: a plain store (no round trip); k_compact_active turns
// the flags into the solve's list.
__device__ __forceinline__ void mark_node(const NodeBufs &nb, int i, int j, int k, const GridGeom &g)
{
    nb.flags[node_block(i, j, k, g)] = 1;
}

struct PState {
    int key, pid;
    uint32_t info;
    float o[3], v[3], s[6], e[6], rho, mass;
    float eqps, ep[6], dmg, smax;
};

template <bool HAS_DP>
__device__ __forceinline__ void store_state(const PView &P, long long i, const PState &st)
{
    P.ii(PF_KEY, i) = st.key;
    P.ii(PF_INFO, i) = (int)st.info;
    P.ii(PF_PID, i) = st.pid;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        P.f(PF_OX + k, i) = st.o[k];
        P.f(PF_VX + k, i) = st.v[k];
    }
#pragma unroll
    for (int k = 0; k < 6; k++) {
        P.f(PF_S0 + k, i) = st.s[k];
        P.f(PF_E0 + k, i) = st.e[k];
    }
    P.f(PF_RHO, i) = st.rho;
    P.f(PF_MASS, i) = st.mass;
    if (HAS_DP) {
        P.f(PF_EQPS, i) = st.eqps;
#pragma unroll
        for (int k = 0; k < 6; k++) P.f(PF_EP0 + k, i) = st.ep[k];
        P.f(PF_DMG, i) = st.dmg;
        P.f(PF_SMAX, i) = st.smax;
    }
}


// A particle whose cell key changed: its bit in the next re-sort's mover words (slot i of the
// order this step writes), and the word's count when the bit was clear
__device__ __forceinline__ void flag_mover(const StepArgs &a, long long i)
{
    const unsigned bit = 1u << (i & 31);
    if (!(atomicOr(&a.mover_mask[i >> 5], bit) & bit)) atomicAdd(&a.mover_cnt[i >> 5], 1);
}

// L2 prefetch of the segment a CTA takes next: the window of PF_WINDOW source slots that
// starts at the slot of the segment's first particle (the slab is in the order of the last
// sort, so a segment's particles sit close together there), for the fields [f0, f1), one
// bulk prefetch per field issued by thread 0.  A hint only: the window stays inside the
// slab, and a short segment costs some L2 space, not results.
constexpr long long PF_WINDOW = 512;
__device__ __forceinline__ void prefetch_next_segment(const PView &P, const int *perm, const int *seg_start, int nseg,
                                                      int next, int f0, int f1)
{
    if (threadIdx.x != 0 || next >= nseg) return;
    const long long s = seg_start[next];
    long long j0 = perm ? (long long)perm[s] : s;
    j0 &= ~3ll;  // 16-byte aligned
    long long len = min(PF_WINDOW, P.cap - j0);
    len &= ~3ll;
    if (len <= 0) return;
    for (int f = f0; f < f1; f++)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(&P.f(f, j0)), "r"((unsigned)(len * 4))
                     : "memory");
}

// ---------------------------------------------------------------------------------------
// Single-body P2G through a shared-memory node tile.  Gravity is added per node in the
// solve as m_node * g, which equals sum_p w m_p g (Extrapolation.cpp:226-278).
//
// A CTA owns one segment (the particles of one 4x4x4 cell block), whose stencils lie in the
// 6x6x6 node tile [4b, 4b+6).  Each chunk of particles is loaded in natural (coalesced)
// order and its GIMP weights and payload are staged in shared memory as pairs of
// neighbouring particles.  The particles of one cell share their 27 stencil nodes, so their
// sums are formed in registers, two particles per packed FP32x2 instruction, and added into
// the tile once per node and cell -- seven shared atomics per node per cell instead of per
// particle.

constexpr int PT = 6;                   // tile edge in nodes
constexpr int PT_NODES = PT * PT * PT;  // 216
constexpr int P2G_FIELDS = 7;           // m, px, py, pz, fx, fy, fz
constexpr int P2G_CH = 128;             // multi-body P2G: particles per chunk = threads per CTA

// Segment bounds when the keys are not freshly sorted: runs of one block can repeat, so
// the run ends at the first index after `base` whose block differs (per chunk).
__device__ __forceinline__ long long segment_chunk_end(const int *skey, long long n, int blk, long long base,
                                                       int chunk, long long *s_end)
{
    if (threadIdx.x == 0) *s_end = base + chunk;
    __syncthreads();
    const long long i = base + threadIdx.x;
    const bool inb = (int)threadIdx.x >= chunk || (i < n && (skey[i] >> CB_SHIFT) == blk);
    if (!inb) atomicMin((unsigned long long *)s_end, (unsigned long long)i);
    __syncthreads();
    const long long e = *s_end;
    __syncthreads();  // every thread has read s_end before thread 0 resets it
    return e;
}

__device__ __forceinline__ int seg_block(const int *skey, long long start) { return skey[start] >> CB_SHIFT; }

// packed FP32x2 arithmetic (sm_100 and later): one instruction for two particles
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

// Single-body P2G kernel.  A lane owns a column of three x nodes (jj, kk) of a run's stencil
// and a warp takes three runs at once (lanes 0-8, 9-17, 18-26), so one shared load of a
// staged pair serves the nine lanes of its run and the y/z factors multiply the payload once
// per column: per pair and lane the three x nodes each add S_x (m, m v) syz and
// G_x B + S_x C, with B = sigma_.x syz and C = sigma_.y G_y S_z + sigma_.z S_y G_z (the
// separable form of the stencil sums).  A CTA of PC_THREADS stages PC_CH particles, one pair
// per thread, about four full cells per warp and chunk.
#ifndef GY_PC_MINB
#define GY_PC_MINB 5  // 96 registers: five CTAs per SM
#endif
#ifndef GY_PC_UNROLL
#define GY_PC_UNROLL 1
#endif
constexpr int PC_UNROLL = GY_PC_UNROLL;
constexpr int PC_THREADS = 128;
constexpr int PC_CH = 2 * PC_THREADS;
// staged pair m sits at slot m + m / 8 of its row: the pairs the three groups of a warp read
// in one load (runs about a third of a chunk apart) then fall in different banks
__device__ __forceinline__ int pslot(int m) { return m + (m >> 3); }
constexpr int PC_NP = PC_THREADS + (PC_THREADS - 1) / 8;  // 143 float4, odd
constexpr int PC_WARPS = PC_THREADS / 32;

// segment bounds of an unsorted chunk with two positions per thread
__device__ __forceinline__ long long segment_chunk_end2(const int *skey, long long n, int blk, long long base,
                                                        long long *s_end)
{
    if (threadIdx.x == 0) *s_end = base + PC_CH;
    __syncthreads();
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const long long i = base + 2 * threadIdx.x + h;
        if (!(i < n && (skey[i] >> CB_SHIFT) == blk)) atomicMin((unsigned long long *)s_end, (unsigned long long)i);
    }
    __syncthreads();
    const long long e = *s_end;
    __syncthreads();
    return e;
}

struct ColAcc {
    float2 m[3], px[3], py[3], pz[3], fx[3], fy[3], fz[3];
};
// heat conduction sums of a column (only with THERMAL): node temperature sum S T m c and
// sum grad S . ((m / rho) k grad T) (the node rate with its sign flipped)
struct ColTh {
    float2 t[3], r[3];
};

// staged pair mp of the run, halves selected by mk (1 = the particle belongs to the run)
template <bool MASKED, bool THERMAL>
__device__ __forceinline__ void col_pair(ColAcc &A, const float4 (*W)[PC_NP], const float4 (*Q)[PC_NP], int mp,
                                         int jj, int kk, float2 mk, ColTh &T, const float4 (*QT)[PC_NP])
{
    const int sl = pslot(mp);
    const float4 Y = W[3 + jj][sl], Z = W[6 + kk][sl];
    const float4 q0 = Q[0][sl], q1 = Q[1][sl], q2 = Q[2][sl], q3 = Q[3][sl], q4 = Q[4][sl];
    float2 syz = mul2(lo2(Y), lo2(Z)), gyz = mul2(hi2(Y), lo2(Z)), syg = mul2(lo2(Y), hi2(Z));
    if (MASKED) {
        syz = mul2(syz, mk);
        gyz = mul2(gyz, mk);
        syg = mul2(syg, mk);
    }
    const float2 mS = mul2(syz, lo2(q0)), pX = mul2(syz, hi2(q0)), pY = mul2(syz, lo2(q1)), pZ = mul2(syz, hi2(q1));
    const float2 s0 = lo2(q2), s1 = hi2(q2), s2 = lo2(q3), s3 = hi2(q3), s4 = lo2(q4), s5 = hi2(q4);
    const float2 Bx = mul2(s0, syz), By = mul2(s3, syz), Bz = mul2(s5, syz);
    const float2 Cx = fma2(s3, gyz, mul2(s5, syg)), Cy = fma2(s1, gyz, mul2(s4, syg));
    const float2 Cz = fma2(s4, gyz, mul2(s2, syg));
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float4 X = W[i][sl];
        const float2 Sx = lo2(X), Gx = hi2(X);
        A.m[i] = fma2(Sx, mS, A.m[i]);
        A.px[i] = fma2(Sx, pX, A.px[i]);
        A.py[i] = fma2(Sx, pY, A.py[i]);
        A.pz[i] = fma2(Sx, pZ, A.pz[i]);
        A.fx[i] = fma2(Gx, Bx, fma2(Sx, Cx, A.fx[i]));
        A.fy[i] = fma2(Gx, By, fma2(Sx, Cy, A.fy[i]));
        A.fz[i] = fma2(Gx, Bz, fma2(Sx, Cz, A.fz[i]));
    }
    if (THERMAL) {
        // QT[0] = (T m c, T m c', g_x, g_x'), QT[1] = (g_y, g_y', g_z, g_z') with g = (m/rho) k grad T / h
        const float4 t0 = QT[0][sl], t1 = QT[1][sl];
        const float2 tS = mul2(syz, lo2(t0)), Bt = mul2(hi2(t0), syz);
        const float2 Ct = fma2(lo2(t1), gyz, mul2(hi2(t1), syg));
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float4 X = W[i][sl];
            T.t[i] = fma2(lo2(X), tS, T.t[i]);
            T.r[i] = fma2(hi2(X), Bt, fma2(lo2(X), Ct, T.r[i]));
        }
    }
}

// THERMAL adds the heat conduction terms of Extrapolation.cpp:280-283 (single body: no rigid
// particles): two more node fields in the tile, flushed into tnode, from the particle
// temperature and gradient kept by insertion index in therm.
template <bool THERMAL>
__global__ void __launch_bounds__(PC_THREADS, GY_PC_MINB) k_p2g_cols(PView P, const int *perm, const int *skey, long long n,
                                                         const int *seg_start, const int *nseg_ptr, int sorted,
                                                         NodeBufs nb, GridGeom g, const float4 *therm, float2 *tnode,
                                                         const DevMaterial *mats)
{
    constexpr int NF = P2G_FIELDS + (THERMAL ? 2 : 0);
    __shared__ float tile[NF * PT_NODES];
    __shared__ float4 QTs[THERMAL ? 2 * PC_NP : 1];
    float4 (*QT)[PC_NP] = reinterpret_cast<float4 (*)[PC_NP]>(QTs);  // used only with THERMAL
    __shared__ float4 W[9][PC_NP];    // pair m: (S, S', G, G') per axis/stencil node
    __shared__ float4 Q[5][PC_NP];    // pair m: (m, m'), (m vx, ..'), (m vy), (m vz), V sigma / h x6
    __shared__ int run_start[PC_CH + 1];
    __shared__ int run_cell[PC_CH];
    __shared__ int wcount[PC_WARPS];
    __shared__ long long s_end;
    const int nseg = *nseg_ptr;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    // lane -> (run group, jj, kk); lanes 27..31 shadow lane 26 and skip the atomics
    const int grp = lane < 27 ? lane / 9 : 2, jk = lane < 27 ? lane % 9 : 8;
    const int jj = jk % 3, kk = jk / 3;
    const bool scatter_lane = lane < 27;
    const float2 z2 = make_float2(0.f, 0.f);
    for (int sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
        prefetch_next_segment(P, perm, seg_start, nseg, sgi + gridDim.x, PF_OX, PF_S5 + 1);
        prefetch_next_segment(P, perm, seg_start, nseg, sgi + gridDim.x, PF_RHO, PF_MASS + 1);
        const long long start = seg_start[sgi];
        const int blk = seg_block(skey, start);
        int bx, by, bz;
        decode_block(blk, g, bx, by, bz);
        const int tox = bx * CB, toy = by * CB, toz = g.is3d ? bz * CB : 0;
        for (int t = tid; t < NF * PT_NODES; t += PC_THREADS) tile[t] = 0.f;
        for (long long base = start;; base += PC_CH) {
            const long long ia = base + 2 * tid, ib = ia + 1;
            int cnt, ka = -1, kb = -1, kp = -1;
            long long ja = 0, jb = 0;
            if (sorted) {
                // the segment's particles in this chunk are a prefix of it; the barriers also
                // end the previous chunk's use of the staging arrays
                ka = ia < n ? skey[ia] : -1;
                kb = ib < n ? skey[ib] : -1;
                kp = (ia < n && tid > 0) ? skey[ia - 1] : -1;
                ja = ia < n ? perm[ia] : 0;
                jb = ib < n ? perm[ib] : 0;
                cnt = __syncthreads_count(ia < n && (ka >> CB_SHIFT) == blk);
                cnt += __syncthreads_count(ib < n && (kb >> CB_SHIFT) == blk);
            } else {
                cnt = (int)min((long long)PC_CH, segment_chunk_end2(skey, n, blk, base, &s_end) - base);
                if (2 * tid < cnt) {
                    ka = skey[ia];
                    kp = tid > 0 ? skey[ia - 1] : -1;
                }
                if (2 * tid + 1 < cnt) kb = skey[ib];
                ja = ia;
                jb = ib;
            }
            if (cnt <= 0) break;
            // ---- stage the pair (2 tid, 2 tid + 1); a particle past the chunk stages zeros ----
            const int st = pslot(tid);
            const bool va = 2 * tid < cnt, vb = 2 * tid + 1 < cnt;
            const int ca = ka & 63, cb = kb & 63;  // cell inside the block: (lz*4 + ly)*4 + lx
            const bool ha = va && (tid == 0 || (kp & 63) != ca);
            const bool hb = vb && cb != ca;
            if (va) {
                float Sa[3], Ga[3], Sb[3] = {0.f, 0.f, 0.f}, Gb[3] = {0.f, 0.f, 0.f};
                gimp_axis(P.f(PF_OX, ja), g, Sa, Ga);
                if (vb) gimp_axis(P.f(PF_OX, jb), g, Sb, Gb);
#pragma unroll
                for (int k = 0; k < 3; k++) W[k][st] = make_float4(Sa[k], Sb[k], Ga[k], Gb[k]);
                gimp_axis(P.f(PF_OY, ja), g, Sa, Ga);
                if (vb) gimp_axis(P.f(PF_OY, jb), g, Sb, Gb);
#pragma unroll
                for (int k = 0; k < 3; k++) W[3 + k][st] = make_float4(Sa[k], Sb[k], Ga[k], Gb[k]);
                if (g.is3d) {
                    gimp_axis(P.f(PF_OZ, ja), g, Sa, Ga);
                    if (vb) gimp_axis(P.f(PF_OZ, jb), g, Sb, Gb);
                } else {
                    Sa[0] = 1.f; Sa[1] = 0.f; Sa[2] = 0.f; Ga[0] = 0.f; Ga[1] = 0.f; Ga[2] = 0.f;
                    if (vb) {
                        Sb[0] = 1.f; Sb[1] = 0.f; Sb[2] = 0.f; Gb[0] = 0.f; Gb[1] = 0.f; Gb[2] = 0.f;
                    }
                }
#pragma unroll
                for (int k = 0; k < 3; k++) W[6 + k][st] = make_float4(Sa[k], Sb[k], Ga[k], Gb[k]);
                const float ma = P.f(PF_MASS, ja), mb = vb ? P.f(PF_MASS, jb) : 0.f;
                const float sca = (ma / P.f(PF_RHO, ja)) * g.inv_h;  // V sigma with the gradient's 1/h
                const float scb = vb ? (mb / P.f(PF_RHO, jb)) * g.inv_h : 0.f;
                const float vxb = vb ? P.f(PF_VX, jb) : 0.f, vyb = vb ? P.f(PF_VY, jb) : 0.f;
                const float vzb = vb ? P.f(PF_VZ, jb) : 0.f;
                Q[0][st] = make_float4(ma, mb, ma * P.f(PF_VX, ja), mb * vxb);
                Q[1][st] = make_float4(ma * P.f(PF_VY, ja), mb * vyb, ma * P.f(PF_VZ, ja), mb * vzb);
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    const float a0 = P.f(PF_S0 + 2 * k, ja) * sca, a1 = P.f(PF_S0 + 2 * k + 1, ja) * sca;
                    const float b0 = vb ? P.f(PF_S0 + 2 * k, jb) * scb : 0.f;
                    const float b1 = vb ? P.f(PF_S0 + 2 * k + 1, jb) * scb : 0.f;
                    Q[2 + k][st] = make_float4(a0, b0, a1, b1);
                }
                if (THERMAL) {
                    const DevMaterial &Ma = mats[info_mat((uint32_t)P.ii(PF_INFO, ja))];
                    const float4 tha = therm[P.ii(PF_PID, ja)];
                    const float vka = (ma / P.f(PF_RHO, ja)) * Ma.k_th * g.inv_h;
                    float4 thb = make_float4(0.f, 0.f, 0.f, 0.f);
                    float cb = 0.f, vkb = 0.f;
                    if (vb) {
                        const DevMaterial &Mb = mats[info_mat((uint32_t)P.ii(PF_INFO, jb))];
                        thb = therm[P.ii(PF_PID, jb)];
                        cb = Mb.c_th;
                        vkb = (mb / P.f(PF_RHO, jb)) * Mb.k_th * g.inv_h;
                    }
                    QT[0][st] = make_float4(tha.x * ma * Ma.c_th, thb.x * mb * cb, vka * tha.y, vkb * thb.y);
                    QT[1][st] = make_float4(vka * tha.z, vkb * thb.z, vka * tha.w, vkb * thb.w);
                }
            } else {
                const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int k = 0; k < 9; k++) W[k][st] = z4;
#pragma unroll
                for (int k = 0; k < 5; k++) Q[k][st] = z4;
                if (THERMAL) {
                    QT[0][st] = z4;
                    QT[1][st] = z4;
                }
            }
            // ---- runs of equal cell, in order: run r is [run_start[r], run_start[r+1]) ----
            const unsigned ba = __ballot_sync(0xffffffffu, ha), bb = __ballot_sync(0xffffffffu, hb);
            if (lane == 0) wcount[warp] = __popc(ba) + __popc(bb);
            __syncthreads();
            int wbase = 0, R = 0;
#pragma unroll
            for (int w2 = 0; w2 < PC_WARPS; w2++) {
                const int c = wcount[w2];
                wbase += (w2 < warp) ? c : 0;
                R += c;
            }
            int ri = wbase + __popc(ba & lt) + __popc(bb & lt);
            if (ha) {
                run_start[ri] = 2 * tid;
                run_cell[ri] = ca;
                ri++;
            }
            if (hb) {
                run_start[ri] = 2 * tid + 1;
                run_cell[ri] = cb;
            }
            if (tid == 0) run_start[R] = cnt;
            __syncthreads();
            // ---- three runs per warp, lane = x column (jj, kk) of its run.  Triple t holds
            // runs t, t + T, t + 2T: cells a third of the chunk apart, whose stencils overlap
            // little, so the groups' shared atomics seldom meet on one node ----
            const int T = (R + 2) / 3;
            for (int t3 = warp; t3 < T; t3 += PC_WARPS) {
                const int r = t3 + grp * T;
                const bool rv = r < R;
                const int p0 = rv ? run_start[r] : 0, p1 = rv ? run_start[r + 1] : 0;
                ColAcc A;
                ColTh TH;
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    A.m[i] = A.px[i] = A.py[i] = A.pz[i] = A.fx[i] = A.fy[i] = A.fz[i] = z2;
                    TH.t[i] = TH.r[i] = z2;
                }
                const bool full = rv && p1 - p0 == 8 && !(p0 & 1);
                if (__all_sync(0xffffffffu, full)) {
                    // three full cells (psep = cellsize / 2) on pair boundaries: four pairs each
#pragma unroll PC_UNROLL
                    for (int k = 0; k < 4; k++) col_pair<false, THERMAL>(A, W, Q, (p0 >> 1) + k, jj, kk, z2, TH, QT);
                } else {
                    const int m0 = p0 >> 1, np = rv ? ((p1 + 1) >> 1) - m0 : 0;
                    const int maxp = __reduce_max_sync(0xffffffffu, np);
                    for (int k = 0; k < maxp; k++) {
                        const int mp = m0 + min(k, max(np - 1, 0));
                        const int q = 2 * mp;
                        const float2 mk = make_float2(k < np && q >= p0 && q < p1 ? 1.f : 0.f,
                                                      k < np && q + 1 >= p0 && q + 1 < p1 ? 1.f : 0.f);
                        col_pair<true, THERMAL>(A, W, Q, mp, jj, kk, mk, TH, QT);
                    }
                }
                if (!scatter_lane || !rv) continue;
                const int cell = run_cell[r];
                const int li = cell & 3, lj = (cell >> 2) & 3, lk = cell >> 4;
                const int t0 = ((lk + kk) * PT + (lj + jj)) * PT + li;
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const float am = A.m[i].x + A.m[i].y;
                    // a node outside every particle's support has no weight and no gradient
                    if (am == 0.f) continue;
                    const int t = t0 + i;
                    atomicAdd(&tile[0 * PT_NODES + t], am);
                    atomicAdd(&tile[1 * PT_NODES + t], A.px[i].x + A.px[i].y);
                    atomicAdd(&tile[2 * PT_NODES + t], A.py[i].x + A.py[i].y);
                    atomicAdd(&tile[3 * PT_NODES + t], A.pz[i].x + A.pz[i].y);
                    atomicAdd(&tile[4 * PT_NODES + t], -(A.fx[i].x + A.fx[i].y));
                    atomicAdd(&tile[5 * PT_NODES + t], -(A.fy[i].x + A.fy[i].y));
                    atomicAdd(&tile[6 * PT_NODES + t], -(A.fz[i].x + A.fz[i].y));
                    if (THERMAL) {
                        atomicAdd(&tile[7 * PT_NODES + t], TH.t[i].x + TH.t[i].y);
                        atomicAdd(&tile[8 * PT_NODES + t], -(TH.r[i].x + TH.r[i].y));
                    }
                }
            }
            if (cnt < PC_CH) break;
        }
        __syncthreads();
        // ---- flush the tile: two vector reductions per touched node ----
        for (int t = tid; t < PT_NODES; t += PC_THREADS) {
            const float m = tile[t], px = tile[PT_NODES + t], py = tile[2 * PT_NODES + t], pz = tile[3 * PT_NODES + t];
            const float fx = tile[4 * PT_NODES + t], fy = tile[5 * PT_NODES + t], fz = tile[6 * PT_NODES + t];
            if (m == 0.f && px == 0.f && py == 0.f && pz == 0.f && fx == 0.f && fy == 0.f && fz == 0.f) continue;
            const int ni = tox + t % PT, nj = toy + (t / PT) % PT, nk = toz + t / (PT * PT);
            if (ni >= g.nx || nj >= g.ny || nk >= g.nz) continue;
            const int nd = node_index(ni, nj, nk, g);
            red_add4(&nb.acc0[nd], m, px, py, pz);
            red_add4(&nb.acc1[nd], fx, fy, fz, 0.f);
            if (THERMAL) {
                atomicAdd(&tnode[nd].x, tile[7 * PT_NODES + t]);
                atomicAdd(&tnode[nd].y, tile[8 * PT_NODES + t]);
            }
            mark_node(nb, ni, nj, nk, g);
        }
        __syncthreads();
    }
}

// Single-body P2G with z-plane lanes.  The segments, chunks and runs of equal cell are
// those of k_p2g_cols; the work of a run is split over three lanes instead of nine: lane kk
// of a run's group owns the 3x3 stencil nodes (i, j, kk) of its plane and sums the run's
// particles into 63 registers (m, p, f of nine nodes, packed along the fields), then adds them
// into the node tile once per run.  Ten groups share a warp (lanes 0-29), one particle per
// group and step, so a particle's staged weights and payload reach three lanes rather than
// nine -- the shared-memory loads per particle, which bound the column kernel, drop about
// threefold -- at the cost of recomputing the y/z factors per lane.  Staged per particle
// (rows swizzled q + q/8 so the ten groups' rows spread over the banks):
//   A = (Sx0, Sx1, Sx2, Gx0)  B = (Gx1, Gx2, Sy0, Sy1)  C = (Sy2, Gy0, Gy1, Gy2)
//   D = (m, m vx, m vy, m vz) E = (s0, s3, s5, s4)      F = (s3, s1, s2, -)
//   Z[kk] = (Sz_kk, Gz_kk),   s = V sigma / h in the order xx yy zz xy yz xz,
// laid out so that every packed FP32x2 operand is a stored pair.
#ifndef GY_PP_MINB
#define GY_PP_MINB 5  // 96 registers (a few bytes spilled): five CTAs per SM
#endif
constexpr int PP_THREADS = 128;
constexpr int PP_GPW = 10;                              // lane groups per warp
constexpr int PP_GROUPS = PP_GPW * (PP_THREADS / 32);   // 40
constexpr int PP_CH = 2 * PP_THREADS;                   // particles per chunk (a pair per thread)
constexpr int PP_ROWS = PP_CH + PP_CH / 8;
__device__ __forceinline__ int pp_row(int q) { return q + (q >> 3); }

static_assert(PP_CH == PC_CH, "the chunk bounds helper assumes two particles per thread");


__device__ __forceinline__ float2 dup2(float x) { return make_float2(x, x); }

// MULTI: the same kernel on a multi-body problem, for the segments it can take whole -- every
// particle deformable and of one object, every tile node with that object as its only body (or
// none) -- where a node's slot-0 mass, momentum and force equal its centre-of-mass sums and no
// normal is read (the solve takes a node's normal only where two bodies meet, and G2P only when
// normals are tracked, in which case this path is not used).  It adds gravity per node (the
// multi-body solve does not) and flushes into the centre-of-mass and slot-0 accumulators.  A
// segment that fails the test, at its start or at any chunk, is appended to `defer`, its tile
// dropped, and k_p2g_multi_tiled takes it.
// THERMAL (single body): the heat conduction sums as in k_p2g_cols -- per node the temperature
// sum S T m c and the rate sum grad S . ((m / rho) k grad T / h) -- staged as one more float4
// per particle and two more tile fields, at four CTAs per SM.
#ifndef GY_PP_MINB_TH
#define GY_PP_MINB_TH 4
#endif
template <bool MULTI, bool THERMAL = false>
__global__ void __launch_bounds__(PP_THREADS, THERMAL ? GY_PP_MINB_TH : GY_PP_MINB)
    k_p2g_planes(PView P, const int *perm, const int *skey, long long n, const int *seg_start, const int *nseg_ptr,
                 int sorted, NodeBufs nb, StepArgs a, int *defer, int *ndefer, const float4 *therm = nullptr,
                 float2 *tnode = nullptr)
{
    constexpr int TF = P2G_FIELDS + (THERMAL ? 2 : 0);  // tile fields
    __shared__ float tile[TF * PT_NODES];
    __shared__ float4 SA[PP_ROWS], SB[PP_ROWS], SC[PP_ROWS], SD[PP_ROWS], SE[PP_ROWS], SF[PP_ROWS];
    __shared__ float4 SG[THERMAL ? PP_ROWS : 1];  // (T m c, g_x, g_y, g_z), g = (m / rho) k grad T / h
    __shared__ float2 SZ[3][PP_ROWS];
    __shared__ int run_start[PP_CH + 1];
    __shared__ int run_cell[PP_CH];
    __shared__ int wcount[PP_THREADS / 32];
    __shared__ long long s_end;
    const GridGeom &g = a.g;
    const int nseg = *nseg_ptr;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int grp = lane / 3, kk = lane - 3 * grp;      // lanes 30, 31: group 10, no run
    const float2 z2 = make_float2(0.f, 0.f);
    for (int sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
        prefetch_next_segment(P, perm, seg_start, nseg, sgi + gridDim.x, PF_OX, PF_S5 + 1);
        prefetch_next_segment(P, perm, seg_start, nseg, sgi + gridDim.x, PF_RHO, PF_MASS + 1);
        const long long start = seg_start[sgi];
        const int blk = seg_block(skey, start);
        int bx, by, bz;
        decode_block(blk, g, bx, by, bz);
        const int tox = bx * CB, toy = by * CB, toz = g.is3d ? bz * CB : 0;
        int obj0 = 0, tb = -1;
        if (MULTI) {
            // the same values in every thread: the segment's first particle and its block's tile
            const uint32_t info0 = (uint32_t)P.ii(PF_INFO, sorted ? perm[start] : start);
            obj0 = info_obj(info0);
            tb = nb.block_body[blk];
            if ((info0 & INFO_RIGID) || (tb != obj0 && tb != -1)) {
                if (tid == 0) defer[atomicAdd(ndefer, 1)] = (int)start;
                continue;
            }
        }
        for (int t = tid; t < TF * PT_NODES; t += PP_THREADS) tile[t] = 0.f;
        bool dropped = false;
        for (long long base = start;; base += PP_CH) {
            const long long ia = base + 2 * tid, ib = ia + 1;
            int cnt, ka = -1, kb = -1, kp = -1;
            long long ja = 0, jb = 0;
            if (sorted) {
                ka = ia < n ? skey[ia] : -1;
                kb = ib < n ? skey[ib] : -1;
                kp = (ia < n && tid > 0) ? skey[ia - 1] : -1;
                ja = ia < n ? perm[ia] : 0;
                jb = ib < n ? perm[ib] : 0;
                cnt = __syncthreads_count(ia < n && (ka >> CB_SHIFT) == blk);
                cnt += __syncthreads_count(ib < n && (kb >> CB_SHIFT) == blk);
            } else {
                cnt = (int)min((long long)PP_CH, segment_chunk_end2(skey, n, blk, base, &s_end) - base);
                if (2 * tid < cnt) {
                    ka = skey[ia];
                    kp = tid > 0 ? skey[ia - 1] : -1;
                }
                if (2 * tid + 1 < cnt) kb = skey[ib];
                ja = ia;
                jb = ib;
            }
            if (cnt <= 0) break;
            // ---- stage particles 2 tid and 2 tid + 1 of the chunk ----
            bool mine_ok = true;
#pragma unroll
            for (int h2 = 0; h2 < 2; h2++) {
                const int q = 2 * tid + h2;
                if (q >= cnt) break;
                const long long j = h2 ? jb : ja;
                const int row = pp_row(q);
                if (MULTI) {
                    const uint32_t info = (uint32_t)P.ii(PF_INFO, j);
                    mine_ok = mine_ok && !(info & INFO_RIGID) && info_obj(info) == obj0;
                }
                float Sx[3], Gx[3], Sy[3], Gy[3], Sz[3], Gz[3];
                gimp_axis(P.f(PF_OX, j), g, Sx, Gx);
                gimp_axis(P.f(PF_OY, j), g, Sy, Gy);
                if (g.is3d) {
                    gimp_axis(P.f(PF_OZ, j), g, Sz, Gz);
                } else {
                    Sz[0] = 1.f; Sz[1] = 0.f; Sz[2] = 0.f; Gz[0] = 0.f; Gz[1] = 0.f; Gz[2] = 0.f;
                }
                const float m = P.f(PF_MASS, j);
                const float sc = (m / P.f(PF_RHO, j)) * g.inv_h;  // V sigma with the gradient's 1/h
                const float s0 = P.f(PF_S0, j) * sc, s1 = P.f(PF_S1, j) * sc, s2 = P.f(PF_S2, j) * sc;
                const float s3 = P.f(PF_S3, j) * sc, s4 = P.f(PF_S4, j) * sc, s5 = P.f(PF_S5, j) * sc;
                SA[row] = make_float4(Sx[0], Sx[1], Sx[2], Gx[0]);
                SB[row] = make_float4(Gx[1], Gx[2], Sy[0], Sy[1]);
                SC[row] = make_float4(Sy[2], Gy[0], Gy[1], Gy[2]);
                SD[row] = make_float4(m, m * P.f(PF_VX, j), m * P.f(PF_VY, j), m * P.f(PF_VZ, j));
                SE[row] = make_float4(s0, s3, s5, s4);
                SF[row] = make_float4(s3, s1, s2, 0.f);
                if (THERMAL) {
                    const DevMaterial &Mt = a.mats[info_mat((uint32_t)P.ii(PF_INFO, j))];
                    const float4 th = therm[P.ii(PF_PID, j)];
                    const float vk = (m / P.f(PF_RHO, j)) * Mt.k_th * g.inv_h;
                    SG[row] = make_float4(th.x * m * Mt.c_th, vk * th.y, vk * th.z, vk * th.w);
                }
#pragma unroll
                for (int z = 0; z < 3; z++) SZ[z][row] = make_float2(Sz[z], Gz[z]);
            }
            // ---- runs of equal cell, in order: run r is [run_start[r], run_start[r+1]) ----
            const bool va = 2 * tid < cnt, vb = 2 * tid + 1 < cnt;
            const int ca = ka & 63, cb = kb & 63;
            const bool ha = va && (tid == 0 || (kp & 63) != ca);
            const bool hb = vb && cb != ca;
            const unsigned ba = __ballot_sync(0xffffffffu, ha), bb = __ballot_sync(0xffffffffu, hb);
            if (lane == 0) wcount[warp] = __popc(ba) + __popc(bb);
            if (MULTI) {
                if (!__syncthreads_and(mine_ok)) {
                    dropped = true;
                    break;
                }
            } else {
                __syncthreads();
            }
            int wbase = 0, R = 0;
#pragma unroll
            for (int w2 = 0; w2 < PP_THREADS / 32; w2++) {
                const int c = wcount[w2];
                wbase += (w2 < warp) ? c : 0;
                R += c;
            }
            int ri = wbase + __popc(ba & lt) + __popc(bb & lt);
            if (ha) {
                run_start[ri] = 2 * tid;
                run_cell[ri] = ca;
                ri++;
            }
            if (hb) {
                run_start[ri] = 2 * tid + 1;
                run_cell[ri] = cb;
            }
            if (tid == 0) run_start[R] = cnt;
            __syncthreads();
            // ---- ten runs per warp and round, three plane lanes per run ----
            for (int rb = warp * PP_GPW; rb < R; rb += PP_GROUPS) {
                const int r = rb + grp;
                const bool rv = grp < PP_GPW && r < R;
                const int p0 = rv ? run_start[r] : 0, len = rv ? run_start[r + 1] - p0 : 0;
                const int maxlen = __reduce_max_sync(0xffffffffu, len);
                float2 amp[3][3], app[3][3], afxy[3][3];
                float afz[3][3];
                float atT[THERMAL ? 3 : 1][3], atR[THERMAL ? 3 : 1][3];  // THERMAL: temperature and rate sums
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        amp[i][j] = app[i][j] = afxy[i][j] = z2;
                        afz[i][j] = 0.f;
                        if (THERMAL) atT[i][j] = atR[i][j] = 0.f;
                    }
                for (int k = 0; k < maxlen; k++) {
                    const int row = pp_row(p0 + min(k, max(len - 1, 0)));
                    const float4 A = SA[row], B = SB[row], C = SC[row], D = SD[row], E = SE[row], F = SF[row];
                    float2 Z = SZ[kk][row];
                    if (k >= len) Z = z2;  // past the run (or no run): the particle adds nothing
                    float4 TG = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (THERMAL) TG = SG[row];
                    const float Sx[3] = {A.x, A.y, A.z}, Gx[3] = {A.w, B.x, B.y};
                    const float Sy[3] = {B.z, B.w, C.x}, Gy[3] = {C.y, C.z, C.w};
                    const float2 mvx = make_float2(D.x, D.y), mvyz = make_float2(D.z, D.w);
                    const float2 s03 = make_float2(E.x, E.y), s54 = make_float2(E.z, E.w);
                    const float2 s31 = make_float2(F.x, F.y);
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        const float syz = Sy[j] * Z.x, gyz = Gy[j] * Z.x, syg = Sy[j] * Z.y;
                        const float2 syz2 = dup2(syz);
                        const float2 mp = mul2(syz2, mvx);                    // (m, m vx) S_y S_z
                        const float2 pp = mul2(syz2, mvyz);                   // (m vy, m vz) S_y S_z
                        const float2 Bxy = mul2(syz2, s03);                   // (s0, s3) S_y S_z
                        const float Bz = E.z * syz;                           // s5 S_y S_z
                        const float2 Cxy = fma2(dup2(gyz), s31, mul2(dup2(syg), s54));  // (s3, s1) G_y S_z + (s5, s4) S_y G_z
                        const float Cz = fmaf(E.w, gyz, F.z * syg);           // s4 G_y S_z + s2 S_y G_z
#pragma unroll
                        for (int i = 0; i < 3; i++) {
                            const float2 sx = dup2(Sx[i]), gx = dup2(Gx[i]);
                            amp[i][j] = fma2(sx, mp, amp[i][j]);
                            app[i][j] = fma2(sx, pp, app[i][j]);
                            afxy[i][j] = fma2(gx, Bxy, fma2(sx, Cxy, afxy[i][j]));
                            afz[i][j] = fmaf(Gx[i], Bz, fmaf(Sx[i], Cz, afz[i][j]));
                        }
                        if (THERMAL) {
                            const float tS = syz * TG.x, Bt = TG.y * syz, Ct = fmaf(TG.z, gyz, TG.w * syg);
#pragma unroll
                            for (int i = 0; i < 3; i++) {
                                atT[i][j] = fmaf(Sx[i], tS, atT[i][j]);
                                atR[i][j] = fmaf(Gx[i], Bt, fmaf(Sx[i], Ct, atR[i][j]));
                            }
                        }
                    }
                }
                if (!rv) continue;
                const int cell = run_cell[r];
                const int li = cell & 3, lj = (cell >> 2) & 3, lk = cell >> 4;
#pragma unroll
                for (int j = 0; j < 3; j++)
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        // a node outside every particle's support has no weight and no gradient
                        if (amp[i][j].x == 0.f) continue;
                        const int t = ((lk + kk) * PT + (lj + j)) * PT + li + i;
                        atomicAdd(&tile[0 * PT_NODES + t], amp[i][j].x);
                        atomicAdd(&tile[1 * PT_NODES + t], amp[i][j].y);
                        atomicAdd(&tile[2 * PT_NODES + t], app[i][j].x);
                        atomicAdd(&tile[3 * PT_NODES + t], app[i][j].y);
                        atomicAdd(&tile[4 * PT_NODES + t], -afxy[i][j].x);
                        atomicAdd(&tile[5 * PT_NODES + t], -afxy[i][j].y);
                        atomicAdd(&tile[6 * PT_NODES + t], -afz[i][j]);
                        if (THERMAL) {
                            atomicAdd(&tile[7 * PT_NODES + t], atT[i][j]);
                            atomicAdd(&tile[8 * PT_NODES + t], -atR[i][j]);
                        }
                    }
            }
            if (cnt < PP_CH) break;
        }
        if (MULTI && dropped) {
            // another object or a rigid particle: the general kernel takes the whole segment
            if (tid == 0) defer[atomicAdd(ndefer, 1)] = (int)start;
            continue;
        }
        __syncthreads();
        // ---- flush the tile: two vector reductions per touched node ----
        float grav[3] = {0.f, 0.f, 0.f};
        if (MULTI)
            for (int c = 0; c < 3; c++) grav[c] = __ldg(&a.sc->gravity[c]);
        for (int t = tid; t < PT_NODES; t += PP_THREADS) {
            const float m = tile[t], px = tile[PT_NODES + t], py = tile[2 * PT_NODES + t], pz = tile[3 * PT_NODES + t];
            float fx = tile[4 * PT_NODES + t], fy = tile[5 * PT_NODES + t], fz = tile[6 * PT_NODES + t];
            if (m == 0.f && px == 0.f && py == 0.f && pz == 0.f && fx == 0.f && fy == 0.f && fz == 0.f) continue;
            const int ni = tox + t % PT, nj = toy + (t / PT) % PT, nk = toz + t / (PT * PT);
            if (ni >= g.nx || nj >= g.ny || nk >= g.nz) continue;
            const int nd = node_index(ni, nj, nk, g);
            if (MULTI) {
                const bool slot0 = tb >= 0 && __ldg(&nb.body[nd].x) >= 0;
                // the multi-body step adds gravity in P2G, as sum w m g (Extrapolation.cpp:226-278)
                fx += m * grav[0];
                fy += m * grav[1];
                fz += m * grav[2];
                if (slot0) {
                    red_add4(&nb.bacc0[0][nd], m, px, py, pz);
                    red_add4(&nb.bacc1[0][nd], fx, fy, fz, 0.f);
                }
            }
            red_add4(&nb.acc0[nd], m, px, py, pz);
            red_add4(&nb.acc1[nd], fx, fy, fz, 0.f);
            if (THERMAL) {
                atomicAdd(&tnode[nd].x, tile[7 * PT_NODES + t]);
                atomicAdd(&tnode[nd].y, tile[8 * PT_NODES + t]);
            }
            mark_node(nb, ni, nj, nk, g);
        }
        __syncthreads();
    }
}

// Multi-body P2G through a shared-memory node tile: segments, staging and runs of equal cell
// as in the single-body kernel, with a warp taking one run at a time (lane k = stencil node
// k), one particle per step, and, per node, the centre-of-mass fields plus the two body
// slots (mass, momentum, force, normal).  A lane's body slot for a particle follows the node's
// body pair (Extrapolation.cpp:191-198) read once per segment into shared memory.
constexpr int MB_FIELDS = 27;                 // COM m, p(3), f(3); slot s: m, p(3), f(3), n(3)
constexpr int MB_NP = P2G_CH + 1;             // staged row length; odd, so rows fall in other banks

__global__ void __launch_bounds__(P2G_CH) k_p2g_multi_tiled(PView P, const int *perm, const int *skey, long long n,
                                                            const int *seg_start, const int *nseg_ptr, int sorted,
                                                            NodeBufs nb, StepArgs a)
{
    __shared__ float tile[MB_FIELDS * PT_NODES];
    __shared__ int2 tbody[PT_NODES];
    __shared__ float2 W[9][MB_NP];    // (S, G) per axis/stencil node and particle
    __shared__ float4 Q0[P2G_CH];     // m, m v
    __shared__ float4 Q1[P2G_CH];     // V sigma / h: xx, yy, zz, xy
    __shared__ float4 Q2[P2G_CH];     // V sigma / h: yz, xz; normal volume / h; object | rigid << 16
    __shared__ int cellof[P2G_CH];
    __shared__ int run_start[P2G_CH + 1];
    __shared__ int wcount[P2G_CH / 32];
    __shared__ long long s_end;
    const GridGeom &g = a.g;
    const int nseg = *nseg_ptr;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ii = lane % 3, jj = (lane / 3) % 3, kk = min(lane / 9, 2);
    const bool scatter_lane = lane < 27;
    const float grx = a.sc->gravity[0], gry = a.sc->gravity[1], grz = a.sc->gravity[2];
    const float init_vol = a.sc->init_volume;
    for (int sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
        const long long start = seg_start[sgi];
        const int blk = seg_block(skey, start);
        int bx, by, bz;
        decode_block(blk, g, bx, by, bz);
        const int tox = bx * CB, toy = by * CB, toz = g.is3d ? bz * CB : 0;
        // the object of the segment's first particle: while every particle met so far belongs
        // to it and is deformable, and every tile node has it as first body (or no body), each
        // particle's slot-0 sums equal its centre-of-mass sums, so the tile holds the latter
        // (and the slot-0 normals) only
        const int obj0 = info_obj((uint32_t)P.ii(PF_INFO, sorted ? perm[start] : start));
        __syncthreads();  // the previous segment's flush is done with the tile
        // the centre-of-mass fields and the slot-0 normals; the other slot fields are set
        // when the segment stops being one object's
        for (int t = tid; t < 7 * PT_NODES; t += P2G_CH) tile[t] = 0.f;
        for (int t = tid; t < 3 * PT_NODES; t += P2G_CH) tile[14 * PT_NODES + t] = 0.f;
        bool tile_one = true;
        for (int t = tid; t < PT_NODES; t += P2G_CH) {
            const int ni = tox + t % PT, nj = toy + (t / PT) % PT, nk = toz + t / (PT * PT);
            const int2 pr = (ni < g.nx && nj < g.ny && nk < g.nz) ? nb.body[node_index(ni, nj, nk, g)] : make_int2(-1, -1);
            tbody[t] = pr;
            tile_one = tile_one && (pr.x == obj0 || pr.x == -1);
        }
        bool uni = __syncthreads_and(tile_one) != 0;
        if (!uni)
            for (int t = tid; t < PT_NODES; t += P2G_CH) {
#pragma unroll
                for (int f = 7; f < 14; f++) tile[f * PT_NODES + t] = 0.f;
#pragma unroll
                for (int f = 17; f < MB_FIELDS; f++) tile[f * PT_NODES + t] = 0.f;
            }
        for (long long base = start;; base += P2G_CH) {
            int cnt, kcur = -1, kprev = -1;
            long long j = 0;
            const long long i = base + tid;
            if (sorted) {
                const bool inr = i < n;
                kcur = inr ? skey[i] : -1;
                kprev = (inr && tid > 0) ? skey[i - 1] : -1;
                j = inr ? perm[i] : 0;
                cnt = __syncthreads_count(tid < P2G_CH && inr && (kcur >> CB_SHIFT) == blk);
            } else {
                cnt = (int)min((long long)P2G_CH, segment_chunk_end(skey, n, blk, base, P2G_CH, &s_end) - base);
                if (tid < cnt) {
                    kcur = skey[i];
                    kprev = tid > 0 ? skey[i - 1] : -1;
                }
                j = i;
            }
            if (cnt <= 0) break;
            bool head = false, mine_one = true;
            if (tid < cnt) {
                const int cell = kcur & 63;
                head = tid == 0 || (kprev & 63) != cell;
                cellof[tid] = cell;
                float S[3], G[3];
                gimp_axis(P.f(PF_OX, j), g, S, G);
#pragma unroll
                for (int k = 0; k < 3; k++) W[0 + k][tid] = make_float2(S[k], G[k]);
                gimp_axis(P.f(PF_OY, j), g, S, G);
#pragma unroll
                for (int k = 0; k < 3; k++) W[3 + k][tid] = make_float2(S[k], G[k]);
                if (g.is3d) {
                    gimp_axis(P.f(PF_OZ, j), g, S, G);
                } else {
                    S[0] = 1.f; S[1] = 0.f; S[2] = 0.f; G[0] = 0.f; G[1] = 0.f; G[2] = 0.f;
                }
#pragma unroll
                for (int k = 0; k < 3; k++) W[6 + k][tid] = make_float2(S[k], G[k]);
                const uint32_t info = (uint32_t)P.ii(PF_INFO, j);
                const bool rigid = (info & INFO_RIGID) != 0;
                const float smass = P.f(PF_MASS, j), rho = P.f(PF_RHO, j);
                // a rigid particle's P2G mass is 1 (Extrapolation.cpp:183); its stored mass still
                // sets the volume the normals use
                const float m = rigid ? 1.0f : smass;
                const float sc = (m / rho) * g.inv_h;
                const float vol_n = ((info & INFO_INIT_VOL) ? init_vol : smass / rho) * g.inv_h;
                Q0[tid] = make_float4(m, m * P.f(PF_VX, j), m * P.f(PF_VY, j), m * P.f(PF_VZ, j));
                Q1[tid] = make_float4(P.f(PF_S0, j) * sc, P.f(PF_S0 + 1, j) * sc, P.f(PF_S0 + 2, j) * sc,
                                      P.f(PF_S0 + 3, j) * sc);
                Q2[tid] = make_float4(P.f(PF_S0 + 4, j) * sc, P.f(PF_S0 + 5, j) * sc, vol_n,
                                      __int_as_float(info_obj(info) | (rigid ? 1 << 16 : 0)));
                mine_one = !rigid && info_obj(info) == obj0;
            }
            const unsigned hm = __ballot_sync(0xffffffffu, head);
            if (lane == 0) wcount[warp] = __popc(hm);
            const bool chunk_one = __syncthreads_and(mine_one) != 0;
            if (uni && !chunk_one) {
                // from here on the slots are summed apart: slot 0 starts from what the
                // centre-of-mass fields hold (all of it slot-0 sums), except at nodes
                // without a body, whose slots receive nothing
                for (int t = tid; t < PT_NODES; t += P2G_CH) {
                    const bool has = tbody[t].x >= 0;
#pragma unroll
                    for (int f = 0; f < 7; f++) tile[(7 + f) * PT_NODES + t] = has ? tile[f * PT_NODES + t] : 0.f;
#pragma unroll
                    for (int f = 17; f < MB_FIELDS; f++) tile[f * PT_NODES + t] = 0.f;
                }
                __syncthreads();
                uni = false;
            }
            int wbase = 0, R = 0;
#pragma unroll
            for (int w2 = 0; w2 < P2G_CH / 32; w2++) {
                const int c = wcount[w2];
                wbase += (w2 < warp) ? c : 0;
                R += c;
            }
            if (head) run_start[wbase + __popc(hm & ((1u << lane) - 1u))] = tid;
            if (tid == 0) run_start[R] = cnt;
            __syncthreads();
            for (int r = warp; r < R; r += P2G_CH / 32) {
                const int p0 = run_start[r], p1 = run_start[r + 1];
                const int cell = cellof[p0];
                const int li = cell & 3, lj = (cell >> 2) & 3, lk = cell >> 4;
                const int t = ((lk + kk) * PT + (lj + jj)) * PT + (li + ii);
                const int2 bp = tbody[t];
                if (uni) {
                    float c[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, nr[3] = {0.f, 0.f, 0.f};
                    for (int p = p0; p < p1; p++) {
                        const float2 X = W[ii][p], Y = W[3 + jj][p], Z = W[6 + kk][p];
                        const float4 q0 = Q0[p], q1 = Q1[p], q2 = Q2[p];
                        const float syz = Y.x * Z.x;
                        const float w = X.x * syz, gx = X.y * syz, gy = X.x * Y.y * Z.x, gz = X.x * Y.x * Z.y;
                        const float wm = w * q0.x;
                        c[0] += wm; c[1] += w * q0.y; c[2] += w * q0.z; c[3] += w * q0.w;
                        c[4] += -(gx * q1.x + gy * q1.w + gz * q2.y) + wm * grx;
                        c[5] += -(gx * q1.w + gy * q1.y + gz * q2.x) + wm * gry;
                        c[6] += -(gx * q2.y + gy * q2.x + gz * q1.z) + wm * grz;
                        nr[0] += gx * q2.z; nr[1] += gy * q2.z; nr[2] += gz * q2.z;
                    }
                    if (!scatter_lane || c[0] == 0.f) continue;
#pragma unroll
                    for (int f = 0; f < 7; f++) atomicAdd(&tile[f * PT_NODES + t], c[f]);
                    if (bp.x >= 0)
#pragma unroll
                        for (int f = 0; f < 3; f++) atomicAdd(&tile[(14 + f) * PT_NODES + t], nr[f]);
                    continue;
                }
                // a run whose particles all belong to one deformable object, the node's first
                // body: its slot-0 mass, momentum and force equal the centre-of-mass sums
                // (gravity included), so only those and the normal are summed
                const int of0 = __float_as_int(Q2[p0].w);
                bool one = !(of0 >> 16);
                for (int p = p0 + 1; p < p1; p++) one = one && __float_as_int(Q2[p].w) == of0;
                if (one && bp.x == (of0 & 0xFFFF)) {
                    float c[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, nr[3] = {0.f, 0.f, 0.f};
                    for (int p = p0; p < p1; p++) {
                        const float2 X = W[ii][p], Y = W[3 + jj][p], Z = W[6 + kk][p];
                        const float4 q0 = Q0[p], q1 = Q1[p], q2 = Q2[p];
                        const float syz = Y.x * Z.x;
                        const float w = X.x * syz, gx = X.y * syz, gy = X.x * Y.y * Z.x, gz = X.x * Y.x * Z.y;
                        const float wm = w * q0.x;
                        c[0] += wm; c[1] += w * q0.y; c[2] += w * q0.z; c[3] += w * q0.w;
                        c[4] += -(gx * q1.x + gy * q1.w + gz * q2.y) + wm * grx;
                        c[5] += -(gx * q1.w + gy * q1.y + gz * q2.x) + wm * gry;
                        c[6] += -(gx * q2.y + gy * q2.x + gz * q1.z) + wm * grz;
                        nr[0] += gx * q2.z; nr[1] += gy * q2.z; nr[2] += gz * q2.z;
                    }
                    if (!scatter_lane || c[0] == 0.f) continue;
#pragma unroll
                    for (int f = 0; f < 7; f++) {
                        atomicAdd(&tile[f * PT_NODES + t], c[f]);
                        atomicAdd(&tile[(7 + f) * PT_NODES + t], c[f]);
                    }
#pragma unroll
                    for (int f = 0; f < 3; f++) atomicAdd(&tile[(14 + f) * PT_NODES + t], nr[f]);
                    continue;
                }
                float c[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                float b0[10] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                float b1[10] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                for (int p = p0; p < p1; p++) {
                    const float2 X = W[ii][p], Y = W[3 + jj][p], Z = W[6 + kk][p];
                    const float4 q0 = Q0[p], q1 = Q1[p], q2 = Q2[p];
                    const float syz = Y.x * Z.x;
                    const float w = X.x * syz, gx = X.y * syz, gy = X.x * Y.y * Z.x, gz = X.x * Y.x * Z.y;
                    const float wm = w * q0.x;
                    const float fx = -(gx * q1.x + gy * q1.w + gz * q2.y);
                    const float fy = -(gx * q1.w + gy * q1.y + gz * q2.x);
                    const float fz = -(gx * q2.y + gy * q2.x + gz * q1.z);
                    const float gfx = wm * grx, gfy = wm * gry, gfz = wm * grz;
                    c[0] += wm; c[1] += w * q0.y; c[2] += w * q0.z; c[3] += w * q0.w;
                    c[4] += fx + gfx; c[5] += fy + gfy; c[6] += fz + gfz;
                    const int of = __float_as_int(q2.w);
                    const int obj = of & 0xFFFF;
                    const float gr = (of >> 16) ? 0.f : 1.f;  // body fields: no gravity on rigid particles
                    const int sel = (bp.x == obj) ? 0 : ((bp.y == obj) ? 1 : -1);
                    if (sel == 0) {
                        b0[0] += wm; b0[1] += w * q0.y; b0[2] += w * q0.z; b0[3] += w * q0.w;
                        b0[4] += fx + gr * gfx; b0[5] += fy + gr * gfy; b0[6] += fz + gr * gfz;
                        b0[7] += gx * q2.z; b0[8] += gy * q2.z; b0[9] += gz * q2.z;
                    } else if (sel == 1) {
                        b1[0] += wm; b1[1] += w * q0.y; b1[2] += w * q0.z; b1[3] += w * q0.w;
                        b1[4] += fx + gr * gfx; b1[5] += fy + gr * gfy; b1[6] += fz + gr * gfz;
                        b1[7] += gx * q2.z; b1[8] += gy * q2.z; b1[9] += gz * q2.z;
                    }
                }
                if (!scatter_lane) continue;
                if (c[0] != 0.f) {
#pragma unroll
                    for (int f = 0; f < 7; f++) atomicAdd(&tile[f * PT_NODES + t], c[f]);
                }
                if (b0[0] != 0.f) {
#pragma unroll
                    for (int f = 0; f < 10; f++) atomicAdd(&tile[(7 + f) * PT_NODES + t], b0[f]);
                }
                if (b1[0] != 0.f) {
#pragma unroll
                    for (int f = 0; f < 10; f++) atomicAdd(&tile[(17 + f) * PT_NODES + t], b1[f]);
                }
            }
            if (cnt < P2G_CH) break;
        }
        __syncthreads();
        // ---- flush: COM fields and the touched body slots, vector reductions ----
        for (int t = tid; t < PT_NODES; t += P2G_CH) {
            const int ni = tox + t % PT, nj = toy + (t / PT) % PT, nk = toz + t / (PT * PT);
            if (ni >= g.nx || nj >= g.ny || nk >= g.nz) continue;
            const float m = tile[t];
            if (m == 0.f) continue;
            const int nd = node_index(ni, nj, nk, g);
            const float *f = tile + t;
            red_add4(&nb.acc0[nd], f[0], f[PT_NODES], f[2 * PT_NODES], f[3 * PT_NODES]);
            red_add4(&nb.acc1[nd], f[4 * PT_NODES], f[5 * PT_NODES], f[6 * PT_NODES], 0.f);
            if (uni) {
                if (tbody[t].x >= 0) {
                    red_add4(&nb.bacc0[0][nd], f[0], f[PT_NODES], f[2 * PT_NODES], f[3 * PT_NODES]);
                    red_add4(&nb.bacc1[0][nd], f[4 * PT_NODES], f[5 * PT_NODES], f[6 * PT_NODES], 0.f);
                    red_add4(&nb.bnrm[0][nd], f[14 * PT_NODES], f[15 * PT_NODES], f[16 * PT_NODES], 0.f);
                }
                mark_node(nb, ni, nj, nk, g);
                continue;
            }
#pragma unroll
            for (int sl = 0; sl < 2; sl++) {
                const float *b = f + (7 + 10 * sl) * PT_NODES;
                if (b[0] == 0.f) continue;
                red_add4(&nb.bacc0[sl][nd], b[0], b[PT_NODES], b[2 * PT_NODES], b[3 * PT_NODES]);
                red_add4(&nb.bacc1[sl][nd], b[4 * PT_NODES], b[5 * PT_NODES], b[6 * PT_NODES], 0.f);
                red_add4(&nb.bnrm[sl][nd], b[7 * PT_NODES], b[8 * PT_NODES], b[9 * PT_NODES], 0.f);
            }
            mark_node(nb, ni, nj, nk, g);
        }
    }
}

void launch_p2g(const PView &p, const int *perm, const int *skey, long long n, const int *seg_start,
                const int *nseg, int persist_grid, const NodeBufs &nb, const StepArgs &a, cudaStream_t s,
                const float4 *therm, float2 *tnode, int lanes, int *defer, int *ndefer)
{
    if (n == 0) return;
    if (a.multi_body) {
        static int mgrid = 0, qgrid = 0;  // persistent grids of the two multi-body kernels
        if (mgrid == 0) {
            int dev = 0, sms = 1, b = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_p2g_multi_tiled, P2G_CH, 0);
            mgrid = sms * std::max(b, 1);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_p2g_planes<true>, PP_THREADS, 0);
            qgrid = sms * std::max(b, 1);
        }
        if (lanes == 3 && defer && ndefer) {
            // the one-object segments with plane lanes, the rest (listed in defer, whose count
            // the caller zeroed) with the body-slot kernel
            k_p2g_planes<true><<<qgrid, PP_THREADS, 0, s>>>(p, perm, skey, n, seg_start, nseg, perm ? 1 : 0, nb, a,
                                                             defer, ndefer);
            k_p2g_multi_tiled<<<mgrid, P2G_CH, 0, s>>>(p, perm, skey, n, defer, ndefer, perm ? 1 : 0, nb, a);
            note_launch(1);
        } else {
            k_p2g_multi_tiled<<<mgrid, P2G_CH, 0, s>>>(p, perm, skey, n, seg_start, nseg, perm ? 1 : 0, nb, a);
        }
    } else {
        if (therm && lanes == 3) {
            static int hgrid = 0;  // persistent grid of the plane-lane variant with heat conduction
            if (hgrid == 0) {
                int dev = 0, sms = 1, b = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_p2g_planes<false, true>, PP_THREADS, 0);
                hgrid = sms * std::max(b, 1);
            }
            k_p2g_planes<false, true><<<hgrid, PP_THREADS, 0, s>>>(p, perm, skey, n, seg_start, nseg, perm ? 1 : 0, nb,
                                                                    a, nullptr, nullptr, therm, tnode);
        } else if (therm) {
            static int tgrid = 0;  // persistent grid of the variant with heat conduction
            if (tgrid == 0) {
                int dev = 0, sms = 1, b = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_p2g_cols<true>, PC_THREADS, 0);
                tgrid = sms * std::max(b, 1);
            }
            k_p2g_cols<true><<<tgrid, PC_THREADS, 0, s>>>(p, perm, skey, n, seg_start, nseg, perm ? 1 : 0, nb, a.g,
                                                           therm, tnode, a.mats);
        } else if (lanes == 3) {
            static int pgrid = 0;  // persistent grid of the plane-lane kernel (its own occupancy)
            if (pgrid == 0) {
                int dev = 0, sms = 1, b = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_p2g_planes<false>, PP_THREADS, 0);
                pgrid = sms * std::max(b, 1);
            }
            k_p2g_planes<false><<<pgrid, PP_THREADS, 0, s>>>(p, perm, skey, n, seg_start, nseg, perm ? 1 : 0, nb, a,
                                                              nullptr, nullptr);
        } else {
            k_p2g_cols<false><<<persist_grid, PC_THREADS, 0, s>>>(p, perm, skey, n, seg_start, nseg, perm ? 1 : 0, nb,
                                                                   a.g, nullptr, nullptr, nullptr);
        }
    }
    note_launch(1);
}

int p2g_blocks_per_sm()
{
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_p2g_cols<false>, PC_THREADS, 0);
    return b > 0 ? b : 1;
}

// ---------------------------------------------------------------------------------------
// periodic fold, Grid.cpp:310-795: node i and node N-3+i (i < 3) both take their sum, for
// mass, momentum and force of the centre-of-mass field and both body fields.

__device__ __forceinline__ bool fold4(float4 *arr, long long p, long long q)
{
    const float4 x = arr[p], y = arr[q];
    const float4 s = make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
    arr[p] = s;
    arr[q] = s;
    return s.x != 0.f || s.y != 0.f || s.z != 0.f || s.w != 0.f;
}

template <bool MULTI>
__global__ void k_fold(NodeBufs nb, GridGeom g, int axis)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int d0, d1;
    if (axis == 0) { d0 = g.ny; d1 = g.nz; }
    else if (axis == 1) { d0 = g.nx; d1 = g.nz; }
    else { d0 = g.nx; d1 = g.ny; }
    const long long plane = (long long)d0 * d1;
    if (t >= 3 * plane) return;
    const int l = (int)(t / plane);
    const long long r = t - (long long)l * plane;
    const int a0 = (int)(r % d0), a1 = (int)(r / d0);
    int pi, pj, pk, qi, qj, qk;
    if (axis == 0) { pi = l; pj = a0; pk = a1; qi = g.nx - 3 + l; qj = a0; qk = a1; }
    else if (axis == 1) { pi = a0; pj = l; pk = a1; qi = a0; qj = g.ny - 3 + l; qk = a1; }
    else { pi = a0; pj = a1; pk = l; qi = a0; qj = a1; qk = g.nz - 3 + l; }
    // the accumulators of a node block P2G (or an earlier axis' fold) did not flag are all
    // zero: a pair of such nodes folds to zeros already in place
    if (!nb.flags[node_block(pi, pj, pk, g)] && !nb.flags[node_block(qi, qj, qk, g)]) return;
    const long long p = node_index(pi, pj, pk, g), q = node_index(qi, qj, qk, g);
    bool any = fold4(nb.acc0, p, q);
    any |= fold4(nb.acc1, p, q);
    if (MULTI) {
        for (int b = 0; b < 2; b++) {
            any |= fold4(nb.bacc0[b], p, q);
            any |= fold4(nb.bacc1[b], p, q);
        }
    }
    if (any) {
        mark_node(nb, pi, pj, pk, g);
        mark_node(nb, qi, qj, qk, g);
    }
}

void launch_fold(const NodeBufs &nb, const StepArgs &a, cudaStream_t s)
{
    const GridGeom &g = a.g;
    const int naxes = g.is3d ? 3 : 2;
    for (int ax = 0; ax < naxes; ax++) {
        const long long plane = ax == 0 ? (long long)g.ny * g.nz : ax == 1 ? (long long)g.nx * g.nz : (long long)g.nx * g.ny;
        const unsigned grid = (unsigned)((3 * plane + 255) / 256);
        if (a.multi_body) k_fold<true><<<grid, 256, 0, s>>>(nb, g, ax);
        else k_fold<false><<<grid, 256, 0, s>>>(nb, g, ax);
        note_launch(1);
    }
}

// ---------------------------------------------------------------------------------------
// nodal solve (Grid.cpp:9-245) + grid BC phase 2 (Grid.cpp:862-1094), active node blocks

struct BCApply {
    int type;
    float4 val;
    int fixed;
    __device__ __forceinline__ void comps(bool set[3], float v[3]) const
    {
        set[0] = set[1] = set[2] = false;
        switch (type) {
        case BC_GRID_VX: set[0] = true; v[0] = val.x; break;
        case BC_GRID_VY: set[1] = true; v[1] = val.x; break;
        case BC_GRID_VX_VY: set[0] = set[1] = true; v[0] = val.x; v[1] = val.y; break;
        case BC_GRID_VZ: if (fixed) { set[2] = true; v[2] = val.x; } break;
        case BC_GRID_VX_VZ: if (fixed) { set[0] = set[2] = true; v[0] = val.x; v[2] = val.y; } break;
        case BC_GRID_VY_VZ: if (fixed) { set[1] = set[2] = true; v[1] = val.x; v[2] = val.y; } break;
        case BC_GRID_VX_VY_VZ:
            if (fixed) { set[0] = set[1] = set[2] = true; v[0] = val.x; v[1] = val.y; v[2] = val.z; }
            break;
        default: break;
        }
    }
};

__device__ __forceinline__ void body_update(float m, const float4 &p, const float4 &f, float dtn, float v[3], float acc[3])
{
    v[0] = p.y / m; v[1] = p.z / m; v[2] = p.w / m;
    acc[0] = f.x / m; acc[1] = f.y / m; acc[2] = f.z / m;
    v[0] += acc[0] * dtn; v[1] += acc[1] * dtn; v[2] += acc[2] * dtn;
}

// calculateColoumbFrictionContactNormals, Grid.cpp:247-308 (only the contact normal is
// used by the solve; the friction outputs are discarded by the caller)
__device__ __forceinline__ void contact_normal(const float rv[3], const float n[3], float mu, float cn[3])
{
    float om0 = rv[1] * n[2] - rv[2] * n[1];
    float om1 = rv[0] * n[2] - rv[2] * n[0];
    float om2 = rv[0] * n[1] - rv[1] * n[0];
    const float mag = sqrtf(om0 * om0 + om1 * om1 + om2 * om2) + 0.001f;
    om0 /= mag; om1 /= mag; om2 /= mag;
    const float mu0 = mag / (rv[0] * n[0] + rv[1] * n[1] + rv[2] * n[2]) + 0.001f;
    const float on0 = om2 * n[1] - om1 * n[2];
    const float on1 = om2 * n[0] - om0 * n[2];
    const float on2 = om1 * n[0] - om0 * n[1];
    if (mu0 < mu) mu = mu0;
    cn[0] = n[0] + on0 * mu;
    cn[1] = n[1] + on1 * mu;
    cn[2] = n[2] + on2 * mu;
}

// One node of an active node block; returns whether the node carries mass.
template <bool MULTI>
__device__ __forceinline__ bool solve_node(const NodeBufs &nb, const StepArgs &a, int keep, long long blk, int lnode)
{
    const GridGeom &g = a.g;
    bool active = false;
    {
        const int lx = lnode & 3, ly = (lnode >> 2) & 3, lz = (lnode >> 4) & 3;
        const int b32 = (int)blk;  // node blocks < 2^31
        const int bx = b32 % g.nnbx, tb = b32 / g.nnbx;
        const int by = tb % g.nnby, bz = tb / g.nnby;
        const int i = bx * 4 + lx, j = by * 4 + ly, k = bz * 4 + lz;
        if (i < g.nx && j < g.ny && k < g.nz) {
            const int nd = node_index(i, j, k, g);
            const float4 A0 = nb.acc0[nd];
            float4 A1 = nb.acc1[nd];
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            // every load of the node is issued before the first store (the accumulators are
            // cleared after they were read)
            float4 B0[2], B1[2], BN[2];
            int2 body = make_int2(-1, -1);
            unsigned char hr = 0;
            // a node block whose nodes all hold one body has nothing in slot 1, and its nodes
            // need no normal unless normals are tracked
            bool two = false;
            if (MULTI) {
                two = nb.nblk_two[blk] != 0;
                B0[0] = nb.bacc0[0][nd];
                B1[0] = nb.bacc1[0][nd];
                body = nb.body[nd];
                hr = nb.has_rigid[nd];
                BN[0] = (two || nb.nrm_out[0]) ? nb.bnrm[0][nd] : z4;
                B0[1] = B1[1] = BN[1] = z4;
                if (two) {
                    B0[1] = nb.bacc0[1][nd];
                    B1[1] = nb.bacc1[1][nd];
                    BN[1] = nb.bnrm[1][nd];
                }
            }
            const int bt = nb.bc_type ? nb.bc_type[nd] : 0;
            nb.acc0[nd] = z4;
            nb.acc1[nd] = z4;
            const float m = A0.x;
            if (!MULTI) {
                // single body: gravity enters here as m_node * g (Extrapolation.cpp:226-228)
                A1.x += m * a.sc->gravity[0];
                A1.y += m * a.sc->gravity[1];
                A1.z += m * a.sc->gravity[2];
            }
            const float dtn = a.sc->dt_node, dt = a.sc->dt;
            float vc[3] = {0.f, 0.f, 0.f};
            float v1[3] = {0.f, 0.f, 0.f}, a1[3] = {0.f, 0.f, 0.f};
            float v2[3] = {0.f, 0.f, 0.f}, a2[3] = {0.f, 0.f, 0.f};
            float n1[3] = {0.f, 0.f, 0.f};
            active = (m != 0.0f);
            if (!MULTI) {
                if (active) {
                    vc[0] = A0.y / m; vc[1] = A0.z / m; vc[2] = A0.w / m;
                    body_update(m, A0, A1, dtn, v1, a1);
                }
            } else {
                nb.bacc0[0][nd] = z4;
                nb.bacc1[0][nd] = z4;
                nb.bnrm[0][nd] = z4;
                if (two) {
                    nb.bacc0[1][nd] = z4;
                    nb.bacc1[1][nd] = z4;
                    nb.bnrm[1][nd] = z4;
                }
                if (active) {
                    vc[0] = A0.y / m; vc[1] = A0.z / m; vc[2] = A0.w / m;
                    const float mag1 = sqrtf(BN[0].x * BN[0].x + BN[0].y * BN[0].y + BN[0].z * BN[0].z);
                    if (mag1 > 1e-8f) { n1[0] = BN[0].x / mag1; n1[1] = BN[0].y / mag1; n1[2] = BN[0].z / mag1; }
                    const float n2[3] = {-n1[0], -n1[1], -n1[2]};  // Grid.cpp:45-47
                    const float m1 = B0[0].x, m2 = B0[1].x;
                    if (body.y != -1) {
                        float ap1 = 0.f, ap2 = 0.f, rv1[3] = {0.f, 0.f, 0.f}, rv2[3] = {0.f, 0.f, 0.f};
                        if (m1 != 0.0f) {
                            rv1[0] = B0[0].y / m1 - vc[0]; rv1[1] = B0[0].z / m1 - vc[1]; rv1[2] = B0[0].w / m1 - vc[2];
                            ap1 = rv1[0] * n1[0] + rv1[1] * n1[1] + rv1[2] * n1[2];
                        }
                        if (m2 != 0.0f) {
                            rv2[0] = B0[1].y / m2 - vc[0]; rv2[1] = B0[1].z / m2 - vc[1]; rv2[2] = B0[1].w / m2 - vc[2];
                            ap2 = rv2[0] * n2[0] + rv2[1] * n2[1] + rv2[2] * n2[2];
                        }
                        if (ap1 > 0.01f || ap2 > 0.01f) {
                            if (hr & 1) {
                                // body 1 rigid: body 2 takes body 1's velocity (Grid.cpp:78-91)
                                if (m1 != 0.0f) {
                                    v1[0] = B0[0].y / m1; v1[1] = B0[0].z / m1; v1[2] = B0[0].w / m1;
                                    if (m2 != 0.0f) {
                                        v2[0] = B0[1].y / m2 - (B0[1].y - m2 * v1[0]) / m2;
                                        v2[1] = B0[1].z / m2 - (B0[1].z - m2 * v1[1]) / m2;
                                        v2[2] = B0[1].w / m2 - (B0[1].w - m2 * v1[2]) / m2;
                                    }
                                }
                            } else if (hr & 2) {
                                if (m2 != 0.0f) {
                                    v2[0] = B0[1].y / m2; v2[1] = B0[1].z / m2; v2[2] = B0[1].w / m2;
                                    if (m1 != 0.0f) {
                                        v1[0] = B0[0].y / m1 - (B0[0].y - m1 * v2[0]) / m1;
                                        v1[1] = B0[0].z / m1 - (B0[0].z - m1 * v2[1]) / m1;
                                        v1[2] = B0[0].w / m1 - (B0[0].w - m1 * v2[2]) / m1;
                                    }
                                }
                            } else {
                                if (m1 != 0.0f) {
                                    float cn[3];
                                    contact_normal(rv1, n1, a.sc->mu, cn);
                                    v1[0] = B0[0].y / m1 - ap1 * cn[0];
                                    v1[1] = B0[0].z / m1 - ap1 * cn[1];
                                    v1[2] = B0[0].w / m1 - ap1 * cn[2];
                                    a1[0] = B1[0].x / m1 - (ap1 * cn[0]) / dt;
                                    a1[1] = B1[0].y / m1 - (ap1 * cn[1]) / dt;
                                    a1[2] = B1[0].z / m1 - (ap1 * cn[2]) / dt;
                                    for (int c = 0; c < 3; c++) v1[c] += a1[c] * dtn;
                                }
                                if (m2 != 0.0f) {
                                    float cn[3];
                                    contact_normal(rv2, n2, a.sc->mu, cn);
                                    v2[0] = B0[1].y / m2 - ap2 * cn[0];
                                    v2[1] = B0[1].z / m2 - ap2 * cn[1];
                                    v2[2] = B0[1].w / m2 - ap2 * cn[2];
                                    a2[0] = B1[1].x / m2 - (ap2 * cn[0]) / dt;
                                    a2[1] = B1[1].y / m2 - (ap2 * cn[1]) / dt;
                                    a2[2] = B1[1].z / m2 - (ap2 * cn[2]) / dt;
                                    for (int c = 0; c < 3; c++) v2[c] += a2[c] * dtn;
                                }
                            }
                        } else {
                            if (m1 != 0.0f) body_update(m1, B0[0], B1[0], dtn, v1, a1);
                            if (m2 != 0.0f) body_update(m2, B0[1], B1[1], dtn, v2, a2);
                        }
                    } else {
                        if (m1 != 0.0f) body_update(m1, B0[0], B1[0], dtn, v1, a1);
                    }
                }
            }
            // grid BC, phase 2 (phase 1 is overwritten by the solve for every node the
            // particles read; phase 3 repeats phase 2)
            if (bt) {
                BCApply bc{bt, nb.bc_val[nd], a.sc->fixed_grid_bcs};
                bool set[3];
                float val[3];
                bc.comps(set, val);
                for (int c = 0; c < 3; c++)
                    if (set[c]) {
                        v1[c] = val[c]; a1[c] = 0.f;
                        v2[c] = val[c]; a2[c] = 0.f;
                        vc[c] = val[c];
                    }
            }
            nb.gv[nd] = make_float4(m, v1[0], v1[1], v1[2]);
            nb.ga[nd] = make_float4(a1[0], a1[1], a1[2], 0.f);
            if (MULTI && two) {
                // slot 0's solved fields are gv / ga; slot 1 is read only where a node holds two
                // bodies
                nb.bgv[1][nd] = make_float4(m, v2[0], v2[1], v2[2]);
                nb.bga[1][nd] = make_float4(a2[0], a2[1], a2[2], 0.f);
            }
            if (MULTI) {
                if (nb.nrm_out[0]) {
                    nb.nrm_out[0][nd] = make_float4(n1[0], n1[1], n1[2], 0.f);
                    nb.nrm_out[1][nd] = make_float4(-n1[0], -n1[1], -n1[2], 0.f);
                }
            }
            if (keep) {
                nb.out_com[nd] = make_float4(vc[0], vc[1], vc[2], 0.f);
                nb.out_force[nd] = make_float4(A1.x, A1.y, A1.z, 0.f);
            }
        }
    }
    return active;
}

// Single-body nodal solve (Grid.cpp:9-245 without contact, then the grid BCs): one warp per
// listed block, each lane owns nodes lane and lane + 32, and all loads of both nodes are
// issued before the first result is needed.
__global__ void __launch_bounds__(256) k_solve_single(NodeBufs nb, StepArgs a, int keep)
{
    const GridGeom &g = a.g;
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    const int nact = *nb.active_n;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float dtn = a.sc->dt_node;
    const float grx = a.sc->gravity[0], gry = a.sc->gravity[1], grz = a.sc->gravity[2];
    const int fixed_bcs = a.sc->fixed_grid_bcs;
    int count = 0;
    for (int w = gw; w < nact; w += nw) {
        const int blk = nb.active_list[w];
        const int bx = blk % g.nnbx, tb = blk / g.nnbx;
        const int by = tb % g.nnby, bz = tb / g.nnby;
        int nd[2];
        bool in[2];
        float4 A0[2], A1[2];
        int bt[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int ln = lane + 32 * h;
            const int i = bx * 4 + (ln & 3), j = by * 4 + ((ln >> 2) & 3), k = bz * 4 + (ln >> 4);
            in[h] = i < g.nx && j < g.ny && k < g.nz;
            nd[h] = in[h] ? node_index(i, j, k, g) : 0;
            A0[h] = in[h] ? nb.acc0[nd[h]] : z4;
            A1[h] = in[h] ? nb.acc1[nd[h]] : z4;
            bt[h] = (in[h] && nb.bc_type) ? (int)nb.bc_type[nd[h]] : 0;
        }
        if (lane == 0) nb.flags[blk] = 0;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (!in[h]) continue;
            nb.acc0[nd[h]] = z4;
            nb.acc1[nd[h]] = z4;
            const float m = A0[h].x;
            float4 F = A1[h];
            // gravity enters here as m_node * g (Extrapolation.cpp:226-228)
            F.x += m * grx;
            F.y += m * gry;
            F.z += m * grz;
            float vc[3] = {0.f, 0.f, 0.f}, v1[3] = {0.f, 0.f, 0.f}, a1[3] = {0.f, 0.f, 0.f};
            if (m != 0.0f) {
                count++;
                vc[0] = A0[h].y / m; vc[1] = A0[h].z / m; vc[2] = A0[h].w / m;
                body_update(m, A0[h], F, dtn, v1, a1);
            }
            // grid BC, phase 2 (phase 1 is overwritten by the solve for every node the
            // particles read; phase 3 repeats phase 2)
            if (bt[h]) {
                BCApply bc{bt[h], nb.bc_val[nd[h]], fixed_bcs};
                bool set[3];
                float val[3];
                bc.comps(set, val);
#pragma unroll
                for (int c = 0; c < 3; c++)
                    if (set[c]) {
                        v1[c] = val[c]; a1[c] = 0.f;
                        vc[c] = val[c];
                    }
            }
            nb.gv[nd[h]] = make_float4(m, v1[0], v1[1], v1[2]);
            nb.ga[nd[h]] = make_float4(a1[0], a1[1], a1[2], 0.f);
            if (keep) {
                nb.out_com[nd[h]] = make_float4(vc[0], vc[1], vc[2], 0.f);
                nb.out_force[nd[h]] = make_float4(F.x, F.y, F.z, 0.f);
            }
        }
    }
    if (nb.active_count) {
        for (int off = 16; off > 0; off >>= 1) count += __shfl_down_sync(0xffffffffu, count, off);
        if (lane == 0 && count) atomicAdd(nb.active_count, count);
    }
}

// The flagged node blocks, appended to the solve's list: one ballot and one atomic per warp.
// It also zeroes the conservation partials the step's G2P adds into (stats, may be null).
__global__ void k_compact_active(NodeBufs nb, int nnb, double *stats)
{
    const int lane = threadIdx.x & 31;
    if (stats && blockIdx.x == 0)
        for (int q = threadIdx.x; q < STATS_SLOTS * 8; q += blockDim.x) stats[q] = 0.0;
    for (int b0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; b0 < nnb; b0 += gridDim.x * blockDim.x) {
        const int b = b0 + lane;
        const bool f = b < nnb && nb.flags[b] != 0;
        const unsigned m = __ballot_sync(0xffffffffu, f);
        if (!m) continue;
        int base = 0;
        if (lane == 0) base = atomicAdd(nb.active_n, __popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (f) nb.active_list[base + __popc(m & ((1u << lane) - 1u))] = b;
    }
}

// Multi-body nodal solve with contact: two warps per active node block from the list P2G
// and the fold built (32 nodes each); the block's flag is cleared for the next step.
#ifndef GY_SOLVE_MINB
#define GY_SOLVE_MINB 5  // resident 256-thread CTAs per SM the multi-body solve is register-capped to (48)
#endif
template <bool MULTI>
__global__ void __launch_bounds__(256, GY_SOLVE_MINB) k_solve_list(NodeBufs nb, StepArgs a, int keep)
{
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    const int nact = *nb.active_n;
    int count = 0;
    // one warp per half block (32 nodes), so the two halves' loads are in flight together
    for (int w = gw; w < 2 * nact; w += nw) {
        const long long blk = nb.active_list[w >> 1];
        count += solve_node<MULTI>(nb, a, keep, blk, lane + 32 * (w & 1)) ? 1 : 0;
        if (lane == 0 && (w & 1) == 0) nb.flags[blk] = 0;
    }
    if (nb.active_count) {
        for (int off = 16; off > 0; off >>= 1) count += __shfl_down_sync(0xffffffffu, count, off);
        if (lane == 0 && count) atomicAdd(nb.active_count, count);
    }
}

void launch_solve(const NodeBufs &nb, const StepArgs &a, bool keep_node_fields, cudaStream_t s)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long cgrid = std::min<long long>((a.g.nnb + 255) / 256, (long long)sms * 8);
    k_compact_active<<<(unsigned)std::max<long long>(cgrid, 1), 256, 0, s>>>(nb, (int)a.g.nnb, a.stats);
    note_launch(1);
    long long grid = std::min<long long>((a.g.nnb + 7) / 8, (long long)sms * 16);  // 8 warps per CTA
    if (grid < 1) grid = 1;
    if (a.multi_body) k_solve_list<true><<<(unsigned)grid, 256, 0, s>>>(nb, a, keep_node_fields ? 1 : 0);
    else k_solve_single<<<(unsigned)grid, 256, 0, s>>>(nb, a, keep_node_fields ? 1 : 0);
    note_launch(1);
}

// ---------------------------------------------------------------------------------------
// G2P + particle BCs + update + constitutive + damage + wrap + key, one particle

// particle BCs, TimeIntegration.cpp:177-296
__device__ __forceinline__ void particle_bc(int type, const float4 &val, float t, float mass, float v[3], float acc[3],
                                            float vg[3], float s[6])
{
    const float w = 2.0f * 3.14159f;
    switch (type) {
    case BC_MP_VX: v[0] = val.x; break;
    case BC_MP_VY: v[0] = 0.f; v[1] = val.x; v[2] = 0.f; break;
    case BC_MP_VZ: v[0] = 0.f; v[1] = 0.f; v[2] = val.x; break;
    case BC_MP_VX_VY: v[0] = val.x; v[1] = val.y; v[2] = 0.f; break;
    case BC_MP_VXSIN: v[0] = val.x * sinf(w * val.y * t); break;
    case BC_MP_VYSIN: v[1] = val.x * sinf(w * val.y * t); vg[1] = 0.f; acc[1] = 0.f; break;
    case BC_MP_SYYSIN:
        s[1] = val.x * sinf(w * val.y * t);
        v[0] = v[1] = v[2] = 0.f;
        vg[0] = vg[1] = vg[2] = 0.f;
        break;
    case BC_MP_FX: acc[0] += val.x / mass; break;
    case BC_MP_FY: acc[0] = 0.f; acc[1] += val.x / mass; break;
    case BC_MP_FZ: acc[2] += val.x / mass; break;
    case BC_MP_FX_FY: acc[0] += val.x / mass; acc[1] += val.y / mass; break;
    case BC_MP_STRESS_XX_YY: s[0] = val.x; s[1] = val.y; break;
    default: break;
    }
}

// move the offset into [lp, 1+lp) and carry whole cells into c
__device__ __forceinline__ void renorm(float &o, int &c, float lp)
{
    const float k = floorf(o - lp);
    if (k != 0.0f) {
        o -= k;
        c += (int)k;
    }
}

// The Drucker-Prager + damage update of one particle with the learned surrogate's hooks
// (DpHooks): a yielding particle without a BC is deferred to the surrogate pass when that is
// on (its stress, plastic strain and damage left as they were; returns true), else the exact
// return mapping runs and, when logging, the yielding particles of the sample record their
// training pair; the damage update follows.
__device__ __forceinline__ bool dp_hooked(Constit &c, const DevMaterial &M, float dt, int is3d, const StepArgs &a,
                                       int pid, int step, long long slot, int bct)
{
    float t[6];
    const bool yields = is3d && dp_trial_yields(c, M, dt, t);
    if (yields && a.dp.pend && bct == 0) {
        const unsigned int e = atomicAdd(a.dp.pend_n, 1u);
        if (e < a.dp.pend_cap) {
            a.dp.pend[2 * e] = make_float4(__int_as_float((int)slot), c.r[0] * dt, c.r[1] * dt, c.r[2] * dt);
            a.dp.pend[2 * e + 1] = make_float4(c.r[3] * dt, c.r[4] * dt, c.r[5] * dt, 0.f);
            return true;
        }
    }
    float s0[6];
#pragma unroll
    for (int k = 0; k < 6; k++) s0[k] = c.s[k];
    const float eq0 = c.eqps, d0 = c.dmg;
    cm_drucker_prager(c, M, dt);
    if (yields && a.dp.log_x && ((unsigned)(pid + step) % (unsigned)a.dp.log_every) == 0u) {
        const unsigned int e = atomicAdd(a.dp.log_n, 1u);
        if (e < a.dp.log_cap) {
            float *x = a.dp.log_x + (size_t)e * 16;
            float *y = a.dp.log_y + (size_t)e * 7;
#pragma unroll
            for (int k = 0; k < 6; k++) {
                x[k] = c.r[k] * dt;
                x[6 + k] = s0[k];
                y[k] = c.s[k] - t[k];
            }
            x[12] = eq0;
            x[13] = d0;
            x[14] = M.cohesion;
            x[15] = M.phi_deg;
            y[6] = c.eqps - eq0;
        }
    }
    if (M.damage && M.damage_model == 1) {
        if (is3d) dm_grady_kipp3(c, M, dt, a.flaw, pid);
        else dm_grady_kipp2(c, M, dt, a.flaw, pid);
    }
    return false;
}

// Everything after the G2P sums, for one particle: particle BCs, update, constitutive model,
// damage, periodic wrap and the new cell key (TimeIntegration.cpp:11-296).  c0 is the cell of
// the particle's first stencil node before the update; slot is where G2P writes the particle.
template <bool HAS_DP>
__device__ __forceinline__ void update_after_g2p(PState &st, const int c0[3], float acc[3], float vg[3],
                                                 const float L[3][3], const StepArgs &a, bool check_finite,
                                                 long long slot)
{
    const GridGeom &g = a.g;
    const StepScalars sc = *a.sc;
    Constit c;
    c.r[0] = L[0][0];
    c.r[1] = L[1][1];
    c.r[2] = L[2][2];
    c.r[3] = 0.5f * (L[1][0] + L[0][1]);
    c.r[4] = 0.5f * (L[2][1] + L[1][2]);
    c.r[5] = 0.5f * (L[2][0] + L[0][2]);
    const float rho_rate = -st.rho * (L[0][0] + L[1][1] + L[2][2]);
#pragma unroll
    for (int k = 0; k < 6; k++) {
        c.s[k] = st.s[k];
        c.e[k] = st.e[k];
        c.ep[k] = st.ep[k];
    }
    c.eqps = st.eqps;
    c.dmg = st.dmg;
    c.smax = st.smax;
    const int bct = info_bc(st.info);
    float4 bcv = make_float4(0.f, 0.f, 0.f, 0.f);
    if (bct) bcv = __ldg(&a.pbc_val[st.pid]);

    // ---- particle BC, phase 4 ----
    if (bct) particle_bc(bct, bcv, sc.t_bc, st.mass, st.v, acc, vg, c.s);

    // ---- update (TimeIntegration.cpp:11-117) ----
    const float dt = sc.dt;
    st.rho += rho_rate * dt;
    if (!(st.info & INFO_HOLD)) {
        st.v[0] = st.v[0] + (acc[0] - sc.damping * st.v[0]) * dt;
        st.v[1] = st.v[1] + (acc[1] - sc.damping * st.v[1]) * dt;
        if (g.is3d) st.v[2] = st.v[2] + (acc[2] - sc.damping * st.v[2]) * dt;
        st.o[0] += vg[0] * dt * g.inv_h;
        st.o[1] += vg[1] * dt * g.inv_h;
        if (g.is3d) st.o[2] += vg[2] * dt * g.inv_h;
    }
#pragma unroll
    for (int k = 0; k < 6; k++) c.e[k] += c.r[k] * dt;
    c.mass = st.mass;
    c.rho = st.rho;
    c.v[0] = st.v[0]; c.v[1] = st.v[1]; c.v[2] = st.v[2];
    if (!(st.info & INFO_RIGID)) {
        const DevMaterial &M = a.mats[info_mat(st.info)];
        if (HAS_DP) {
            if (M.model == 4 && (a.dp.pend || a.dp.log_x))
                dp_hooked(c, M, dt, g.is3d, a, st.pid, sc.step, slot, bct);
            else
                constitutive_update(c, M, dt, g.is3d, a.flaw, st.pid);
        } else {
            if (M.model == 1) cm_elastic(c, M, dt);
            else if (M.model == 2) cm_newtonian(c, M.K, M.viscosity, dt, g.is3d, false);
        }
    }

    // ---- periodic wrap (TimeIntegration.cpp:80-108) and the new cell ----
    int cc[3] = {c0[0], c0[1], c0[2]};
    const int naxes = g.is3d ? 3 : 2;
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        if (ax >= naxes) break;
        renorm(st.o[ax], cc[ax], g.lp);
        const float X = (float)cc[ax] + st.o[ax];
        int sh = 0;
        float sf = 0.f;
        if (X > g.wrap_hi[ax]) { sh = g.wrap_shift_int[ax]; sf = g.wrap_shift_frac[ax]; }
        if (X + (float)sh + sf < 1.0f) { sh -= g.wrap_shift_int[ax]; sf -= g.wrap_shift_frac[ax]; }
        if (sh != 0 || sf != 0.f) {
            cc[ax] += sh;
            st.o[ax] += sf;
            renorm(st.o[ax], cc[ax], g.lp);
        }
    }
    const int lim[3] = {g.ncx - 2, g.ncy - 2, g.ncz - 2};
    bool bad = false;
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        if (ax >= naxes) break;
        if (cc[ax] < 0) { cc[ax] = 0; bad = true; }
        if (cc[ax] > lim[ax]) { cc[ax] = lim[ax]; bad = true; }
    }
    if (bad) atomicOr(a.status, ERR_RANGE);
    st.key = encode_key(cc[0], cc[1], g.is3d ? cc[2] : 0, g);

    // ---- particle BC, phase 5 ----
    if (bct) particle_bc(bct, bcv, sc.t_bc, st.mass, st.v, acc, vg, c.s);

    if (check_finite) {
        bool fin = isfinite(st.v[0]) && isfinite(st.v[1]) && isfinite(st.v[2]) && isfinite(st.rho);
#pragma unroll
        for (int k = 0; k < 6; k++) fin = fin && isfinite(c.s[k]);
        if (!fin) atomicOr(a.status, ERR_NONFINITE);
    }
#pragma unroll
    for (int k = 0; k < 6; k++) {
        st.s[k] = c.s[k];
        st.e[k] = c.e[k];
        st.ep[k] = c.ep[k];
    }
    st.eqps = c.eqps;
    st.dmg = c.dmg;
    st.smax = c.smax;
    st.info &= ~INFO_INIT_VOL;
}

// G2P CTA size and the resident CTAs per SM it is register-limited to: twelve (80 registers;
// 16 CTAs at 64 registers spill in the update and measured 3 % slower)
#ifndef GY_G2P_MINB
#define GY_G2P_MINB 12
#endif
#ifndef GY_G2P_THREADS
#define GY_G2P_THREADS 64
#endif
#define GY_G2P_MINB_TH 12  // the variant with heat conduction: 80 registers
// multi-body G2P: CTA size and resident CTAs per SM (the node tile holds two body slots, so
// a larger CTA shares it among more particles)
#ifndef GY_G2PM_THREADS
#define GY_G2PM_THREADS 128
#endif
#ifndef GY_G2PM_MINB
#define GY_G2PM_MINB 5
#endif


// particle fields G2P does not need, staged in shared memory while the G2P sums run:
// velocity, stress, strain, density, mass, info, pid, then (DP / damage) eqps, plastic
// strain, damage, smax
__device__ __forceinline__ constexpr int g2p_stage_field(int f)
{
    return f < 3 ? PF_VX + f : f < 9 ? PF_S0 + (f - 3) : f < 15 ? PF_E0 + (f - 9) : f == 15 ? PF_RHO
         : f == 16 ? PF_MASS : f == 17 ? PF_INFO : f == 18 ? PF_PID : f == 19 ? PF_EQPS
         : f < 26 ? PF_EP0 + (f - 20) : f == 26 ? PF_DMG : PF_SMAX;
}
constexpr int G2P_NBASE = 19, G2P_NDP = 9;

// Conservation sums of the updated particles, fused into G2P: each thread adds its particles'
// momentum, kinetic and strain energy into its own shared-memory column (FP32, a few dozen
// particles per thread), and the CTA adds its columns in FP64 into one of STATS_SLOTS global
// partials at the end; the host adds the partials.  The total mass does not change in a step
// and is summed when the state is set.
constexpr int NSTAT = 5;

template <int NT>
__device__ __forceinline__ void particle_stats(float (*col)[NT], const PState &st)
{
    const int t = threadIdx.x;
    col[0][t] += st.mass * st.v[0];
    col[1][t] += st.mass * st.v[1];
    col[2][t] += st.mass * st.v[2];
    col[3][t] += 0.5f * st.mass * (st.v[0] * st.v[0] + st.v[1] * st.v[1] + st.v[2] * st.v[2]);
    float se = 0.f;
#pragma unroll
    for (int k = 0; k < 3; k++) se += st.s[k] * st.e[k];
#pragma unroll
    for (int k = 3; k < 6; k++) se += 2.f * st.s[k] * st.e[k];
    col[4][t] += 0.5f * __fdividef(st.mass, st.rho) * se;  // volume m / rho (diagnostic precision)
}

template <int NT>
__device__ __forceinline__ void stats_cta_flush(double *out, float (*col)[NT])
{
    __syncthreads();
    if (threadIdx.x < NSTAT) {
        double v = 0.0;
        for (int t = 0; t < NT; t++) v += (double)col[threadIdx.x][t];
        atomicAdd(&out[(blockIdx.x % STATS_SLOTS) * 8 + 1 + threadIdx.x], v);
    }
}

// G2P sums of one particle over its 27 stencil nodes from a 6x6x6 node tile, separable per
// axis: for every (j, k) node row the three x nodes are contracted first, then weighted by the
// y/z factors.  TV = (v1x, v1y, v1z, a1z) and TA = (a1x, a1y), zero at massless nodes;
// THERMAL also sums the node (T, rate) tile TN into th = (grad T, T rate).
template <bool THERMAL>
__device__ __forceinline__ void g2p_node_sums(const float4 *TV, const float2 *TA, const float2 *TN, const float o[3],
                                              int key, const GridGeom &g, float acc[3], float vg[3], float L[3][3],
                                              float th[4])
{
    float Sx[3], Gx[3], Sy[3], Gy[3], Sz[3], Gz[3];
    gimp_axis(o[0], g, Sx, Gx);
    gimp_axis(o[1], g, Sy, Gy);
    if (g.is3d) {
        gimp_axis(o[2], g, Sz, Gz);
    } else {
        Sz[0] = 1.f; Sz[1] = 0.f; Sz[2] = 0.f; Gz[0] = 0.f; Gz[1] = 0.f; Gz[2] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        Gx[k] *= g.inv_h;
        Gy[k] *= g.inv_h;
        Gz[k] *= g.inv_h;
    }
    const int lc = key & 63;
    const int t0 = ((lc >> 4) * PT + ((lc >> 2) & 3)) * PT + (lc & 3);
    // FP32x2 sums: x/y components in pairs, the z velocity with the z acceleration
    const float2 z2 = make_float2(0.f, 0.f);
    float2 vg01 = z2, acc01 = z2, vz_az = z2;       // (vg_x, vg_y), (a_x, a_y), (vg_z, a_z)
    float2 Lc0 = z2, Lc1 = z2, Lc2 = z2;            // (L[0][b], L[1][b]) for b = x, y, z
    float L20 = 0.f, L21 = 0.f, L22 = 0.f;           // L[2][b]
    float gtx = 0.f, gty = 0.f, gtz = 0.f, trate = 0.f;
    float2 Sx2[3], Gx2[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        Sx2[k] = make_float2(Sx[k], Sx[k]);
        Gx2[k] = make_float2(Gx[k], Gx[k]);
    }
#pragma unroll
    for (int kk = 0; kk < 3; kk++) {
        if (kk > 0 && !g.is3d) break;
#pragma unroll
        for (int jj = 0; jj < 3; jj++) {
            const float4 *tv = TV + t0 + (kk * PT + jj) * PT;
            const float2 *ta = TA + t0 + (kk * PT + jj) * PT;
            float2 xv01 = z2, xv2a2 = z2, yv01 = z2, xa01 = z2;
            float yv2 = 0.f;
#pragma unroll
            for (int ii = 0; ii < 3; ii++) {
                const float4 V = tv[ii];
                const float2 A = ta[ii];
                xv01 = fma2(Sx2[ii], lo2(V), xv01);
                xv2a2 = fma2(Sx2[ii], hi2(V), xv2a2);
                yv01 = fma2(Gx2[ii], lo2(V), yv01);
                yv2 = fmaf(Gx[ii], V.z, yv2);
                xa01 = fma2(Sx2[ii], A, xa01);
            }
            const float syz = Sy[jj] * Sz[kk], gyz = Gy[jj] * Sz[kk], syg = Sy[jj] * Gz[kk];
            const float2 syz2 = make_float2(syz, syz), gyz2 = make_float2(gyz, gyz);
            const float2 syg2 = make_float2(syg, syg);
            vg01 = fma2(syz2, xv01, vg01);
            vz_az = fma2(syz2, xv2a2, vz_az);
            acc01 = fma2(syz2, xa01, acc01);
            Lc0 = fma2(syz2, yv01, Lc0);
            L20 = fmaf(syz, yv2, L20);
            Lc1 = fma2(gyz2, xv01, Lc1);
            L21 = fmaf(gyz, xv2a2.x, L21);
            Lc2 = fma2(syg2, xv01, Lc2);
            L22 = fmaf(syg, xv2a2.x, L22);
            if (THERMAL) {
                const float2 *tn = TN + t0 + (kk * PT + jj) * PT;
                float xT = 0.f, xgT = 0.f, xR = 0.f;
#pragma unroll
                for (int ii = 0; ii < 3; ii++) {
                    const float2 q = tn[ii];
                    xT = fmaf(Sx[ii], q.x, xT);
                    xgT = fmaf(Gx[ii], q.x, xgT);
                    xR = fmaf(Sx[ii], q.y, xR);
                }
                gtx = fmaf(syz, xgT, gtx);
                gty = fmaf(gyz, xT, gty);
                gtz = fmaf(syg, xT, gtz);
                trate = fmaf(syz, xR, trate);
            }
        }
    }
    acc[0] = acc01.x; acc[1] = acc01.y; acc[2] = vz_az.y;
    vg[0] = vg01.x; vg[1] = vg01.y; vg[2] = vz_az.x;
    L[0][0] = Lc0.x; L[0][1] = Lc1.x; L[0][2] = Lc2.x;
    L[1][0] = Lc0.y; L[1][1] = Lc1.y; L[1][2] = Lc2.y;
    L[2][0] = L20;   L[2][1] = L21;   L[2][2] = L22;
    th[0] = gtx; th[1] = gty; th[2] = gtz; th[3] = trate;
}

// Single-body G2P + update through a shared-memory node tile.  A CTA owns one segment (the
// particles of one 4x4x4 cell block): it loads the block's 6x6x6 solved node tile once, with
// massless nodes zeroed (they are skipped, Extrapolation.cpp:301-303), then runs one thread
// per particle in sorted order.  The G2P sums are separable per axis: for every (j, k) node
// row the three x nodes are contracted first, then weighted by the y/z factors.
// THERMAL adds the heat conduction terms (Extrapolation.cpp:132-134, 358-362 and
// TimeIntegration.cpp:49-50): the node (T, rate) tile, the particle's temperature gradient and
// rate summed with the same weights, and its temperature update, in therm by insertion index.
template <bool HAS_DP, bool THERMAL>
__global__ void __launch_bounds__(GY_G2P_THREADS, THERMAL ? GY_G2P_MINB_TH : GY_G2P_MINB)
    k_g2p_tiled(PView src, PView dst, const int *perm, const int *skey, long long n, const int *seg_start,
                const int *nseg_ptr, int sorted, NodeBufs nb, StepArgs a, int check_finite, float4 *therm,
                const float2 *tnode)
{
    constexpr int NST = G2P_NBASE + (HAS_DP ? G2P_NDP : 0);
    __shared__ float4 TV[PT_NODES];  // (v1x, v1y, v1z, a1z), zero for massless nodes
    __shared__ float2 TA[PT_NODES];  // (a1x, a1y)
    __shared__ float2 TN[THERMAL ? PT_NODES : 1];  // node (T sum, T rate)
    __shared__ float stage[NST][GY_G2P_THREADS];
    __shared__ float s_st[NSTAT][GY_G2P_THREADS];
    __shared__ long long s_end;
    const GridGeom &g = a.g;
    const int nseg = *nseg_ptr;
    const int tid = threadIdx.x;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < NSTAT; k++) s_st[k][tid] = 0.f;  // each thread's own column
    for (int sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
        const long long start = seg_start[sgi];
        const int blk = seg_block(skey, start);
        int bx, by, bz;
        decode_block(blk, g, bx, by, bz);
        const int tox = bx * CB, toy = by * CB, toz = g.is3d ? bz * CB : 0;
        // the solved node tile, loaded into registers before anything waits on it
        constexpr int TILE_ITERS = (PT_NODES + GY_G2P_THREADS - 1) / GY_G2P_THREADS;
        float4 TVr[TILE_ITERS], TAr[TILE_ITERS];
        float2 TNr[THERMAL ? TILE_ITERS : 1];
#pragma unroll
        for (int h = 0; h < TILE_ITERS; h++) {
            const int t = tid + h * GY_G2P_THREADS;
            TVr[h] = z4;
            TAr[h] = z4;
            if (THERMAL) TNr[h] = make_float2(0.f, 0.f);
            const int ni = tox + t % PT, nj = toy + (t / PT) % PT, nk = toz + t / (PT * PT);
            if (t < PT_NODES && ni < g.nx && nj < g.ny && nk < g.nz) {
                const int nd = node_index(ni, nj, nk, g);
                TVr[h] = __ldg(&nb.gv[nd]);
                TAr[h] = __ldg(&nb.ga[nd]);
                if (THERMAL) TNr[h] = __ldg(&tnode[nd]);
            }
        }
        __syncthreads();  // the previous segment's particles are done with the tile
#pragma unroll
        for (int h = 0; h < TILE_ITERS; h++) {
            const int t = tid + h * GY_G2P_THREADS;
            if (t >= PT_NODES) break;
            float4 V = TVr[h], A = TAr[h];
            if (V.x == 0.0f) { V = z4; A = z4; }
            TV[t] = make_float4(V.y, V.z, V.w, A.z);
            TA[t] = make_float2(A.x, A.y);
            if (THERMAL) TN[t] = TNr[h];
        }
        for (long long base = start;; base += blockDim.x) {
            int cnt, key = 0;
            long long j = 0;
            const long long i = base + tid;
            if (sorted) {
                // the particle's key and slot are loaded together; the barrier also publishes
                // the tile.  skey[i] is the key of particle perm[i].
                const bool inr = i < n;
                key = inr ? skey[i] : -1;
                j = inr ? perm[i] : 0;
                cnt = __syncthreads_count(inr && (key >> CB_SHIFT) == blk);
            } else {
                cnt = (int)min((long long)blockDim.x, segment_chunk_end(skey, n, blk, base, blockDim.x, &s_end) - base);
                if (tid < cnt) key = skey[i];
                j = i;
            }
            if (cnt <= 0) break;
            if (tid < cnt) {
                PState st;
                st.key = key;
#pragma unroll
                for (int k = 0; k < 3; k++) st.o[k] = src.f(PF_OX + k, j);
                // the rest of the state travels to shared memory during the G2P sums
#pragma unroll
                for (int f = 0; f < NST; f++) cp_async4(&stage[f][tid], &src.f(g2p_stage_field(f), j));
                cp_async_commit();
                float acc[3], vg[3], L[3][3], thg[4];
                g2p_node_sums<THERMAL>(TV, TA, TN, st.o, st.key, g, acc, vg, L, thg);
                cp_async_wait_all();
#pragma unroll
                for (int k = 0; k < 3; k++) st.v[k] = stage[k][tid];
#pragma unroll
                for (int k = 0; k < 6; k++) {
                    st.s[k] = stage[3 + k][tid];
                    st.e[k] = stage[9 + k][tid];
                }
                st.rho = stage[15][tid];
                st.mass = stage[16][tid];
                st.info = __float_as_uint(stage[17][tid]);
                st.pid = __float_as_int(stage[18][tid]);
                if (HAS_DP) {
                    st.eqps = stage[G2P_NBASE + (HAS_DP ? 0 : 0)][tid];
#pragma unroll
                    for (int k = 0; k < 6; k++) st.ep[k] = stage[G2P_NBASE + (HAS_DP ? 1 + k : 0)][tid];
                    st.dmg = stage[G2P_NBASE + (HAS_DP ? 7 : 0)][tid];
                    st.smax = stage[G2P_NBASE + (HAS_DP ? 8 : 0)][tid];
                } else {
                    st.eqps = 0.f;
#pragma unroll
                    for (int k = 0; k < 6; k++) st.ep[k] = 0.f;
                    st.dmg = 0.f;
                    st.smax = 0.f;
                }
                float4 th = make_float4(0.f, 0.f, 0.f, 0.f);
                if (THERMAL) th = therm[st.pid];  // loads while the update runs
                int c0[3];
                decode_key(st.key, g, c0[0], c0[1], c0[2]);
                if (!g.is3d) c0[2] = 0;
                update_after_g2p<HAS_DP>(st, c0, acc, vg, L, a, check_finite != 0, i);
                store_state<HAS_DP>(dst, i, st);
                if (a.mover_mask && st.key != key) flag_mover(a, i);
                if (THERMAL) therm[st.pid] = make_float4(th.x + thg[3] * a.sc->dt, thg[0], thg[1], thg[2]);
                if (a.stats) particle_stats(s_st, st);
            }
            if (cnt < (int)blockDim.x) break;
        }
    }
    if (a.stats) stats_cta_flush(a.stats, s_st);
}

// Multi-body G2P + update through a shared-memory node tile: per node the body pair (or
// none when the node has no mass, so it is skipped, Extrapolation.cpp:301-303) and both body
// slots' solved fields; each particle reads the slot of its own object (Extrapolation.cpp:
// 311-355), with the weight zeroed where the node holds neither of its bodies.
template <bool HAS_DP, bool NRM>
__global__ void __launch_bounds__(GY_G2PM_THREADS, GY_G2PM_MINB) k_g2p_multi_tiled(PView src, PView dst, const int *perm,
                                                                    const int *skey, long long n,
                                                                    const int *seg_start, const int *nseg_ptr,
                                                                    int sorted, NodeBufs nb, StepArgs a,
                                                                    int check_finite)
{
    constexpr int NST = G2P_NBASE + (HAS_DP ? G2P_NDP : 0);
    __shared__ int2 TP[PT_NODES];
    __shared__ float4 TVb[2][PT_NODES];  // (m, v1) per body slot
    __shared__ float4 TAb[2][PT_NODES];  // (a1, -) per body slot
    __shared__ float4 TN[NRM ? 2 : 1][NRM ? PT_NODES : 1];
    __shared__ float stage[NST][GY_G2PM_THREADS];
    __shared__ float s_st[NSTAT][GY_G2PM_THREADS];
    __shared__ long long s_end;
    const GridGeom &g = a.g;
    const int nseg = *nseg_ptr;
    const int tid = threadIdx.x;
#pragma unroll
    for (int k = 0; k < NSTAT; k++) s_st[k][tid] = 0.f;  // each thread's own column
    for (int sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
        const long long start = seg_start[sgi];
        const int blk = seg_block(skey, start);
        int bx, by, bz;
        decode_block(blk, g, bx, by, bz);
        const int tox = bx * CB, toy = by * CB, toz = g.is3d ? bz * CB : 0;
        // a tile of one body (the cell block's summary): every node with mass and that body
        // carries it in slot 0, whose solved fields the solve also stores as the node's gv / ga,
        // so the particles of that body take the single-body tile and sums; the others see
        // nothing, as in the slot-by-slot sums.  Not with tracked normals.
        const int tb = NRM ? -2 : nb.block_body[blk];
        const bool one = tb >= 0;
        float4 *TV1 = TVb[0];
        float2 *TA1 = reinterpret_cast<float2 *>(TAb[0]);
        __syncthreads();  // the previous segment's particles are done with the tile
        if (one) {
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int t = tid; t < PT_NODES; t += blockDim.x) {
                const int ni = tox + t % PT, nj = toy + (t / PT) % PT, nk = toz + t / (PT * PT);
                float4 V = z4, A = z4;
                if (ni < g.nx && nj < g.ny && nk < g.nz) {
                    const int nd = node_index(ni, nj, nk, g);
                    V = __ldg(&nb.gv[nd]);
                    A = __ldg(&nb.ga[nd]);
                    if (V.x == 0.0f || __ldg(&nb.body[nd].x) < 0) { V = z4; A = z4; }
                }
                TV1[t] = make_float4(V.y, V.z, V.w, A.z);
                TA1[t] = make_float2(A.x, A.y);
            }
        }
        for (int t = tid; t < (one ? 0 : PT_NODES); t += blockDim.x) {
            const int ni = tox + t % PT, nj = toy + (t / PT) % PT, nk = toz + t / (PT * PT);
            int2 pr = make_int2(-1, -1);
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            float4 v0 = z4, v1 = z4, a0 = z4, a1 = z4, n0 = z4, n1 = z4;
            if (ni < g.nx && nj < g.ny && nk < g.nz) {
                const int nd = node_index(ni, nj, nk, g);
                if (__ldg(&nb.gv[nd].x) != 0.0f) {
                    pr = __ldg(&nb.body[nd]);
                    v0 = __ldg(&nb.bgv[0][nd]);
                    v1 = __ldg(&nb.bgv[1][nd]);
                    a0 = __ldg(&nb.bga[0][nd]);
                    a1 = __ldg(&nb.bga[1][nd]);
                    if (NRM) {
                        n0 = __ldg(&nb.nrm_out[0][nd]);
                        n1 = __ldg(&nb.nrm_out[1][nd]);
                    }
                }
            }
            TP[t] = pr;
            TVb[0][t] = v0;
            TVb[1][t] = v1;
            TAb[0][t] = a0;
            TAb[1][t] = a1;
            if (NRM) {
                TN[0][t] = n0;
                TN[1][t] = n1;
            }
        }
        for (long long base = start;; base += blockDim.x) {
            int cnt, key = 0;
            long long j = 0;
            const long long i = base + tid;
            if (sorted) {
                const bool inr = i < n;
                key = inr ? skey[i] : -1;
                j = inr ? perm[i] : 0;
                cnt = __syncthreads_count(inr && (key >> CB_SHIFT) == blk);
            } else {
                cnt = (int)min((long long)blockDim.x, segment_chunk_end(skey, n, blk, base, blockDim.x, &s_end) - base);
                if (tid < cnt) key = skey[i];
                j = i;
            }
            if (cnt <= 0) break;
            if (tid < cnt) {
                PState st;
                st.key = key;
#pragma unroll
                for (int k = 0; k < 3; k++) st.o[k] = src.f(PF_OX + k, j);
                const int obj = info_obj((uint32_t)src.ii(PF_INFO, j));
#pragma unroll
                for (int f = 0; f < NST; f++) cp_async4(&stage[f][tid], &src.f(g2p_stage_field(f), j));
                cp_async_commit();
                float acc[3] = {0.f, 0.f, 0.f}, vg[3] = {0.f, 0.f, 0.f};
                float L[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
                float nrm[3] = {0.f, 0.f, 0.f};
                if (one) {
                    if (obj == tb) {
                        float thg[4];
                        g2p_node_sums<false>(TV1, TA1, nullptr, st.o, st.key, g, acc, vg, L, thg);
                    }
                } else {
                    float S[3][3], G[3][3];
                    gimp_axis(st.o[0], g, S[0], G[0]);
                    gimp_axis(st.o[1], g, S[1], G[1]);
                    if (g.is3d) {
                        gimp_axis(st.o[2], g, S[2], G[2]);
                    } else {
                        S[2][0] = 1.f; S[2][1] = 0.f; S[2][2] = 0.f; G[2][0] = 0.f; G[2][1] = 0.f; G[2][2] = 0.f;
                    }
                    const int lc = st.key & 63;
                    const int t0 = ((lc >> 4) * PT + ((lc >> 2) & 3)) * PT + (lc & 3);
    #pragma unroll
                    for (int kk = 0; kk < 3; kk++) {
                        if (kk > 0 && !g.is3d) break;
    #pragma unroll
                        for (int jj = 0; jj < 3; jj++) {
                            const float syz = S[1][jj] * S[2][kk];
                            const float gyz = G[1][jj] * S[2][kk] * g.inv_h, syg = S[1][jj] * G[2][kk] * g.inv_h;
    #pragma unroll
                            for (int ii = 0; ii < 3; ii++) {
                                const int t = t0 + (kk * PT + jj) * PT + ii;
                                const int2 pr = TP[t];
                                const int slot = (pr.x == obj) ? 0 : ((pr.y == obj) ? 1 : -1);
                                const int sl = slot > 0 ? 1 : 0;
                                const float on = slot >= 0 ? 1.f : 0.f;  // a third body sees nothing here
                                const float4 Vb = TVb[sl][t], Ab = TAb[sl][t];
                                const float wgt = S[0][ii] * syz * on;
                                const float gx = G[0][ii] * syz * g.inv_h * on, gy = S[0][ii] * gyz * on;
                                const float gz = S[0][ii] * syg * on;
                                acc[0] += wgt * Ab.x; acc[1] += wgt * Ab.y; acc[2] += wgt * Ab.z;
                                vg[0] += wgt * Vb.y; vg[1] += wgt * Vb.z; vg[2] += wgt * Vb.w;
                                L[0][0] += Vb.y * gx; L[0][1] += Vb.y * gy; L[0][2] += Vb.y * gz;
                                L[1][0] += Vb.z * gx; L[1][1] += Vb.z * gy; L[1][2] += Vb.z * gz;
                                L[2][0] += Vb.w * gx; L[2][1] += Vb.w * gy; L[2][2] += Vb.w * gz;
                                if (NRM) {
                                    const float4 N = TN[sl][t];
                                    nrm[0] += wgt * N.x; nrm[1] += wgt * N.y; nrm[2] += wgt * N.z;
                                }
                            }
                        }
                    }
                }
                cp_async_wait_all();
#pragma unroll
                for (int k = 0; k < 3; k++) st.v[k] = stage[k][tid];
#pragma unroll
                for (int k = 0; k < 6; k++) {
                    st.s[k] = stage[3 + k][tid];
                    st.e[k] = stage[9 + k][tid];
                }
                st.rho = stage[15][tid];
                st.mass = stage[16][tid];
                st.info = __float_as_uint(stage[17][tid]);
                st.pid = __float_as_int(stage[18][tid]);
                if (HAS_DP) {
                    st.eqps = stage[G2P_NBASE + (HAS_DP ? 0 : 0)][tid];
#pragma unroll
                    for (int k = 0; k < 6; k++) st.ep[k] = stage[G2P_NBASE + (HAS_DP ? 1 + k : 0)][tid];
                    st.dmg = stage[G2P_NBASE + (HAS_DP ? 7 : 0)][tid];
                    st.smax = stage[G2P_NBASE + (HAS_DP ? 8 : 0)][tid];
                } else {
                    st.eqps = 0.f;
#pragma unroll
                    for (int k = 0; k < 6; k++) st.ep[k] = 0.f;
                    st.dmg = 0.f;
                    st.smax = 0.f;
                }
                int c0[3];
                decode_key(st.key, g, c0[0], c0[1], c0[2]);
                if (!g.is3d) c0[2] = 0;
                update_after_g2p<HAS_DP>(st, c0, acc, vg, L, a, check_finite != 0, i);
                store_state<HAS_DP>(dst, i, st);
                if (a.mover_mask && st.key != key) flag_mover(a, i);
                if (NRM) {
                    dst.f(PF_NX, i) = nrm[0];
                    dst.f(PF_NY, i) = nrm[1];
                    dst.f(PF_NZ, i) = nrm[2];
                }
                if (a.stats) particle_stats(s_st, st);
            }
            if (cnt < (int)blockDim.x) break;
        }
    }
    if (a.stats) stats_cta_flush(a.stats, s_st);
}

int g2p_blocks_per_sm(bool has_dp)
{
    int b = 0;
    if (has_dp) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_g2p_tiled<true, false>, GY_G2P_THREADS, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_g2p_tiled<false, false>, GY_G2P_THREADS, 0);
    return b > 0 ? b : 1;
}

void launch_g2p_update(const PView &src, const PView &dst, const int *perm, const int *skey, long long n,
                       const int *seg_start, const int *nseg, int g2p_grid, const NodeBufs &nb, const StepArgs &a,
                       bool track_normals, bool check_finite, bool has_dp, cudaStream_t s, float4 *therm,
                       const float2 *tnode)
{
    if (n == 0) return;
    const int tn = track_normals ? 1 : 0, cf = check_finite ? 1 : 0;
    if (a.multi_body) {
        const int srt = perm ? 1 : 0;
        static int mgrid[4] = {0, 0, 0, 0};  // persistent grids of the four multi-body variants
        const int vi = (has_dp ? 2 : 0) + (tn ? 1 : 0);
        if (mgrid[vi] == 0) {
            int dev = 0, sms = 1, b = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            const void *k = vi == 3 ? (const void *)k_g2p_multi_tiled<true, true>
                          : vi == 2 ? (const void *)k_g2p_multi_tiled<true, false>
                          : vi == 1 ? (const void *)k_g2p_multi_tiled<false, true>
                                    : (const void *)k_g2p_multi_tiled<false, false>;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, GY_G2PM_THREADS, 0);
            mgrid[vi] = sms * std::max(b, 1);
        }
        const unsigned mg = (unsigned)mgrid[vi];
        if (has_dp && tn)
            k_g2p_multi_tiled<true, true><<<mg, GY_G2PM_THREADS, 0, s>>>(src, dst, perm, skey, n, seg_start, nseg, srt, nb, a, cf);
        else if (has_dp)
            k_g2p_multi_tiled<true, false><<<mg, GY_G2PM_THREADS, 0, s>>>(src, dst, perm, skey, n, seg_start, nseg, srt, nb, a, cf);
        else if (tn)
            k_g2p_multi_tiled<false, true><<<mg, GY_G2PM_THREADS, 0, s>>>(src, dst, perm, skey, n, seg_start, nseg, srt, nb, a, cf);
        else
            k_g2p_multi_tiled<false, false><<<mg, GY_G2PM_THREADS, 0, s>>>(src, dst, perm, skey, n, seg_start, nseg, srt, nb, a, cf);
    } else {
        const int srt = perm ? 1 : 0;
        if (therm) {
            static int tgrid[2] = {0, 0};  // persistent grids of the variants with heat conduction
            if (tgrid[has_dp] == 0) {
                int dev = 0, sms = 1, b = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                if (has_dp) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_g2p_tiled<true, true>, GY_G2P_THREADS, 0);
                else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_g2p_tiled<false, true>, GY_G2P_THREADS, 0);
                tgrid[has_dp] = sms * std::max(b, 1);
            }
            if (has_dp)
                k_g2p_tiled<true, true><<<tgrid[1], GY_G2P_THREADS, 0, s>>>(src, dst, perm, skey, n, seg_start, nseg, srt,
                                                                             nb, a, cf, therm, tnode);
            else
                k_g2p_tiled<false, true><<<tgrid[0], GY_G2P_THREADS, 0, s>>>(src, dst, perm, skey, n, seg_start, nseg, srt,
                                                                              nb, a, cf, therm, tnode);
        } else if (has_dp) {
            k_g2p_tiled<true, false><<<g2p_grid, GY_G2P_THREADS, 0, s>>>(src, dst, perm, skey, n, seg_start, nseg, srt, nb,
                                                                          a, cf, nullptr, nullptr);
        } else {
            k_g2p_tiled<false, false><<<g2p_grid, GY_G2P_THREADS, 0, s>>>(src, dst, perm, skey, n, seg_start, nseg, srt, nb,
                                                                           a, cf, nullptr, nullptr);
        }
    }
    note_launch(1);
}

// ---------------------------------------------------------------------------------------
// Body slots (Extrapolation.cpp:191-208).  The reference assigns each node's two body slots
// to the objects of the first particles it visits in its 4x4x4 cell window (cells in
// increasing linear id, particles in sorted order within a cell), using the cell table of
// the last sort.  Here a per-(cell, object) table holds the smallest particle id of that
// object in the cell (the within-cell order both sides use) plus a rigid bit per object,
// and each node scans its window in the reference's order.

constexpr int NO_PARTICLE = 0x7fffffff;

__global__ void k_body_tables(PView P, long long n, StepArgs a, int *cell_min, int nbody, const int *refkeys)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t info = (uint32_t)P.ii(PF_INFO, i);
    const int obj = info_obj(info);
    const int pid = P.ii(PF_PID, i);
    int rk;
    if (refkeys) {
        rk = refkeys[pid];
    } else {
        // the reference's binning key from the current position (TimeIntegration.cpp:110-115)
        int ci, cj, ck;
        decode_key(P.ii(PF_KEY, i), a.g, ci, cj, ck);
        const int ix = (int)((float)ci + P.f(PF_OX, i) - 0.25f);
        const int iy = (int)((float)cj + P.f(PF_OY, i) - 0.25f);
        const int iz = a.g.is3d ? (int)((float)ck + P.f(PF_OZ, i) - 0.25f) : 0;
        rk = ix + iy * a.g.ncx + iz * a.g.ncx * a.g.ncy;
    }
    if (rk < 0 || rk >= a.g.nc) return;
    atomicMin(&cell_min[(long long)rk * (nbody + 1) + obj], pid);
    if (info & INFO_RIGID) atomicOr(&cell_min[(long long)rk * (nbody + 1) + nbody], 1 << obj);
}

__global__ void k_body_clear(int *cell_min, long long nc, int nbody)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int *row = cell_min + c * (nbody + 1);
    for (int b = 0; b < nbody; b++) row[b] = NO_PARTICLE;
    row[nbody] = 0;
}

void launch_body_tables(const PView &p, long long n, const StepArgs &a, int *cell_min, int nbody,
                        const int *refkeys, cudaStream_t s)
{
    k_body_clear<<<(unsigned)((a.g.nc + 255) / 256), 256, 0, s>>>(cell_min, a.g.nc, nbody);
    note_launch(1);
    if (n == 0) return;
    k_body_tables<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p, n, a, cell_min, nbody, refkeys);
    note_launch(1);
}

// Body pair of every node (Extrapolation.cpp:191-208): the window of 4x4x4 cells from the
// node's cell - 2 is scanned in k, j, i order; the first particle of the first occupied cell
// names body 1, and the first particle of another object in that or a later cell names body
// 2; the rigid flags are ORed over the whole window.  Cells are addressed by the linear cell
// index as the reference forms it (an index outside [0, nc) is skipped, one outside a row
// wraps into the neighbouring row).
//
// One CTA per 4x4x4 node block: the union of its nodes' windows (at most 8 cells per axis) is
// summarised into shared memory once, one word per cell -- its first and second body by
// particle order and its rigid bits -- so each node's 64-cell scan reads shared memory.  With
// the first body b1 of the first occupied cell fixed, a later cell's "first particle of
// another object" is its first body when that differs from b1, else its second.
constexpr int BA_SPAN = 8;

__device__ __forceinline__ int body_cell_summary(const int *row, int nbody)
{
    int f = -1, fp = NO_PARTICLE, s2 = -1, sp = NO_PARTICLE;
    for (int b = 0; b < nbody; b++) {
        const int pid = row[b];
        if (pid == NO_PARTICLE) continue;
        if (pid < fp) { s2 = f; sp = fp; f = b; fp = pid; }
        else if (pid < sp) { s2 = b; sp = pid; }
    }
    return (f + 1) | ((s2 + 1) << 5) | (row[nbody] << 10);
}

__global__ void __launch_bounds__(64) k_body_assign(NodeBufs nb, GridGeom g, const int *cell_min, int nbody,
                                                    const int *nidx_x, const int *nidx_y, const int *nidx_z)
{
    __shared__ int cs[BA_SPAN * BA_SPAN * BA_SPAN];
    const long long blk = blockIdx.x;
    const int bx = (int)(blk % g.nnbx), by = (int)((blk / g.nnbx) % g.nnby), bz = (int)(blk / ((long long)g.nnbx * g.nnby));
    const int i0 = bx * 4, j0 = by * 4, k0 = bz * 4;
    const int cx0 = nidx_x[i0] - 2, cy0 = nidx_y[j0] - 2, cz0 = g.is3d ? nidx_z[k0] - 2 : 0;
    const int zspan = g.is3d ? BA_SPAN : 1;
    const int stride = nbody + 1;
    const long long plane = (long long)g.ncx * g.ncy;
    for (int q = threadIdx.x; q < BA_SPAN * BA_SPAN * zspan; q += blockDim.x) {
        const int lx = q % BA_SPAN, ly = (q / BA_SPAN) % BA_SPAN, lz = q / (BA_SPAN * BA_SPAN);
        const long long c = (long long)(cx0 + lx) + (long long)(cy0 + ly) * g.ncx + (long long)(cz0 + lz) * plane;
        cs[q] = (c >= 0 && c < g.nc) ? body_cell_summary(cell_min + c * stride, nbody) : 0;
    }
    __syncthreads();
    const int lx = threadIdx.x & 3, ly = (threadIdx.x >> 2) & 3, lz = threadIdx.x >> 4;
    const int i = i0 + lx, j = j0 + ly, k = k0 + lz;
    if (i >= g.nx || j >= g.ny || k >= g.nz) return;
    const int ox = nidx_x[i] - cx0, oy = nidx_y[j] - cy0, oz = g.is3d ? nidx_z[k] - cz0 : 2;
    int b0 = -1, b1 = -1;
    int rig = 0;  // OR of rigid bits over the window
    const int kmin = g.is3d ? -2 : 0, kmax = g.is3d ? 2 : 1;
    for (int kk = kmin; kk < kmax; kk++)
        for (int jj = -2; jj < 2; jj++)
            for (int ii = -2; ii < 2; ii++) {
                const int v = cs[((g.is3d ? oz + kk : 0) * BA_SPAN + (oy + jj)) * BA_SPAN + (ox + ii)];
                rig |= v >> 10;
                if (b1 != -1) continue;
                const int first = (v & 31) - 1;
                if (first < 0) continue;
                if (b0 == -1) b0 = first;
                const int other = first != b0 ? first : ((v >> 5) & 31) - 1;
                if (other >= 0) b1 = other;
            }
    const long long nd = node_index(i, j, k, g);
    nb.body[nd] = make_int2(b0, b1);
    unsigned char hr = 0;
    if (b0 >= 0 && (rig >> b0) & 1) hr |= 1;
    if (b1 >= 0 && (rig >> b1) & 1) hr |= 2;
    nb.has_rigid[nd] = hr;
}

// Per 4x4x4 cell block, the body of its 6x6x6 node tile when the tile has one (every node with
// body pair (b, -1) or (-1, -1)): b, -1 for none, -2 for two or more; one warp per block.
// P2G sends the one-object segments of such blocks to the plane-lane kernel.
__global__ void __launch_bounds__(128) k_block_body(NodeBufs nb, GridGeom g)
{
    const int lane = threadIdx.x & 31;
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= (long long)g.nbx * g.nby * g.nbz) return;  // whole warps
    int bx, by, bz;
    decode_block((int)w, g, bx, by, bz);
    const int tox = bx * CB, toy = by * CB, toz = g.is3d ? bz * CB : 0;
    bool two = false;
    int lo = 0x7fffffff, hi = -1;
    for (int t = lane; t < PT_NODES; t += 32) {
        const int ni = tox + t % PT, nj = toy + (t / PT) % PT, nk = toz + t / (PT * PT);
        if (ni >= g.nx || nj >= g.ny || nk >= g.nz) continue;
        const int2 pr = nb.body[node_index(ni, nj, nk, g)];
        two = two || pr.y != -1;
        if (pr.x >= 0) {
            lo = min(lo, pr.x);
            hi = max(hi, pr.x);
        }
    }
    two = __any_sync(0xffffffffu, two);
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (lane == 0) nb.block_body[w] = (two || (hi >= 0 && lo != hi)) ? -2 : hi;
}

void launch_body_assign(const NodeBufs &nb, const StepArgs &a, const int *cell_min, int nbody, const int *nidx_x,
                        const int *nidx_y, const int *nidx_z, cudaStream_t s)
{
    k_body_assign<<<(unsigned)a.g.nnb, 64, 0, s>>>(nb, a.g, cell_min, nbody, nidx_x, nidx_y, nidx_z);
    note_launch(1);
    launch_block_body(nb, a.g, s);
}

// Per 4x4x4 node block: whether one of its nodes holds two bodies (one warp per block).
__global__ void __launch_bounds__(128) k_nblock_two(NodeBufs nb, GridGeom g)
{
    const int lane = threadIdx.x & 31;
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= g.nnb) return;  // whole warps
    const int b32 = (int)w;
    const int bx = b32 % g.nnbx, tb = b32 / g.nnbx;
    const int by = tb % g.nnby, bz = tb / g.nnby;
    bool two = false;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int ln = lane + 32 * h;
        const int i = bx * 4 + (ln & 3), j = by * 4 + ((ln >> 2) & 3), k = bz * 4 + (ln >> 4);
        if (i < g.nx && j < g.ny && k < g.nz) two = two || nb.body[node_index(i, j, k, g)].y != -1;
    }
    two = __any_sync(0xffffffffu, two);
    if (lane == 0) nb.nblk_two[w] = two ? 1 : 0;
}

void launch_block_body(const NodeBufs &nb, const GridGeom &g, cudaStream_t s)
{
    const long long ncb = (long long)g.nbx * g.nby * g.nbz;
    k_block_body<<<(unsigned)((ncb + 3) / 4), 128, 0, s>>>(nb, g);
    k_nblock_two<<<(unsigned)((g.nnb + 3) / 4), 128, 0, s>>>(nb, g);
    note_launch(2);
}

// ---------------------------------------------------------------------------------------
// Slab reorder: dst field f slot i = src field f slot perm[i], 32-bit words (every field).

__global__ void __launch_bounds__(256) k_gather_slab(const float *src, float *dst, const int *perm, long long n,
                                                     long long cap, int nfields)
{
    const long long total = n * nfields;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const long long f = q / n, i = q - f * n;
        dst[f * cap + i] = src[f * cap + perm[i]];
    }
}

void launch_gather_slab(const float *src, float *dst, const int *perm, long long n, long long cap, int nfields,
                        cudaStream_t s)
{
    if (n <= 0) return;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long grid = std::min<long long>((n * nfields + 255) / 256, (long long)sms * 16);
    k_gather_slab<<<(unsigned)grid, 256, 0, s>>>(src, dst, perm, n, cap, nfields);
    note_launch(1);
}

// ---------------------------------------------------------------------------------------
// Conservation sums: mass, momentum, kinetic energy, strain energy, of a state that no step
// has summed (after initialisation or a state load; a step's G2P sums its own output).
// Each thread sums its few particles in FP32 (the state's own precision), the mass in FP64
// so that its total is exact to FP64 rounding; warps, CTAs and the grid add in FP64 into the
// first partial slot.

__global__ void k_stats(PView P, long long n, double *out)
{
    __shared__ double sh[8][8];
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    double msum = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float m = P.f(PF_MASS, i);
        const float vx = P.f(PF_VX, i), vy = P.f(PF_VY, i), vz = P.f(PF_VZ, i);
        msum += (double)m;
        acc[1] += m * vx;
        acc[2] += m * vy;
        acc[3] += m * vz;
        acc[4] += 0.5f * m * (vx * vx + vy * vy + vz * vz);
        const float V = m / P.f(PF_RHO, i);
        float se = 0.f;
#pragma unroll
        for (int k = 0; k < 3; k++) se += P.f(PF_S0 + k, i) * P.f(PF_E0 + k, i);
#pragma unroll
        for (int k = 3; k < 6; k++) se += 2.f * P.f(PF_S0 + k, i) * P.f(PF_E0 + k, i);
        acc[5] += 0.5f * V * se;
    }
#pragma unroll
    for (int k = 0; k < 6; k++) {
        double v = k == 0 ? msum : (double)acc[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffff, v, off);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += sh[w][threadIdx.x];
        atomicAdd(&out[threadIdx.x], v);
    }
}

void launch_stats(const PView &p, long long n, double *out8, cudaStream_t s)
{
    cudaMemsetAsync(out8, 0, STATS_SLOTS * 8 * sizeof(double), s);
    if (n == 0) return;
    long long blocks = (n + 255) / 256;
    if (blocks > 2048) blocks = 2048;
    k_stats<<<(unsigned)blocks, 256, 0, s>>>(p, n, out8);
    note_launch(1);
}

}  // namespace gy
