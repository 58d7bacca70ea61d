// gy_thermal.cu -- heat conduction terms of the step, run only when a particle temperature
// has been set (otherwise every term is zero: node temperature sum S T m c = 0).
//
// Reference: P2G Extrapolation.cpp:280-283 (node temperature sum_p S T m c, not normalised
// by the thermal mass, and node rate -sum_p (m / rho) k grad S . grad T_p with the particle
// gradient of the previous G2P; a rigid particle counts with m = 1), G2P
// Extrapolation.cpp:132-134, 358-362 (grad T_p = sum grad S T_node, rate = sum S rate_node
// over nodes with mass, whatever their bodies), update TimeIntegration.cpp:49-50
// (T += rate dt for every particle).  No periodic fold and no node BC acts on these fields
// (Grid.cpp:310-795 folds only mass, momentum and force; the temperature BC bodies are
// empty, Grid.cpp:991-1094).
//
// State: a float4 (T, dT/dx, dT/dy, dT/dz) per particle indexed by insertion index, so the
// sort never moves it, and a float2 (T, rate) per node, zero outside the step's active node
// blocks.  Each pass is one segment-tiled kernel like the mechanical P2G and G2P: a CTA
// owns a 4x4x4 cell block and its 6x6x6 node tile in shared memory.
#include <algorithm>

#include "gy_kernels.cuh"

namespace gy {

namespace {

constexpr int TT = 6;                 // node tile edge
constexpr int TT_NODES = TT * TT * TT;
constexpr int TH_THREADS = 128;       // particles per chunk = threads per CTA
constexpr int TH_NP = TH_THREADS + 1;

__device__ __forceinline__ long long th_chunk_end(const int *skey, long long n, int blk, long long base,
                                                  long long *s_end)
{
    if (threadIdx.x == 0) *s_end = base + TH_THREADS;
    __syncthreads();
    const long long i = base + threadIdx.x;
    if (!(i < n && (skey[i] >> CB_SHIFT) == blk)) atomicMin((unsigned long long *)s_end, (unsigned long long)i);
    __syncthreads();
    const long long e = *s_end;
    __syncthreads();
    return e;
}

// P2G of the two thermal node fields.  Runs of equal cell share their 27 stencil nodes: a
// warp takes a run with lane k owning stencil node k and sums its particles in registers,
// then adds two shared atomics per node; the tile is flushed with global adds.
__global__ void __launch_bounds__(TH_THREADS) k_thermal_p2g(PView P, const float4 *therm, const int *perm,
                                                            const int *skey, long long n, const int *seg_start,
                                                            const int *nseg_ptr, int sorted, float2 *tnode,
                                                            StepArgs a)
{
    __shared__ float tile[2 * TT_NODES];
    __shared__ float2 W[9][TH_NP];   // (S, G) per axis/stencil node and particle
    __shared__ float4 Q[TH_THREADS]; // (T m c, (m / rho) k dT/dx / h, .. y, .. z)
    __shared__ int run_start[TH_THREADS + 1];
    __shared__ int run_cell[TH_THREADS];
    __shared__ int wcount[TH_THREADS / 32];
    __shared__ long long s_end;
    const GridGeom &g = a.g;
    const int nseg = *nseg_ptr;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int ii = lane % 3, jj = (lane / 3) % 3, kk = min(lane / 9, 2);
    const bool scatter_lane = lane < 27;
    for (int sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
        const long long start = seg_start[sgi];
        const int blk = skey[start] >> CB_SHIFT;
        int bx, by, bz;
        decode_block(blk, g, bx, by, bz);
        const int tox = bx * CB, toy = by * CB, toz = g.is3d ? bz * CB : 0;
        for (int t = tid; t < 2 * TT_NODES; t += TH_THREADS) tile[t] = 0.f;
        for (long long base = start;; base += TH_THREADS) {
            const long long i = base + tid;
            int cnt, kc = -1, kp = -1;
            long long j = 0;
            if (sorted) {
                const bool inr = i < n;
                kc = inr ? skey[i] : -1;
                kp = (inr && tid > 0) ? skey[i - 1] : -1;
                j = inr ? perm[i] : 0;
                cnt = __syncthreads_count(inr && (kc >> CB_SHIFT) == blk);
            } else {
                cnt = (int)min((long long)TH_THREADS, th_chunk_end(skey, n, blk, base, &s_end) - base);
                if (tid < cnt) {
                    kc = skey[i];
                    kp = tid > 0 ? skey[i - 1] : -1;
                }
                j = i;
            }
            if (cnt <= 0) break;
            const bool valid = tid < cnt;
            const int cell = kc & 63;
            const bool head = valid && (tid == 0 || (kp & 63) != cell);
            if (valid) {
                float S[3], G[3];
                gimp_axis(P.f(PF_OX, j), g, S, G);
#pragma unroll
                for (int k = 0; k < 3; k++) W[k][tid] = make_float2(S[k], G[k]);
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
                const DevMaterial &M = a.mats[info_mat(info)];
                const float m = (info & INFO_RIGID) ? 1.f : P.f(PF_MASS, j);  // Extrapolation.cpp:183
                const float4 th = therm[P.ii(PF_PID, j)];
                const float vk = (m / P.f(PF_RHO, j)) * M.k_th * g.inv_h;
                Q[tid] = make_float4(th.x * m * M.c_th, vk * th.y, vk * th.z, vk * th.w);
            }
            const unsigned hm = __ballot_sync(0xffffffffu, head);
            if (lane == 0) wcount[warp] = __popc(hm);
            __syncthreads();
            int wbase = 0, R = 0;
#pragma unroll
            for (int w2 = 0; w2 < TH_THREADS / 32; w2++) {
                const int c = wcount[w2];
                wbase += (w2 < warp) ? c : 0;
                R += c;
            }
            if (head) {
                const int r = wbase + __popc(hm & lt);
                run_start[r] = tid;
                run_cell[r] = cell;
            }
            if (tid == 0) run_start[R] = cnt;
            __syncthreads();
            for (int r = warp; r < R; r += TH_THREADS / 32) {
                const int p0 = run_start[r], p1 = run_start[r + 1];
                float tn = 0.f, rn = 0.f;
                for (int p = p0; p < p1; p++) {
                    const float2 X = W[ii][p], Y = W[3 + jj][p], Z = W[6 + kk][p];
                    const float4 q = Q[p];
                    const float syz = Y.x * Z.x;
                    tn = fmaf(X.x * syz, q.x, tn);
                    rn = fmaf(X.y * syz, q.y, fmaf(X.x * Y.y * Z.x, q.z, fmaf(X.x * Y.x * Z.y, q.w, rn)));
                }
                if (!scatter_lane || (tn == 0.f && rn == 0.f)) continue;
                const int c = run_cell[r];
                const int t = (((c >> 4) + kk) * TT + (((c >> 2) & 3) + jj)) * TT + ((c & 3) + ii);
                atomicAdd(&tile[t], tn);
                atomicAdd(&tile[TT_NODES + t], -rn);
            }
            if (cnt < TH_THREADS) break;
        }
        __syncthreads();
        for (int t = tid; t < TT_NODES; t += TH_THREADS) {
            const float tn = tile[t], rn = tile[TT_NODES + t];
            if (tn == 0.f && rn == 0.f) continue;
            const int ni = tox + t % TT, nj = toy + (t / TT) % TT, nk = toz + t / (TT * TT);
            if (ni >= g.nx || nj >= g.ny || nk >= g.nz) continue;
            float2 *dst = &tnode[node_index(ni, nj, nk, g)];
            atomicAdd(&dst->x, tn);
            atomicAdd(&dst->y, rn);
        }
        __syncthreads();
    }
}

// G2P of the temperature gradient and rate, and the temperature update, thread per particle
// over the segment's node tile.
__global__ void __launch_bounds__(TH_THREADS) k_thermal_g2p(PView P, float4 *therm, const int *perm,
                                                            const int *skey, long long n, const int *seg_start,
                                                            const int *nseg_ptr, int sorted, const float2 *tnode,
                                                            StepArgs a)
{
    __shared__ float2 TN[TT_NODES];
    __shared__ long long s_end;
    const GridGeom &g = a.g;
    const int nseg = *nseg_ptr;
    const int tid = threadIdx.x;
    const float dt = a.sc->dt;
    for (int sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
        const long long start = seg_start[sgi];
        const int blk = skey[start] >> CB_SHIFT;
        int bx, by, bz;
        decode_block(blk, g, bx, by, bz);
        const int tox = bx * CB, toy = by * CB, toz = g.is3d ? bz * CB : 0;
        __syncthreads();  // the previous segment's particles are done with the tile
        for (int t = tid; t < TT_NODES; t += TH_THREADS) {
            const int ni = tox + t % TT, nj = toy + (t / TT) % TT, nk = toz + t / (TT * TT);
            TN[t] = (ni < g.nx && nj < g.ny && nk < g.nz) ? tnode[node_index(ni, nj, nk, g)] : make_float2(0.f, 0.f);
        }
        for (long long base = start;; base += TH_THREADS) {
            const long long i = base + tid;
            int cnt, key = 0;
            long long j = 0;
            if (sorted) {
                const bool inr = i < n;
                key = inr ? skey[i] : -1;
                j = inr ? perm[i] : 0;
                cnt = __syncthreads_count(inr && (key >> CB_SHIFT) == blk);
            } else {
                cnt = (int)min((long long)TH_THREADS, th_chunk_end(skey, n, blk, base, &s_end) - base);
                if (tid < cnt) key = skey[i];
                j = i;
            }
            if (cnt <= 0) break;
            if (tid < cnt) {
                float Sx[3], Gx[3], Sy[3], Gy[3], Sz[3], Gz[3];
                gimp_axis(P.f(PF_OX, j), g, Sx, Gx);
                gimp_axis(P.f(PF_OY, j), g, Sy, Gy);
                if (g.is3d) {
                    gimp_axis(P.f(PF_OZ, j), g, Sz, Gz);
                } else {
                    Sz[0] = 1.f; Sz[1] = 0.f; Sz[2] = 0.f; Gz[0] = 0.f; Gz[1] = 0.f; Gz[2] = 0.f;
                }
                const int lc = key & 63;
                const int t0 = ((lc >> 4) * TT + ((lc >> 2) & 3)) * TT + (lc & 3);
                float gtx = 0.f, gty = 0.f, gtz = 0.f, rate = 0.f;
#pragma unroll
                for (int kk = 0; kk < 3; kk++) {
#pragma unroll
                    for (int jj = 0; jj < 3; jj++) {
#pragma unroll
                        for (int ii = 0; ii < 3; ii++) {
                            const float2 v = TN[t0 + (kk * TT + jj) * TT + ii];
                            const float syz = Sy[jj] * Sz[kk];
                            gtx = fmaf(Gx[ii] * syz, v.x, gtx);
                            gty = fmaf(Sx[ii] * Gy[jj] * Sz[kk], v.x, gty);
                            gtz = fmaf(Sx[ii] * Sy[jj] * Gz[kk], v.x, gtz);
                            rate = fmaf(Sx[ii] * syz, v.y, rate);
                        }
                    }
                }
                const int pid = P.ii(PF_PID, j);
                float4 th = therm[pid];
                th.x += rate * dt;
                th.y = gtx * g.inv_h;
                th.z = gty * g.inv_h;
                th.w = gtz * g.inv_h;
                therm[pid] = th;
            }
            if (cnt < (int)blockDim.x) break;
        }
    }
}

// zero the node fields of the step's active node blocks (every node P2G reached)
__global__ void __launch_bounds__(256) k_thermal_clear(NodeBufs nb, GridGeom g, float2 *tnode)
{
    const int nact = *nb.active_n;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < 64LL * nact;
         q += (long long)gridDim.x * blockDim.x) {
        const int blk = nb.active_list[q >> 6], ln = (int)(q & 63);
        const int bx = blk % g.nnbx, tb = blk / g.nnbx;
        const int by = tb % g.nnby, bz = tb / g.nnby;
        const int i = bx * 4 + (ln & 3), j = by * 4 + ((ln >> 2) & 3), k = bz * 4 + (ln >> 4);
        if (i < g.nx && j < g.ny && k < g.nz) tnode[node_index(i, j, k, g)] = make_float2(0.f, 0.f);
    }
}

// MaterialPoints::setTemp between steps: therm[id].x = T for the listed insertion indices
__global__ void k_thermal_set(float4 *therm, const int *ids, const float *T, int count, long long n)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    const int id = ids[q];
    if (id >= 0 && id < n) therm[id].x = T[q];  // the host checked the indices
}

int grid_of(long long work, int per_cta_threads, int cap_per_sm)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (work + per_cta_threads - 1) / per_cta_threads;
    return (int)std::max<long long>(1, std::min<long long>(want, (long long)sms * cap_per_sm));
}

}  // namespace

void launch_thermal_p2g(const PView &p, const float4 *therm, const int *perm, const int *skey, long long n,
                        const int *seg_start, const int *nseg, float2 *tnode, const StepArgs &a, cudaStream_t s)
{
    if (n == 0) return;
    static int grid = 0;
    if (grid == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_thermal_p2g, TH_THREADS, 0);
        grid = grid_of((long long)1 << 40, 1, std::max(b, 1));
    }
    k_thermal_p2g<<<grid, TH_THREADS, 0, s>>>(p, therm, perm, skey, n, seg_start, nseg, perm ? 1 : 0, tnode, a);
    note_launch(1);
}

void launch_thermal_g2p(const PView &p, float4 *therm, const int *perm, const int *skey, long long n,
                        const int *seg_start, const int *nseg, const float2 *tnode, const NodeBufs &nb,
                        const StepArgs &a, cudaStream_t s)
{
    if (n == 0) return;
    static int grid = 0;
    if (grid == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_thermal_g2p, TH_THREADS, 0);
        grid = grid_of((long long)1 << 40, 1, std::max(b, 1));
    }
    k_thermal_g2p<<<grid, TH_THREADS, 0, s>>>(p, therm, perm, skey, n, seg_start, nseg, perm ? 1 : 0, tnode, a);
    note_launch(1);
    launch_thermal_clear(nb, a, const_cast<float2 *>(tnode), s);
}

void launch_thermal_clear(const NodeBufs &nb, const StepArgs &a, float2 *tnode, cudaStream_t s)
{
    k_thermal_clear<<<grid_of(64LL * a.g.nnb, 256, 8), 256, 0, s>>>(nb, a.g, tnode);
    note_launch(1);
}

void launch_thermal_set(float4 *therm, const int *ids, const float *T, int count, long long n, cudaStream_t s)
{
    if (count <= 0) return;
    k_thermal_set<<<(count + 255) / 256, 256, 0, s>>>(therm, ids, T, count, n);
    note_launch(1);
}

}  // namespace gy
