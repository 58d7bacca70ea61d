// gy_sort.cu -- stable counting sort of particles by cell.
//
// The reference sorts particle indices by cellID with std::sort and permutes ~40 arrays
// (Extrapolation.cpp:370-503).  Here only the keys are sorted -- the permutation is applied
// by the particle kernels, which read their input through it -- with a stable
// least-significant-digit radix
// sort over 8-bit digits of the cell key: per pass one histogram kernel, one exclusive scan
// over the (digit, block) counts and one stable scatter.  Stability within a pass comes
// from a block-local rank: warps walk their elements in order, peers with the same digit
// are found with __match_any_sync, and per-warp digit counters are prefix-summed across
// warps.  The result is bit-identical to a CPU stable sort of the same keys.
#include <algorithm>
#include <mutex>

#include "../../include/graphyt_gpu.h"
#include "gy_kernels.cuh"

namespace gy {

constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 8;                       // per thread
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS; // 2048 elements per block
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int RADIX = 256;

__global__ void __launch_bounds__(SORT_THREADS) k_radix_hist(const int *keys, long long n, int shift, int *hist, int nblocks)
{
    pdl_prologue();
    __shared__ int cnt[RADIX];
    for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) cnt[d] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * SORT_TILE;
    for (int it = 0; it < SORT_ITEMS; it++) {
        const long long e = base + (long long)it * SORT_THREADS + threadIdx.x;
        if (e < n) atomicAdd(&cnt[(keys[e] >> shift) & 0xFF], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) hist[(long long)d * nblocks + blockIdx.x] = cnt[d];
}

__global__ void __launch_bounds__(SORT_THREADS) k_radix_scatter(const int *keys_in, const int *vals_in, int *keys_out,
                                                                 int *vals_out, long long n, int shift,
                                                                 const int *offsets, int nblocks)
{
    pdl_prologue();
    __shared__ int wcnt[SORT_WARPS][RADIX];   // per-warp digit counts, then per-warp bases
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int d = lane; d < RADIX; d += 32) wcnt[warp][d] = 0;
    __syncwarp();
    // warp w owns elements [base + w*256, base + (w+1)*256), walked in 8 rounds of 32
    const long long wbase = (long long)blockIdx.x * SORT_TILE + (long long)warp * (32 * SORT_ITEMS);
    int key[SORT_ITEMS], val[SORT_ITEMS], rnk[SORT_ITEMS];
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < SORT_ITEMS; r++) {
        const long long e = wbase + (long long)r * 32 + lane;
        const bool ok = e < n;
        key[r] = ok ? keys_in[e] : 0;
        val[r] = ok ? (vals_in ? vals_in[e] : (int)e) : 0;  // first pass: values are the indices
        const int d = ok ? ((key[r] >> shift) & 0xFF) : RADIX;  // sentinel digit for padding
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int before = __popc(peers & lt);
        int basecnt = 0;
        if (ok) basecnt = wcnt[warp][d];
        __syncwarp();
        rnk[r] = basecnt + before;
        if (ok && before == 0) wcnt[warp][d] = basecnt + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // exclusive prefix over warps for each digit; add the global (digit, block) offset
    for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) {
        int run = offsets[(long long)d * nblocks + blockIdx.x];
        for (int w = 0; w < SORT_WARPS; w++) {
            const int c = wcnt[w][d];
            wcnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
    for (int r = 0; r < SORT_ITEMS; r++) {
        const long long e = wbase + (long long)r * 32 + lane;
        if (e < n) {
            const int d = (key[r] >> shift) & 0xFF;
            const int pos = wcnt[warp][d] + rnk[r];
            keys_out[pos] = key[r];
            vals_out[pos] = val[r];
        }
    }
}

// ---- exclusive scan of int arrays (three-phase, recursive over block sums) ----

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile(const int *in, int *out, long long n, int *block_sums)
{
    pdl_prologue();
    __shared__ int wsum[SCAN_THREADS / 32];
    const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS], tsum = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        tsum += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = tsum;
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = (lane < SCAN_THREADS / 32) ? wsum[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        if (lane < SCAN_THREADS / 32) wsum[lane] = w;
    }
    __syncthreads();
    int run = incl - tsum + (warp > 0 ? wsum[warp - 1] : 0);
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == SCAN_THREADS - 1 && block_sums) block_sums[blockIdx.x] = wsum[SCAN_THREADS / 32 - 1];
}

__global__ void k_scan_add(int *out, long long n, const int *block_off)
{
    pdl_prologue();
    const long long i = (long long)blockIdx.x * SCAN_TILE + threadIdx.x;
    const int add = block_off[blockIdx.x];
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const long long e = i + (long long)k * SCAN_THREADS;
        if (e < n) out[e] += add;
    }
}

// the add pass when the tile sums fit one tile: each CTA sums the tile sums before its own
// (at most SCAN_TILE of them), so the scan of the sums needs no launch of its own
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_add_self(int *out, long long n, const int *block_sums)
{
    pdl_prologue();
    __shared__ int red[SCAN_THREADS / 32];
    if (blockIdx.x == 0) return;  // the first tile's prefix is zero
    int part = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += SCAN_THREADS) part += block_sums[b];
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = part;
    __syncthreads();
    int add = 0;
#pragma unroll
    for (int w = 0; w < SCAN_THREADS / 32; w++) add += red[w];
    const long long i = (long long)blockIdx.x * SCAN_TILE + threadIdx.x;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const long long e = i + (long long)k * SCAN_THREADS;
        if (e < n) out[e] += add;
    }
}

void exclusive_scan_int(const int *in, int *out, long long n, int *tmp, cudaStream_t s, cudaError_t *err)
{
    if (n <= 0) return;
    const long long nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb == 1) {
        keep_first(err, launch_pdl(k_scan_tile, 1, SCAN_THREADS, s, in, out, n, nullptr));
        note_launch(1);
        return;
    }
    int *sums = tmp, *sums_scan = tmp + nb + 16;
    keep_first(err, launch_pdl(k_scan_tile, (unsigned)nb, SCAN_THREADS, s, in, out, n, sums));
    note_launch(1);
    if (nb <= SCAN_TILE) {
        keep_first(err, launch_pdl(k_scan_add_self, (unsigned)nb, SCAN_THREADS, s, out, n, sums));
        note_launch(1);
        return;
    }
    exclusive_scan_int(sums, sums_scan, nb, tmp + 2 * nb + 32, s, err);
    keep_first(err, launch_pdl(k_scan_add, (unsigned)nb, SCAN_THREADS, s, out, n, sums_scan));
    note_launch(1);
}

// ---- sort driver ----
size_t sort_scratch_bytes(long long n)
{
    const long long nblocks = (n + SORT_TILE - 1) / SORT_TILE;
    return (size_t)(4 * n + 2 * RADIX * nblocks) * sizeof(int) + scan_tmp_ints(RADIX * nblocks) * sizeof(int);
}

// Sorts keys_in[0..n) (non-negative, < 2^key_bits) stably; perm_out[i] is the input index
// of the i-th element in sorted order.  Returns the device array holding the sorted keys.
const int *sort_pairs(const int *keys_in, int *perm_out, long long n, int key_bits, SortScratch &ws, cudaStream_t s,
                      cudaError_t *err)
{
    if (n <= 0) return keys_in;
    const int nblocks = (int)((n + SORT_TILE - 1) / SORT_TILE);
    int passes = (key_bits + 7) / 8;
    if (passes < 1) passes = 1;
    const int *kin = keys_in;
    const int *vin = nullptr;
    int cur = 0;
    for (int p = 0; p < passes; p++) {
        const int shift = 8 * p;
        int *kout = ws.keys[cur];
        int *vout = (p == passes - 1) ? perm_out : ws.vals[cur];
        keep_first(err, launch_pdl(k_radix_hist, nblocks, SORT_THREADS, s, kin, n, shift, ws.hist, nblocks));
        note_launch(1);
        exclusive_scan_int(ws.hist, ws.hist + (long long)RADIX * nblocks, (long long)RADIX * nblocks, ws.scan_tmp, s,
                           err);
        keep_first(err, launch_pdl(k_radix_scatter, nblocks, SORT_THREADS, s, kin, vin, kout, vout, n, shift,
                                   ws.hist + (long long)RADIX * nblocks, nblocks));
        note_launch(1);
        kin = kout;
        vin = vout;
        cur ^= 1;
    }
    return kin;
}

// Segments: starts of the runs of equal cell block in key order (the list is unordered).
// Each CTA walks a contiguous range in tiles of 4096 keys -- four 16-byte loads per thread,
// all issued first; a key's predecessor is the previous thread's last key -- and gathers its
// heads in shared memory; one global atomic per CTA flush reserves their places.
constexpr int BH_THREADS = 256;
constexpr int BH_TILE = 16 * BH_THREADS;
constexpr int BH_BUF = 2 * BH_TILE;

// nseg must be zero on entry.  The kernel also zeroes up to three counters of the caller
// (clear0..2, may be null) that nothing reads while it runs, and writes each head's position
// at its block's entry of blk_first (may be null).
__global__ void __launch_bounds__(BH_THREADS) k_block_heads(const int *skey, long long n, int *seg_start, int *nseg,
                                                            int *clear0, int *clear1, int *clear2, int *blk_first)
{
    pdl_prologue();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (clear0) *clear0 = 0;
        if (clear1) *clear1 = 0;
        if (clear2) *clear2 = 0;
    }
    __shared__ int buf[BH_BUF];
    __shared__ int bcount, bbase;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const long long tiles = (n + BH_TILE - 1) / BH_TILE;
    const long long t0 = tiles * blockIdx.x / gridDim.x, t1 = tiles * (blockIdx.x + 1) / gridDim.x;
    const int4 *k4 = reinterpret_cast<const int4 *>(skey);
    const bool vec = (reinterpret_cast<unsigned long long>(skey) & 15ull) == 0;  // 16-byte loads need it
    if (threadIdx.x == 0) bcount = 0;
    __syncthreads();
    for (long long t = t0; t < t1; t++) {
        // element e of vector u of this thread: index b0 + u * 4 * BH_THREADS + 4 * tid + e
        const long long b0 = t * BH_TILE;
        int4 kv[4];
        int kprev[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const long long i = b0 + (long long)u * 4 * BH_THREADS + 4 * threadIdx.x;
            if (vec && i + 3 < n) {
                kv[u] = k4[i >> 2];
            } else {
                kv[u].x = i < n ? skey[i] : 0;
                kv[u].y = i + 1 < n ? skey[i + 1] : 0;
                kv[u].z = i + 2 < n ? skey[i + 2] : 0;
                kv[u].w = i + 3 < n ? skey[i + 3] : 0;
            }
            kprev[u] = (lane == 0 && i > 0 && i <= n) ? skey[i - 1] : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const long long i = b0 + (long long)u * 4 * BH_THREADS + 4 * threadIdx.x;
            const int up = __shfl_up_sync(0xffffffffu, kv[u].w, 1);
            const int before = lane == 0 ? kprev[u] : up;
            const int e[4] = {kv[u].x, kv[u].y, kv[u].z, kv[u].w};
            int pk = before;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const long long ie = i + q;
                const bool head = ie < n && (ie == 0 || (e[q] >> CB_SHIFT) != (pk >> CB_SHIFT));
                pk = e[q];
                const unsigned mask = __ballot_sync(0xffffffffu, head);
                if (!mask) continue;
                int base = 0;
                if (lane == 0) base = atomicAdd(&bcount, __popc(mask));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (head) {
                    buf[base + __popc(mask & lt)] = (int)ie;
                    if (blk_first) blk_first[e[q] >> CB_SHIFT] = (int)ie;
                }
            }
        }
        __syncthreads();
        const int c = bcount;
        __syncthreads();  // every thread has read the count before the next tile adds to it
        if (c > BH_BUF - BH_TILE || (t == t1 - 1 && c > 0)) {
            if (threadIdx.x == 0) bbase = atomicAdd(nseg, c);
            __syncthreads();
            for (int q = threadIdx.x; q < c; q += BH_THREADS) seg_start[bbase + q] = buf[q];
            __syncthreads();
            if (threadIdx.x == 0) bcount = 0;
            __syncthreads();
        }
    }
}

void launch_block_heads(const int *skey, long long n, int *seg_start, int *nseg, cudaStream_t s, int *clear0,
                        int *clear1, int *clear2, int *blk_first)
{
    if (n > 0) {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const long long grid = std::min<long long>((n + BH_TILE - 1) / BH_TILE, (long long)sms * 4);
        launch_pdl(k_block_heads, (unsigned)grid, BH_THREADS, s, skey, n, seg_start, nseg, clear0, clear1, clear2,
                   blk_first);
        note_launch(1);
    } else {
        for (int *c : {clear0, clear1, clear2})
            if (c) cudaMemsetAsync(c, 0, sizeof(int), s);
    }
}

// ---- allocation-free sort (gy_sort_keys_static) ----
// The scratch of the radix sort -- two key and two index ping-pong buffers, the per-pass
// (digit, block) histograms and the scan workspace -- for up to GY_SORT_STATIC_MAX keys, in
// one file-scope device array.  Every GPU that loads this library holds it (1,118,208 ints:
// 4.47 MB, 4.27 MiB) until the process exits.
constexpr long long kStaticMax = GY_SORT_STATIC_MAX;
constexpr long long kStaticBlocks = (kStaticMax + SORT_TILE - 1) / SORT_TILE;
constexpr long long kStaticScanInts = 4096;
constexpr long long kStaticInts = 4 * kStaticMax + 2 * RADIX * kStaticBlocks + kStaticScanInts;
static_assert(scan_tmp_ints(RADIX * kStaticBlocks) <= (size_t)kStaticScanInts,
              "the scan workspace of the fixed scratch is too small for GY_SORT_STATIC_MAX keys");
static __device__ __align__(256) int g_sort_static[kStaticInts];

// Device address of g_sort_static per device ordinal, looked up once with that device current.
// The address belongs to the device's primary context: a cudaDeviceReset by the caller
// replaces that context and leaves the cached address stale.
static std::mutex g_static_mu;
static int *g_static_addr[256] = {};

static gy_status static_scratch(int **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return GY_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_sort_static) != cudaSuccess || !p) return GY_ERR_CUDA;
        g_static_addr[dev] = static_cast<int *>(p);
    }
    *out = g_static_addr[dev];
    return GY_OK;
}

}  // namespace gy

extern "C" gy_status gy_sort_keys_static(const int *d_keys, int64_t n, int key_bits, int *d_perm_out, void *stream)
{
    using namespace gy;
    if (n < 0 || n > kStaticMax) return GY_ERR_ARG;  // the fixed scratch holds GY_SORT_STATIC_MAX keys
    if (key_bits < 1 || key_bits > 31) return GY_ERR_ARG;
    if (n == 0) return GY_OK;
    if (!d_keys || !d_perm_out) return GY_ERR_ARG;
    int *base = nullptr;
    gy_status st = static_scratch(&base);
    if (st != GY_OK) return st;
    // carve the static array exactly as the allocating sort carves its buffer; every
    // region is fully rewritten by each pass, so nothing needs clearing between calls
    SortScratch ws{};
    int *p = base;
    ws.keys[0] = p; p += kStaticMax;
    ws.keys[1] = p; p += kStaticMax;
    ws.vals[0] = p; p += kStaticMax;
    ws.vals[1] = p; p += kStaticMax;
    ws.hist = p; p += 2 * RADIX * kStaticBlocks;
    ws.scan_tmp = p;
    ws.cap = kStaticMax;
    ws.nblocks_cap = (int)kStaticBlocks;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the status is this call's own launches' (errors left by earlier work of the caller
    // stay where they are); faults while the kernels run surface at the caller's next sync
    cudaError_t err = cudaSuccess;
    (void)sort_pairs(d_keys, d_perm_out, n, key_bits, ws, s, &err);
    return err == cudaSuccess ? GY_OK : GY_ERR_CUDA;
}
