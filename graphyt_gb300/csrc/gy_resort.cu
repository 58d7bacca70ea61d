// gy_resort.cu -- incremental stable re-sort of the particle cell keys.
//
// After a sorted step the slab holds the particles in the order of that sort, and only the
// particles that changed cell since ("movers") break it: the others ("stayers") still have
// the key stored at their slot in the previous sorted key array, which is non-decreasing, so
// they form a sorted run by (key, slot).  The stable order of the new keys is the merge of
// the stayers with the movers ordered by (key, slot):
//   * mover (k, i) has a gap g = the stayers below it in (key, slot) order, one search of the
//     previous keys, and lands at g + (movers before it in (key, slot) order).  The movers
//     before it are those of lower key buckets (a bucket is a range of 2^shift keys, a 4x4x4
//     cell block on grids of up to 2^24 cells), counted per bucket and prefix-summed, plus
//     those of its own bucket that precede it, counted over the bucket's few movers;
//   * stayer r (r-th stayer in slot order) lands at r + (movers with g <= r).
// A bucket holding more than RS_BUCKET_MAX movers (a flow far outside the time-step limit,
// or keys that are not cells) sends all movers through a one-CTA stable radix sort instead.
// In the step the movers come flagged: G2P sets a bit per slot whose key it changes (with a
// count per 32 slots), and the stayer placement, their last reader, clears the bits.  The
// result is the permutation the full stable radix sort produces, at a fraction of its traffic
// when few particles move; the full sort runs whenever the previous order is not known
// (initialisation, restored state).
#include <algorithm>
#include <cstdint>

#include "gy_kernels.cuh"

namespace gy {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_RADIX = 256;
constexpr int RS_BUCKET_BITS = 18;     // at most 2^18 key buckets
constexpr int RS_BUCKET_MAX = 512;     // movers per bucket ranked by counting
constexpr int RB_THREADS = 1024;       // the one-CTA fallback sort
constexpr int RB_ITEMS = 8;
constexpr int RB_TILE = RB_THREADS * RB_ITEMS;
constexpr int RB_WARPS = RB_THREADS / 32;

__device__ __forceinline__ long long movers_before(long long P, const unsigned *wmask, const int *wpref)
{
    const long long w = P >> 5;
    const int b = (int)(P & 31);
    return (long long)wpref[w] + (b ? __popc(wmask[w] & ((1u << b) - 1u)) : 0);
}

// mover mask and count per 32 slots from the two key arrays, for callers whose particle
// update did not flag the movers: a warp takes four words at a time, all loads first
__global__ void __launch_bounds__(RS_THREADS) k_rs_mask(const int *key, const int *prev, long long n, unsigned *wmask,
                                                          int *wcnt, long long nw)
{
    pdl_prologue();
    const int lane = threadIdx.x & 31;
    const long long wstride = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long w0 = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 4; w0 < nw; w0 += wstride * 4) {
        int ka[4], kb[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const long long i = (w0 + u) * 32 + lane;
            ka[u] = i < n ? key[i] : 0;
            kb[u] = i < n ? prev[i] : 0;
        }
        unsigned mine = 0u;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const unsigned m = __ballot_sync(0xffffffffu, ka[u] != kb[u]);
            if (lane == u) mine = m;
        }
        if (lane < 4 && w0 + lane < nw) {
            wmask[w0 + lane] = mine;
            wcnt[w0 + lane] = __popc(mine);
        }
    }
}

// the movers' slots in slot order.  A warp takes 32 words at once (one mask per lane) and
// visits only the words that hold movers.  The kernel also clears the gap counters the
// previous re-sort left (its *mlast movers are still listed in gap[]), this re-sort's bucket
// counters and the fallback flag.
__global__ void __launch_bounds__(RS_THREADS) k_rs_compact(const unsigned *wmask, const int *wpref, long long nw,
                                                             int *bidx, const int *gap, const int *mlast, int *gapcnt,
                                                             int *gwcnt, int *bcnt, int nbk, int *big)
{
    pdl_prologue();
    {
        const int mprev = *mlast;
        const int t = blockIdx.x * blockDim.x + threadIdx.x, tstride = gridDim.x * blockDim.x;
        for (int q = t; q < mprev; q += tstride) {
            gapcnt[gap[q]] = 0;
            gwcnt[gap[q] >> 5] = 0;
        }
        for (int q = t; q < nbk; q += tstride) bcnt[q] = 0;
        if (t == 0) *big = 0;
    }
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    // warp w takes the words [nw w / W, nw (w+1) / W), 32 at a time
    const long long W = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long wend = nw * (wid + 1) / W;
    for (long long w0 = nw * wid / W; w0 < wend; w0 += 32) {
        const long long wl = w0 + lane;
        const unsigned mk = wl < wend ? wmask[wl] : 0u;
        const int pref = mk ? wpref[wl] : 0;
        unsigned nz = __ballot_sync(0xffffffffu, mk != 0u);
        while (nz) {
            const int u = __ffs(nz) - 1;
            nz &= nz - 1u;
            const unsigned m = __shfl_sync(0xffffffffu, mk, u);
            const int base = __shfl_sync(0xffffffffu, pref, u);
            if ((m >> lane) & 1u) bidx[base + __popc(m & lt)] = (int)((w0 + u) * 32 + lane);
        }
    }
}

// mover q (slot order): its key, its gap g -- the stayers below it in (key, slot) order --
// counted per gap and per 32-gap word, and its arrival order within its key bucket.  blk_first (may be null)
// holds the first position of each cell block in the order of prev, as the segment heads of
// that sort wrote it; an entry is used only where prev confirms it.
__global__ void __launch_bounds__(RS_THREADS) k_rs_gaps(const int *key, const int *prev, long long n,
                                                          const unsigned *wmask, const int *wpref, long long nw,
                                                          const int *bidx, int shift, const int *blk_first, int *bkey,
                                                          int *gap, int *gapcnt, int *gwcnt, int *bcnt, int *bslot)
{
    pdl_prologue();
    const int m = wpref[nw];
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
        const int i = bidx[q], k = key[i];
        bkey[q] = k;
        // first slot s with (prev[s], s) >= (k, i).  From the head p of k's cell block in
        // prev, every slot below p holds a smaller key: gallop up from p.  Otherwise (the
        // block was empty) a mover's new key is usually near its old one: gallop out from its
        // old slot i.  Then bisect.
        int p = -1;
        if (blk_first) {
            const int b = k >> CB_SHIFT;
            const int c = blk_first[b];
            if (c >= 0 && c < n && (prev[c] >> CB_SHIFT) == b && (c == 0 || (prev[c - 1] >> CB_SHIFT) != b)) p = c;
        }
        long long lo, hi;
        if (p >= 0) {
            long long step = 1;
            lo = p;
            hi = p;
            while (hi < n && (prev[hi] < k || (prev[hi] == k && hi < i))) {
                lo = hi + 1;
                hi = p + step;
                step <<= 1;
            }
            if (hi > n) hi = n;
        } else if (prev[i] < k) {  // the answer lies above i
            long long step = 1;
            lo = i + 1;
            hi = i + 1;
            while (hi < n && prev[hi] <= k && (prev[hi] < k || hi < i)) {
                lo = hi + 1;
                hi = i + 1 + step;
                step <<= 1;
            }
            if (hi > n) hi = n;
        } else {  // prev[i] >= k: the answer is at or below i
            long long step = 1;
            hi = i;
            lo = i;
            while (lo > 0 && (prev[lo - 1] > k || (prev[lo - 1] == k && lo - 1 >= i))) {
                hi = lo - 1;
                lo = (i - step > 0) ? i - step : 0;
                step <<= 1;
            }
        }
        while (lo < hi) {
            const long long mid = (lo + hi) >> 1;
            const int pk = prev[mid];
            if (pk > k || (pk == k && mid >= i)) hi = mid;
            else lo = mid + 1;
        }
        const int g = (int)(lo - movers_before(lo, wmask, wpref));
        gap[q] = g;
        atomicAdd(&gapcnt[g], 1);
        atomicAdd(&gwcnt[g >> 5], 1);
        bslot[q] = atomicAdd(&bcnt[k >> shift], 1);
    }
}

// a mover as one word ordered like (key, slot): both are non-negative ints
__device__ __forceinline__ unsigned long long key_slot(int k, int i)
{
    return ((unsigned long long)(unsigned)k << 32) | (unsigned)i;
}

// the movers grouped by key bucket, in arrival order inside a bucket: bucket b's occupy
// [bpref[b] - m, bpref[b] - m + bcnt[b]) of the staging array (bpref is the bucket part of a
// scan that starts with the m gap-word counts)
__global__ void __launch_bounds__(RS_THREADS) k_rs_stage(const int *wpref, long long nw, const int *bkey,
                                                           const int *bidx, const int *bslot, const int *bpref,
                                                           int shift, unsigned long long *stage)
{
    pdl_prologue();
    const int m = wpref[nw];
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
        const int k = bkey[q];
        stage[bpref[k >> shift] - m + bslot[q]] = key_slot(k, bidx[q]);
    }
}

// mover q lands at g + (movers of lower buckets) + (movers of its bucket before it in (key,
// slot) order), the last counted over the bucket's staged movers, eight independent loads at
// a time (a bucket can hold a few hundred movers when a layer of particles crosses a cell
// boundary at once).  A bucket of more than RS_BUCKET_MAX movers raises *big, and k_rs_big
// places every mover instead.
__global__ void __launch_bounds__(RS_THREADS) k_rs_rank(const int *wpref, long long nw, const int *bkey,
                                                          const int *bidx, const int *gap, const int *bcnt,
                                                          const int *bpref, int shift,
                                                          const unsigned long long *stage, int *big, int *skey_out,
                                                          int *perm_out)
{
    pdl_prologue();
    const int m = wpref[nw];
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
        const int k = bkey[q], i = bidx[q], b = k >> shift;
        const int c = bcnt[b];
        if (c > RS_BUCKET_MAX) {
            *big = 1;
            continue;
        }
        const unsigned long long me = key_slot(k, i);
        const int j0 = bpref[b] - m, j1 = j0 + c;
        int r = 0, j = j0;
        for (; j + 8 <= j1; j += 8) {
            unsigned long long v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) v[u] = __ldg(&stage[j + u]);
#pragma unroll
            for (int u = 0; u < 8; u++) r += v[u] < me ? 1 : 0;
        }
        for (; j < j1; j++) r += __ldg(&stage[j]) < me ? 1 : 0;
        const long long pos = (long long)gap[q] + j0 + r;
        skey_out[pos] = k;
        perm_out[pos] = i;
    }
}

// Fallback for crowded buckets: one CTA sorts all m movers stably by key (LSD, 8-bit digits;
// tiles in slot order, ranks inside a tile by warps in order and peers by __match_any_sync,
// per-digit bases carried from tile to tile) and places every one of them at g + its index.
// Movers k_rs_rank placed already get the same position and value again.
__global__ void __launch_bounds__(RB_THREADS) k_rs_big(const int *big, const int *wpref, long long nw,
                                                         const int *bkey, const int *bidx, const int *gap, int passes,
                                                         int *ka, int *va, int *kb, int *vb, int *skey_out,
                                                         int *perm_out)
{
    pdl_prologue();
    if (!*big) return;
    __shared__ int wcnt[RB_WARPS][RS_RADIX];  // per-warp digit counts, then per-warp bases
    __shared__ int base[RS_RADIX];            // running per-digit base
    const int m = wpref[nw];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int *kin = bkey, *vin = nullptr;  // pass 0's value is the slot-order index itself
    int *kout = ka, *vout = va;
    for (int p = 0; p < passes; p++) {
        const int shift = 8 * p;
        for (int d = threadIdx.x; d < RS_RADIX; d += RB_THREADS) base[d] = 0;
        __syncthreads();
        for (int e = threadIdx.x; e < m; e += RB_THREADS) atomicAdd(&base[(kin[e] >> shift) & 0xFF], 1);
        __syncthreads();
        if (warp == 0) {  // exclusive scan of the 256 digit counts, eight per lane
            int v[RS_RADIX / 32], sum = 0;
#pragma unroll
            for (int u = 0; u < RS_RADIX / 32; u++) {
                v[u] = base[lane * (RS_RADIX / 32) + u];
                sum += v[u];
            }
            int inc = sum;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, inc, off);
                if (lane >= off) inc += y;
            }
            int run = inc - sum;
#pragma unroll
            for (int u = 0; u < RS_RADIX / 32; u++) {
                base[lane * (RS_RADIX / 32) + u] = run;
                run += v[u];
            }
        }
        __syncthreads();
        for (int t0 = 0; t0 < m; t0 += RB_TILE) {
            for (int d = lane; d < RS_RADIX; d += 32) wcnt[warp][d] = 0;
            __syncthreads();  // the bases of the previous tile are final; the counters are clear
            const int wb = t0 + warp * (32 * RB_ITEMS);
            int key[RB_ITEMS], val[RB_ITEMS], rnk[RB_ITEMS];
            for (int r = 0; r < RB_ITEMS; r++) {
                const int e = wb + r * 32 + lane;
                const bool ok = e < m;
                key[r] = ok ? kin[e] : 0;
                val[r] = ok ? (vin ? vin[e] : e) : 0;
                const int d = ok ? ((key[r] >> shift) & 0xFF) : RS_RADIX;
                const unsigned peers = __match_any_sync(0xffffffffu, d);
                const int before = __popc(peers & lt);
                int bc = 0;
                if (ok) bc = wcnt[warp][d];
                __syncwarp();
                rnk[r] = bc + before;
                if (ok && before == 0) wcnt[warp][d] = bc + __popc(peers);
                __syncwarp();
            }
            __syncthreads();
            for (int d = threadIdx.x; d < RS_RADIX; d += RB_THREADS) {
                int run = base[d];
                for (int w = 0; w < RB_WARPS; w++) {
                    const int c = wcnt[w][d];
                    wcnt[w][d] = run;
                    run += c;
                }
                base[d] = run;
            }
            __syncthreads();
            for (int r = 0; r < RB_ITEMS; r++) {
                const int e = wb + r * 32 + lane;
                if (e < m) {
                    const int pos = wcnt[warp][(key[r] >> shift) & 0xFF] + rnk[r];
                    kout[pos] = key[r];
                    vout[pos] = val[r];
                }
            }
            __syncthreads();  // wcnt is reused by the next tile; this pass's output is complete
        }
        kin = kout;
        vin = vout;
        kout = (kout == ka) ? kb : ka;
        vout = (vout == va) ? vb : va;
    }
    for (int j = threadIdx.x; j < m; j += RB_THREADS) {
        const int q = vin[j];
        const long long pos = (long long)gap[q] + j;
        skey_out[pos] = kin[j];
        perm_out[pos] = bidx[q];
    }
}

// ---- placement ----------------------------------------------------------------------

// stayer r lands at r + (movers with gap <= r).  A warp takes 32 words at once: their masks,
// prefixes and gap-word data load one per lane; the keys load eight words ahead.  The stayer
// ranks of one word lie in at most two consecutive 32-gap words, whose counts the warp loads
// and prefix-sums only when they hold movers.  The kernel is the last reader of the mover
// words, so it clears them for the particle update that flags the next movers, and it records
// the mover count for the next re-sort's clearing.
__global__ void __launch_bounds__(RS_THREADS) k_rs_place_stayers(const int *key, long long n, unsigned *wmask,
                                                                   int *wcnt, const int *wpref, long long nw,
                                                                   const int *gapcnt, const int *gwcnt,
                                                                   const int *gwpref, int *skey_out, int *perm_out,
                                                                   int *mlast)
{
    pdl_prologue();
    if (blockIdx.x == 0 && threadIdx.x == 0) *mlast = wpref[nw];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    // warp w takes the words [nw w / W, nw (w+1) / W), 32 at a time
    const long long W = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long wend = nw * (wid + 1) / W;
    for (long long w0 = nw * wid / W; w0 < wend; w0 += 32) {
        const long long wl = w0 + lane;
        const bool wv = wl < wend;
        const unsigned mk = wv ? wmask[wl] : 0u;
        if (wv && mk) {  // the last read of the word: clear it for the next step's movers
            wmask[wl] = 0u;
            wcnt[wl] = 0;
        }
        const int rb = wv ? (int)(wl * 32 - wpref[wl]) : 0;  // rank of the word's first stayer (n < 2^31)
        const int gwl = rb >> 5;
        const int gb = wv ? gwpref[gwl] : 0;
        const int gc = wv ? (gwcnt[gwl] | gwcnt[gwl + 1]) : 0;
        const int nwords = (int)min((long long)32, wend - w0);
        for (int u0 = 0; u0 < nwords; u0 += 8) {
            int kv[8];
#pragma unroll
            for (int v = 0; v < 8; v++) {
                const long long i = (w0 + u0 + v) * 32 + lane;
                kv[v] = (u0 + v < nwords && i < n) ? key[i] : 0;
            }
#pragma unroll
            for (int v = 0; v < 8; v++) {
                const int u = u0 + v;
                if (u >= nwords) break;  // warp-uniform
                const unsigned m = __shfl_sync(0xffffffffu, mk, u);
                const int rbase = __shfl_sync(0xffffffffu, rb, u);
                const int gbase = __shfl_sync(0xffffffffu, gb, u);
                const long long i = (w0 + u) * 32 + lane;
                const bool stay = i < n && !((m >> lane) & 1u);
                const int r = rbase + lane - __popc(m & lt);
                int add = 0;
                if (__shfl_sync(0xffffffffu, gc, u)) {
                    // movers in the gaps of the word's stayer ranks, which lie in two 32-gap
                    // words: their counts prefix-summed across the lanes
                    const int gw0 = rbase >> 5;
                    int c0 = gapcnt[gw0 * 32 + lane], c1 = gapcnt[gw0 * 32 + 32 + lane];
#pragma unroll
                    for (int off = 1; off < 32; off <<= 1) {
                        const int y0 = __shfl_up_sync(0xffffffffu, c0, off), y1 = __shfl_up_sync(0xffffffffu, c1, off);
                        if (lane >= off) {
                            c0 += y0;
                            c1 += y1;
                        }
                    }
                    const int tot0 = __shfl_sync(0xffffffffu, c0, 31);
                    const int rr = r - gw0 * 32;  // 0..62 for a stayer
                    const int in0 = __shfl_sync(0xffffffffu, c0, rr & 31), in1 = __shfl_sync(0xffffffffu, c1, rr & 31);
                    add = rr < 32 ? in0 : tot0 + in1;
                }
                if (stay) {
                    const long long pos = (long long)r + gbase + add;
                    skey_out[pos] = kv[v];
                    perm_out[pos] = (int)i;
                }
            }
        }
    }
}

// ---- scratch and driver ---------------------------------------------------------------

constexpr long long RS_NBK = 1LL << RS_BUCKET_BITS;

size_t resort_scratch_ints(long long cap)
{
    const long long nw = (cap + 31) / 32;
    const long long ngw = (cap + 2 + 63) / 32 + 2;  // 32-gap words, one spare word past the end
    // + 64: the fallback flag, the last mover count and the 8-byte alignment of the staging
    return (size_t)(3 * (nw + 1) + scan_tmp_ints(nw + 1) + 7 * cap + ngw * 32 + 2 * (ngw + 1 + RS_NBK) +
                    scan_tmp_ints(ngw + 1 + RS_NBK) + 64);
}

void resort_bind(ResortScratch &rs, int *mem, long long cap)
{
    const long long nw = (cap + 31) / 32;
    const long long ngw = (cap + 2 + 63) / 32 + 2;
    int *p = mem;
    rs.wmask = reinterpret_cast<unsigned *>(p); p += nw + 1;
    rs.wcnt = p; p += nw + 1;
    rs.wpref = p; p += nw + 1;
    rs.wscan_tmp = p; p += scan_tmp_ints(nw + 1);
    rs.bkey = p; p += cap;
    rs.bidx = p; p += cap;
    rs.gap = p; p += cap;
    rs.bslot = p; p += cap;
    p = reinterpret_cast<int *>((reinterpret_cast<uintptr_t>(p) + 7) & ~(uintptr_t)7);  // 8-byte words next
    rs.stage = reinterpret_cast<unsigned long long *>(p); p += 2 * cap;
    rs.tval = p; p += cap;
    rs.gapcnt = p; p += ngw * 32;
    rs.gwcnt = p; p += ngw + 1 + RS_NBK;  // the gap-word counts, then the bucket counts: one scan
    rs.gwpref = p; p += ngw + 1 + RS_NBK;
    rs.gscan_tmp = p; p += scan_tmp_ints(ngw + 1 + RS_NBK);
    rs.big = p;
    rs.mlast = p + 1;
    rs.cap = cap;
    rs.ngw = ngw;
}

// The scratch must be zero before the first call (it is zeroed once); each call clears the
// gap counters its predecessor left and the bucket counters it uses.  mask_ready: the mover
// words (wmask, wcnt) already flag every slot whose key differs from prev_skey -- the particle
// update sets them, and flagging more slots than that is harmless -- so the two key arrays are
// not compared here; otherwise k_rs_mask builds them.
void resort_keys(const int *key, const int *prev_skey, int *skey_out, int *perm_out, long long n, int key_bits,
                 ResortScratch &rs, cudaStream_t s, bool mask_ready, const int *blk_first)
{
    if (n <= 0) return;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long nw = (n + 31) / 32;
    const unsigned wgrid = (unsigned)std::min<long long>((nw + 4 * RS_WARPS - 1) / (4 * RS_WARPS), (long long)sms * 16);
    // compaction and stayer placement: one resident wave of CTAs, the words split evenly over
    // their warps (at least 32 words a warp).  The resident CTAs per SM depend only on the
    // kernels, built for one architecture, so they are looked up once per process.
    static int occ_c = 0, occ_s = 0;
    if (!occ_c) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_c, k_rs_compact, RS_THREADS, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, k_rs_place_stayers, RS_THREADS, 0);
        occ_c = std::max(occ_c, 1);
        occ_s = std::max(occ_s, 1);
    }
    const long long nw32 = (nw + 31) / 32;
    const long long cmax = (nw32 + RS_WARPS - 1) / RS_WARPS;
    const unsigned cgrid = (unsigned)std::max<long long>(1, std::min<long long>(cmax, (long long)sms * occ_c));
    const unsigned sgrid = (unsigned)std::max<long long>(1, std::min<long long>(cmax, (long long)sms * occ_s));
    const unsigned qgrid = (unsigned)std::min<long long>((n + RS_THREADS - 1) / RS_THREADS, (long long)sms * 4);
    const int bits = std::max(1, key_bits);
    const int shift = std::max(0, bits - RS_BUCKET_BITS);
    const int nbk = 1 << (bits - shift);
    const int passes = std::max(1, std::min(4, (bits + 7) / 8));
    int *bcnt = rs.gwcnt + rs.ngw + 1;
    const int *bpref = rs.gwpref + rs.ngw + 1;
    if (!mask_ready) {
        launch_pdl(k_rs_mask, wgrid, RS_THREADS, s, key, prev_skey, n, rs.wmask, rs.wcnt, nw);
        note_launch(1);
    }
    exclusive_scan_int(rs.wcnt, rs.wpref, nw + 1, rs.wscan_tmp, s);
    // movers in slot order (their count is wpref[nw]), their gaps and bucket counts
    launch_pdl(k_rs_compact, cgrid, RS_THREADS, s, rs.wmask, rs.wpref, nw, rs.bidx, rs.gap, rs.mlast, rs.gapcnt,
                                              rs.gwcnt, bcnt, nbk, rs.big);
    launch_pdl(k_rs_gaps, qgrid, RS_THREADS, s, key, prev_skey, n, rs.wmask, rs.wpref, nw, rs.bidx, shift, blk_first,
                                           rs.bkey, rs.gap, rs.gapcnt, rs.gwcnt, bcnt, rs.bslot);
    note_launch(2);
    // gap-word prefixes for the stayers, bucket bases for the movers
    exclusive_scan_int(rs.gwcnt, rs.gwpref, rs.ngw + 1 + nbk, rs.gscan_tmp, s);
    launch_pdl(k_rs_stage, qgrid, RS_THREADS, s, rs.wpref, nw, rs.bkey, rs.bidx, rs.bslot, bpref, shift, rs.stage);
    launch_pdl(k_rs_rank, qgrid, RS_THREADS, s, rs.wpref, nw, rs.bkey, rs.bidx, rs.gap, bcnt, bpref, shift, rs.stage,
                                           rs.big, skey_out, perm_out);
    // the fallback's two key/value buffers: the staging words' ints, and the slot of each
    // mover in the bucket (not needed after the staging) with tval
    int *st_ints = reinterpret_cast<int *>(rs.stage);
    launch_pdl(k_rs_big, 1, RB_THREADS, s, rs.big, rs.wpref, nw, rs.bkey, rs.bidx, rs.gap, passes, st_ints,
                                          st_ints + rs.cap, rs.bslot, rs.tval, skey_out, perm_out);
    launch_pdl(k_rs_place_stayers, sgrid, RS_THREADS, s, key, n, rs.wmask, rs.wcnt, rs.wpref, nw, rs.gapcnt, rs.gwcnt,
                                                    rs.gwpref, skey_out, perm_out, rs.mlast);
    note_launch(4);
}

}  // namespace gy
