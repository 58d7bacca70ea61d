// gy_resort.cu -- incremental stable re-sort of the particle cell keys.
//
// After a sorted step the slab holds the particles in the order of that sort, and only the
// particles that changed cell since ("movers") break it: the others ("stayers") still have
// the key stored at their slot in the previous sorted key array, which is non-decreasing, so
// they form a sorted run by (key, slot).  The stable order of the new keys is the merge of
// the stayers with the movers sorted by (key, slot):
//   * the movers, compacted in slot order, are sorted stably by key (a radix sort whose
//     length lives on the device, so the host never waits for it); mover q of that order
//     lands at q + g(q), g = the stayers below it -- one binary search on the previous keys;
//   * stayer r (r-th stayer in slot order) lands at r + (movers with g <= r).
// The result is the permutation the full stable radix sort produces, at a fraction of its
// traffic when few particles move; the full sort runs whenever the previous order is not
// known (first step, restored state).
#include <algorithm>

#include "gy_kernels.cuh"

namespace gy {

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;                          // per thread in the mover sort
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;       // 2048
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_RADIX = 256;
constexpr int RS_MAX_CTAS = 1024;                    // mover-sort CTAs (2 per SM)
constexpr int RS_MAX_PASSES = 4;                     // 8-bit digits of a non-negative int key

__device__ __forceinline__ long long movers_before(long long P, const unsigned *wmask, const int *wpref)
{
    const long long w = P >> 5;
    const int b = (int)(P & 31);
    return (long long)wpref[w] + (b ? __popc(wmask[w] & ((1u << b) - 1u)) : 0);
}

// CTA c of the mover sort owns [m c / G, m (c+1) / G); the owner of position pos is the
// largest c with floor(m c / G) <= pos
__device__ __forceinline__ int owner_cta(int pos, int m, int G)
{
    const int c = (int)(((long long)(pos + 1) * G - 1) / m);
    return c < G - 1 ? c : G - 1;
}

// mover mask and count per 32 slots: a warp takes four words at a time, all loads first.
// The kernel also clears the gap counters the previous re-sort left (its m movers are still
// listed in gap[] and wpref[nw]) and the digit histograms this re-sort accumulates.
__global__ void __launch_bounds__(RS_THREADS) k_rs_mask(const int *key, const int *prev, long long n, unsigned *wmask,
                                                          int *wcnt, long long nw, const int *gap, const int *wpref,
                                                          int *gapcnt, int *gwcnt, int *hist, int hist_ints)
{
    pdl_prologue();
    const int lane = threadIdx.x & 31;
    const long long wstride = ((long long)gridDim.x * blockDim.x) >> 5;
    {
        const int mprev = wpref[nw];
        const int t = blockIdx.x * blockDim.x + threadIdx.x, tstride = gridDim.x * blockDim.x;
        for (int q = t; q < mprev; q += tstride) {
            gapcnt[gap[q]] = 0;
            gwcnt[gap[q] >> 5] = 0;
        }
        for (int q = t; q < hist_ints; q += tstride) hist[q] = 0;
        if (t == 0) wcnt[nw] = 0;  // the scan's last entry, so that wpref[nw] is the mover count
    }
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

// movers (key, slot) in slot order.  A warp takes 32 words at once (one mask per lane) and
// visits only the words that hold movers.
__global__ void __launch_bounds__(RS_THREADS) k_rs_compact(const int *key, const unsigned *wmask, const int *wpref,
                                                             long long nw, int *bkey, int *bidx, int *hist0, int G)
{
    pdl_prologue();
    const int mtot = wpref[nw];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const long long wstride = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long w0 = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; w0 < nw; w0 += wstride * 32) {
        const long long wl = w0 + lane;
        const unsigned mk = wl < nw ? wmask[wl] : 0u;
        const int pref = mk ? wpref[wl] : 0;
        unsigned nz = __ballot_sync(0xffffffffu, mk != 0u);
        while (nz) {
            const int u = __ffs(nz) - 1;
            nz &= nz - 1u;
            const unsigned m = __shfl_sync(0xffffffffu, mk, u);
            const int base = __shfl_sync(0xffffffffu, pref, u);
            if ((m >> lane) & 1u) {
                const long long i = (w0 + u) * 32 + lane;
                const int pos = base + __popc(m & lt);
                const int k = key[i];
                bkey[pos] = k;
                bidx[pos] = (int)i;
                atomicAdd(&hist0[(k & 0xFF) * G + owner_cta(pos, mtot, G)], 1);  // first pass's digit counts
            }
        }
    }
}

// ---- stable LSD radix sort of the m movers, m read on the device ----------------------
// CTA c of the G owns the contiguous range [m c / G, m (c+1) / G) and walks it in tiles of
// RS_TILE; ranks inside a tile follow k_radix_scatter (warps in order, peers by
// __match_any_sync), and per-digit bases carry from tile to tile.

__device__ __forceinline__ void cta_range(int m, int &c0, int &c1)
{
    c0 = (int)((long long)m * blockIdx.x / gridDim.x);
    c1 = (int)((long long)m * (blockIdx.x + 1) / gridDim.x);
}

// hist_next (or null on the last pass) receives the next pass's digit counts per owner CTA of
// each output position, so no separate histogram launch is needed
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const int *keys_in, const int *vals_in, int *keys_out,
                                                             int *vals_out, const int *m_ptr, int shift,
                                                             const int *offsets, int *hist_next)
{
    pdl_prologue();
    __shared__ int wcnt[RS_WARPS][RS_RADIX];  // per-warp digit counts, then per-warp bases
    __shared__ int base[RS_RADIX];            // running per-digit base of this CTA
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (int d = threadIdx.x; d < RS_RADIX; d += RS_THREADS) base[d] = offsets[d * gridDim.x + blockIdx.x];
    int c0, c1;
    cta_range(*m_ptr, c0, c1);
    for (int t0 = c0; t0 < c1; t0 += RS_TILE) {
        for (int d = lane; d < RS_RADIX; d += 32) wcnt[warp][d] = 0;
        __syncthreads();  // the bases of the previous tile are final; the counters are clear
        const int wb = t0 + warp * (32 * RS_ITEMS);
        int key[RS_ITEMS], val[RS_ITEMS], rnk[RS_ITEMS];
        for (int r = 0; r < RS_ITEMS; r++) {
            const int e = wb + r * 32 + lane;
            const bool ok = e < c1;
            key[r] = ok ? keys_in[e] : 0;
            val[r] = ok ? vals_in[e] : 0;
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
        for (int d = threadIdx.x; d < RS_RADIX; d += RS_THREADS) {
            int run = base[d];
            for (int w = 0; w < RS_WARPS; w++) {
                const int c = wcnt[w][d];
                wcnt[w][d] = run;
                run += c;
            }
            base[d] = run;
        }
        __syncthreads();
        for (int r = 0; r < RS_ITEMS; r++) {
            const int e = wb + r * 32 + lane;
            if (e < c1) {
                const int d = (key[r] >> shift) & 0xFF;
                const int pos = wcnt[warp][d] + rnk[r];
                keys_out[pos] = key[r];
                vals_out[pos] = val[r];
                if (hist_next)
                    atomicAdd(&hist_next[((key[r] >> (shift + 8)) & 0xFF) * gridDim.x + owner_cta(pos, *m_ptr, gridDim.x)], 1);
            }
        }
        __syncthreads();  // wcnt is reused by the next tile
    }
}

// ---- placement ----------------------------------------------------------------------

// mover q of the sorted order: stayers below it (gap g), placed at q + g; gaps counted
__global__ void __launch_bounds__(RS_THREADS) k_rs_place_movers(const int *prev, long long n, const unsigned *wmask,
                                                                  const int *wpref, long long nw, const int *skey,
                                                                  const int *sidx, int *gap, int *gapcnt, int *gwcnt,
                                                                  int *skey_out, int *perm_out)
{
    pdl_prologue();
    const int m = wpref[nw];
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
        const int k = skey[q], i = sidx[q];
        // first slot s with (prev[s], s) >= (k, i): a mover's new key is usually near its
        // old one, so gallop out from its old slot i before bisecting (cache-near probes)
        long long lo, hi;
        if (prev[i] < k) {  // the answer lies above i
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
        const long long pos = (long long)q + g;
        skey_out[pos] = k;
        perm_out[pos] = i;
    }
}

// stayer r lands at r + (movers with gap <= r).  A warp takes 32 words at once: their masks,
// prefixes and gap-word data load one per lane; the keys load eight words ahead.  The stayer
// ranks of one word lie in at most two consecutive 32-gap words, whose counts the warp loads
// and prefix-sums only when they hold movers.
__global__ void __launch_bounds__(RS_THREADS) k_rs_place_stayers(const int *key, long long n, const unsigned *wmask,
                                                                   const int *wpref, long long nw, const int *gapcnt,
                                                                   const int *gwcnt, const int *gwpref, int *skey_out,
                                                                   int *perm_out)
{
    pdl_prologue();
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const long long wstride = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long w0 = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; w0 < nw; w0 += wstride * 32) {
        const long long wl = w0 + lane;
        const bool wv = wl < nw;
        const unsigned mk = wv ? wmask[wl] : 0u;
        const long long rb = wv ? wl * 32 - wpref[wl] : 0;  // rank of the word's first stayer
        const long long gwl = rb >> 5;
        const int gb = wv ? gwpref[gwl] : 0;
        const int gc = wv ? (gwcnt[gwl] | gwcnt[gwl + 1]) : 0;
        const int nwords = (int)min((long long)32, nw - w0);
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
                const long long rbase = __shfl_sync(0xffffffffu, rb, u);
                const long long gw0 = rbase >> 5;
                int c0 = 0, c1 = 0;
                if (__shfl_sync(0xffffffffu, gc, u)) {
                    c0 = gapcnt[gw0 * 32 + lane];
                    c1 = gapcnt[gw0 * 32 + 32 + lane];
#pragma unroll
                    for (int off = 1; off < 32; off <<= 1) {
                        const int y0 = __shfl_up_sync(0xffffffffu, c0, off), y1 = __shfl_up_sync(0xffffffffu, c1, off);
                        if (lane >= off) {
                            c0 += y0;
                            c1 += y1;
                        }
                    }
                }
                const int gbase = __shfl_sync(0xffffffffu, gb, u);
                const int tot0 = __shfl_sync(0xffffffffu, c0, 31);
                const long long i = (w0 + u) * 32 + lane;
                const bool stay = i < n && !((m >> lane) & 1u);
                const long long r = rbase + lane - __popc(m & lt);
                const int rr = (int)(r - gw0 * 32);  // 0..62 for a stayer
                const int in0 = __shfl_sync(0xffffffffu, c0, rr & 31), in1 = __shfl_sync(0xffffffffu, c1, rr & 31);
                if (stay) {
                    const long long pos = r + gbase + (rr < 32 ? in0 : tot0 + in1);
                    skey_out[pos] = kv[v];
                    perm_out[pos] = (int)i;
                }
            }
        }
    }
}

// ---- scratch and driver ---------------------------------------------------------------

size_t resort_scratch_ints(long long cap)
{
    const long long nw = (cap + 31) / 32;
    const long long ngw = (cap + 2 + 63) / 32 + 2;  // 32-gap words, one spare word past the end
    const long long hist = (long long)RS_RADIX * RS_MAX_CTAS;
    return (size_t)(3 * (nw + 1) + scan_tmp_ints(nw + 1) + 5 * cap + ngw * 32 + 2 * (ngw + 1) +
                    scan_tmp_ints(ngw + 1) + (RS_MAX_PASSES + 1) * hist + scan_tmp_ints(hist) + 64);
}

void resort_bind(ResortScratch &rs, int *mem, long long cap)
{
    const long long nw = (cap + 31) / 32;
    const long long ngw = (cap + 2 + 63) / 32 + 2;
    const long long hist = (long long)RS_RADIX * RS_MAX_CTAS;
    int *p = mem;
    rs.wmask = reinterpret_cast<unsigned *>(p); p += nw + 1;
    rs.wcnt = p; p += nw + 1;
    rs.wpref = p; p += nw + 1;
    rs.wscan_tmp = p; p += scan_tmp_ints(nw + 1);
    rs.bkey = p; p += cap;
    rs.bidx = p; p += cap;
    rs.tkey = p; p += cap;
    rs.tidx = p; p += cap;
    rs.gap = p; p += cap;
    rs.gapcnt = p; p += ngw * 32;
    rs.gwcnt = p; p += ngw + 1;
    rs.gwpref = p; p += ngw + 1;
    rs.gscan_tmp = p; p += scan_tmp_ints(ngw + 1);
    rs.hist = p; p += (RS_MAX_PASSES + 1) * hist;  // a digit histogram per pass, then the offsets
    rs.hscan_tmp = p;
    rs.cap = cap;
    rs.ngw = ngw;
}

// The scratch must be zero before the first call (it is zeroed once); each call clears the
// gap counters its predecessor left and the digit histograms it uses.
void resort_keys(const int *key, const int *prev_skey, int *skey_out, int *perm_out, long long n, int key_bits,
                 ResortScratch &rs, cudaStream_t s)
{
    if (n <= 0) return;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long nw = (n + 31) / 32;
    const unsigned wgrid = (unsigned)std::min<long long>((nw + 4 * RS_WARPS - 1) / (4 * RS_WARPS), (long long)sms * 16);
    const long long nw32 = (nw + 31) / 32;  // 32-word batches (compaction, stayer placement)
    const unsigned bgrid = (unsigned)std::max<long long>(1, std::min<long long>((nw32 + RS_WARPS - 1) / RS_WARPS, (long long)sms * 16));
    const unsigned qgrid = (unsigned)std::min<long long>((n + RS_THREADS - 1) / RS_THREADS, (long long)sms * 8);
    const int G = std::min(2 * sms, RS_MAX_CTAS);
    const int passes = std::min(RS_MAX_PASSES, std::max(1, (key_bits + 7) / 8));
    const int hg = RS_RADIX * G;                                    // one pass's histogram
    int *offsets = rs.hist + (long long)RS_MAX_PASSES * RS_RADIX * RS_MAX_CTAS;
    launch_pdl(k_rs_mask, wgrid, RS_THREADS, s, key, prev_skey, n, rs.wmask, rs.wcnt, nw, rs.gap, rs.wpref, rs.gapcnt,
                                           rs.gwcnt, rs.hist, passes * hg);
    exclusive_scan_int(rs.wcnt, rs.wpref, nw + 1, rs.wscan_tmp, s);
    // movers in slot order, with the first pass's digit counts per mover-sort CTA
    launch_pdl(k_rs_compact, bgrid, RS_THREADS, s, key, rs.wmask, rs.wpref, nw, rs.bkey, rs.bidx, rs.hist, G);
    note_launch(2);
    // stable sort of the movers by key; their count is wpref[nw]
    const int *m_ptr = rs.wpref + nw;
    int *kin = rs.bkey, *vin = rs.bidx, *kout = rs.tkey, *vout = rs.tidx;
    for (int p = 0; p < passes; p++) {
        exclusive_scan_int(rs.hist + (long long)p * hg, offsets, hg, rs.hscan_tmp, s);
        launch_pdl(k_rs_scatter, G, RS_THREADS, s, kin, vin, kout, vout, m_ptr, 8 * p, offsets,
                                              p + 1 < passes ? rs.hist + (long long)(p + 1) * hg : nullptr);
        note_launch(1);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    launch_pdl(k_rs_place_movers, qgrid, RS_THREADS, s, prev_skey, n, rs.wmask, rs.wpref, nw, kin, vin, rs.gap, rs.gapcnt,
                                                   rs.gwcnt, skey_out, perm_out);
    exclusive_scan_int(rs.gwcnt, rs.gwpref, rs.ngw + 1, rs.gscan_tmp, s);
    launch_pdl(k_rs_place_stayers, bgrid, RS_THREADS, s, key, n, rs.wmask, rs.wpref, nw, rs.gapcnt, rs.gwcnt, rs.gwpref,
                                                    skey_out, perm_out);
    note_launch(2);
}

}  // namespace gy
