// Visible-slot compaction, depth order, key duplication and tile ranges.
//
// The reference rasterizer (published 3DGS method) sorts one 64-bit key per
// (tile, Gaussian) pair, (tile << 32 | depth bits), with a stable radix sort, so ties keep
// the duplication order.  The same order is produced here with far less traffic:
//   1. k_compact: the visible (view, Gaussian) slots, in slot order, with their depth bits
//      (block-local scans of the per-(view, block) visible counts written by preprocess);
//   2. a stable onesweep sort of those N_vis slots by depth (32-bit keys, 4 passes);
//   3. k_sorted_sums + scan: tiles touched per block of depth-sorted slots -> key offsets;
//   4. k_duplicate: in depth order, one (tile id, slot) pair per tile of the slot's rect
//      (row-major), 32-bit keys;
//   5. a stable onesweep sort of the pairs by tile id alone (tile bits only: 2 passes for
//      up to 65536 tiles).
// Within a tile the result is in depth order with ties in slot order - exactly the order
// of the full (tile | depth) key sort - but the large array is sorted on 32-bit keys over
// 2 passes instead of 64-bit keys over 6.
// k_ranges: [start, end) of every global tile in the sorted pairs.
//
// The batched tracker replaces steps 4-5 by binning through 4x4-tile super-tiles:
// k_duplicate_coarse writes one (super-tile, slot) pair per super-tile of the slot's rect
// (4.6x fewer pairs), a stable sort by super-tile keeps each group in depth order, and
// k_filter_tiles cuts every tile's list out of its super-tile's group, in order.  The
// per-tile lists equal those of steps 4-5 (gs_launch_bin_coarse).
// With at most 256 super-tiles (the layout's super_tiles) the super-tile sort is a single
// pass whose first block also writes the super-tile ranges (no range kernel).  When the
// depth sort runs as one cooperative launch (sort.cu), that launch also produces the
// super-tile lists and ranges (steps 3-5 of the coarse path in the same grid), and only
// the filter follows.
#include "common.cuh"

template <typename KT>
int gs_launch_sort_t(KT *const keys[2], uint32_t *const vals[2], const uint32_t *count, uint32_t capacity,
                     int bits, uint32_t max_keys, int kpt, const Workspace &ws, int *out_buf, cudaStream_t s,
                     uint2 *ranges, uint32_t nranges);

namespace {

// exclusive scan of n block sums (one block of 1024 threads; shuffle scans within warps
// and over the warp totals); total into *total and an overflow flag when the total exceeds
// `capacity` (0: no check)
__device__ void scan_blocks(const uint32_t *sums, uint32_t *offs, int n, uint32_t *total, uint32_t *status,
                            uint32_t capacity, unsigned long long *part);
__global__ void __launch_bounds__(1024) k_scan_blocks(const uint32_t *sums, uint32_t *offs, int n, uint32_t *total,
                                                      uint32_t *status, uint32_t capacity)
{
    __shared__ unsigned long long part[1024];
    scan_blocks(sums, offs, n, total, status, capacity, part);
}

// Two independent scans in one launch (the fine and the coarse pair counts); also
// resets the fine-list region cursor (status[7]) of the filter that follows.
__global__ void __launch_bounds__(1024) k_scan_blocks2(const uint32_t *sums, uint32_t *offs, uint32_t *total,
                                                       const uint32_t *sums2, uint32_t *offs2, uint32_t *total2,
                                                       int n, uint32_t *status, uint32_t capacity)
{
    __shared__ unsigned long long part[1024];
    if (threadIdx.x == 0) status[7] = 0u;
    scan_blocks(sums, offs, n, total, status, capacity, part);
    __syncthreads();
    scan_blocks(sums2, offs2, n, total2, status, capacity, part);
}

__device__ void scan_blocks(const uint32_t *sums, uint32_t *offs, int n, uint32_t *total, uint32_t *status,
                            uint32_t capacity, unsigned long long *part)
{
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int per = (n + 1023) / 1024;
    const int b = t * per, e = min(n, b + per);
    unsigned long long s = 0;
    for (int i = b; i < e; ++i) s += sums[i];
    // warp-shuffle scan of the 1024 thread sums (64-bit), then of the 32 warp totals
    unsigned long long inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) part[w] = inc;
    __syncthreads();
    if (w == 0) {
        const unsigned long long v = part[lane];
        unsigned long long wi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        part[lane] = wi - v;
        if (lane == 31) part[32] = wi;
    }
    __syncthreads();
    unsigned long long run = part[w] + inc - s;
    for (int i = b; i < e; ++i) {
        offs[i] = (uint32_t)min(run, 0xffffffffull);
        run += sums[i];
    }
    if (t == 0) {
        const unsigned long long tot = part[32];
        *total = (uint32_t)min(tot, 0xffffffffull);
        if (capacity && tot > capacity) atomicOr(&status[0], GSEVT_STATUS_KEY_OVERFLOW);
    }
}

// ---- multi-block exclusive scan (for more block sums than one block scans quickly) ----
// Three launches: 4096-element chunk sums, a one-block scan of the chunk sums (with the
// total and the overflow check), and the per-chunk rescan that writes the offsets.  The
// 64-bit chunk sums live in a scratch region (the sort-count table, free between sorts).
#define SCAN_CHUNK 4096
#define SCAN_SMALL 8192  // up to this many sums the one-block scan is used

__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v, unsigned long long *wsum)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) wsum[w] = v;
    __syncthreads();
    unsigned long long t = 0;
    if (w == 0) {
        t = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;  // valid in warp 0
}

__global__ void __launch_bounds__(1024) k_scan_part(const uint32_t *sums, int n, unsigned long long *part)
{
    __shared__ unsigned long long wsum[32];
    const int base = blockIdx.x * SCAN_CHUNK + 4 * (int)threadIdx.x;
    unsigned long long s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (base + k < n) s += sums[base + k];
    const unsigned long long t = block_sum_u64(s, wsum);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// exclusive scan of the chunk sums in place (one block), total and overflow flag; also
// clears status[7] when asked (the filter's region cursor)
__global__ void __launch_bounds__(1024) k_scan_top(unsigned long long *part, int nparts, uint32_t *total,
                                                   uint32_t *status, uint32_t capacity, int clear_cursor)
{
    __shared__ unsigned long long wsc[32];
    __shared__ unsigned long long carry;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (t == 0) carry = 0;
    if (t == 0 && clear_cursor) status[7] = 0u;
    __syncthreads();
    for (int b0 = 0; b0 < nparts; b0 += 1024) {
        const unsigned long long v = b0 + t < nparts ? part[b0 + t] : 0ull;
        unsigned long long inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsc[w] = inc;
        __syncthreads();
        unsigned long long wb = 0;
        for (int i = 0; i < w; ++i) wb += wsc[i];
        const unsigned long long c = carry;
        if (b0 + t < nparts) part[b0 + t] = c + wb + inc - v;
        __syncthreads();
        if (t == 1023) carry = c + wb + inc;
        __syncthreads();
    }
    if (t == 0) {
        const unsigned long long tot = carry;
        *total = (uint32_t)min(tot, 0xffffffffull);
        if (capacity && tot > capacity) atomicOr(&status[0], GSEVT_STATUS_KEY_OVERFLOW);
    }
}

__global__ void __launch_bounds__(1024) k_scan_final(const uint32_t *sums, int n, const unsigned long long *part,
                                                     uint32_t *offs)
{
    __shared__ unsigned long long wsc[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int base = blockIdx.x * SCAN_CHUNK + 4 * (int)threadIdx.x;
    uint32_t v[4];
    unsigned long long s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = base + k < n ? sums[base + k] : 0u;
        s += v[k];
    }
    unsigned long long inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wsc[w] = inc;
    __syncthreads();
    unsigned long long run = part[blockIdx.x] + inc - s;
    for (int i = 0; i < w; ++i) run += wsc[i];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) offs[base + k] = (uint32_t)min(run, 0xffffffffull);
        run += v[k];
    }
}

__device__ __forceinline__ int find_view_by_sb(const gsevt_view *views, int num_views, int sb)
{
    int lo = 0, hi = num_views - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (views[mid].sb_offset <= sb) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int find_view_by_vg(const gsevt_view *views, int num_views, uint32_t vg)
{
    int lo = 0, hi = num_views - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if ((uint32_t)views[mid].vg_offset <= vg) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// block-wide exclusive scan of one value per thread; returns the exclusive prefix
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *wtot)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wtot[w] = inc;
    __syncthreads();
    uint32_t wbase = 0;
    for (int i = 0; i < w; ++i) wbase += wtot[i];
    return wbase + inc - v;
}

struct BinParams {
    const gsevt_view *views;
    int num_views;
    const gsevt_map *maps;
    Workspace ws;
    uint32_t capacity;
    int rgb;
    uint32_t super_bound;  // number of super-tile ids the layout provides for
};

__global__ void __launch_bounds__(GS_BLOCK) k_compact(BinParams p)
{
    __shared__ uint32_t wtot[GS_BLOCK / 32];
    const int sb = blockIdx.x;
    const gsevt_view &V = p.views[find_view_by_sb(p.views, p.num_views, sb)];
    const int n = p.maps[V.map].n;
    const int g = (sb - V.sb_offset) * GS_BLOCK + threadIdx.x;
    const size_t vg = (size_t)V.vg_offset + g;
    int4 bin = make_int4(0, 0, 0, 0);
    if (g < n) bin = p.ws.bin[vg];
    const uint32_t vis = bin.x > 0 ? 1u : 0u;
    const uint32_t c = p.ws.vis_offs[sb] + block_excl_scan(vis, wtot);
    if (g < n) {
        // the adjoint blend accumulates into these with atomics: clear them here, in slot
        // order (coalesced), for every slot, so that a zero gradient also marks the slots
        // the adjoint never reached (the cached twist adjoint skips them)
        p.ws.gradA[vg] = make_float4(0, 0, 0, 0);
        p.ws.gradB[vg] = make_float4(0, 0, 0, 0);
        if (p.rgb) p.ws.gradC[vg] = make_float4(0, 0, 0, 0);
    }
    if (vis) {
        p.ws.dkeys[0][c] = (uint32_t)bin.w;
        p.ws.dvals[0][c] = (uint32_t)vg;
    }
}

// super-tile rectangle [sx0, sx1) x [sy0, sy1) of a tile rectangle (bin.y = x0 | y0 << 16,
// bin.z = x1 | y1 << 16, exclusive upper bounds)
__device__ __forceinline__ void super_rect(int4 bin, int &sx0, int &sy0, int &sx1, int &sy1)
{
    sx0 = (bin.y & 0xffff) / GS_SUPER;
    sy0 = ((bin.y >> 16) & 0xffff) / GS_SUPER;
    sx1 = ((bin.z & 0xffff) - 1) / GS_SUPER + 1;
    sy1 = (((bin.z >> 16) & 0xffff) - 1) / GS_SUPER + 1;
}

// tiles touched per block of 256 depth-sorted visible slots; with COARSE also the
// super-tiles touched (csums) and, in block 0, the first super-tile of every view (soffs)
template <bool COARSE>
__global__ void __launch_bounds__(GS_BLOCK) k_sorted_sums(BinParams p, const uint32_t *sorted_vals)
{
    __shared__ uint32_t wsum[GS_BLOCK / 32], wsum2[GS_BLOCK / 32];
    if (gs_sort_timed_out(p.ws.status)) return;  // the depth order is incomplete (uniform)
    const uint32_t nvis = p.ws.status[5];
    const uint32_t i = blockIdx.x * GS_BLOCK + threadIdx.x;
    uint32_t cnt = 0, scnt = 0;
    if (i < nvis) {
        const int4 b = p.ws.bin[sorted_vals[i]];
        cnt = (uint32_t)b.x;
        if (COARSE && cnt > 0) {
            int sx0, sy0, sx1, sy1;
            super_rect(b, sx0, sy0, sx1, sy1);
            scnt = (uint32_t)((sx1 - sx0) * (sy1 - sy0));
        }
        if (COARSE) {
            // the slot's tile rectangle in depth order (the depth sort's second buffers are
            // free), so that the coarse duplication reads it coalesced
            p.ws.dkeys[1][i] = (uint32_t)b.y;
            p.ws.dvals[1][i] = (uint32_t)b.z;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if (COARSE) scnt += __shfl_xor_sync(0xffffffffu, scnt, o);
    }
    if ((threadIdx.x & 31) == 0) { wsum[threadIdx.x >> 5] = cnt; wsum2[threadIdx.x >> 5] = scnt; }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0, t2 = 0;
        for (int w = 0; w < GS_BLOCK / 32; ++w) { t += wsum[w]; t2 += wsum2[w]; }
        p.ws.tsums[blockIdx.x] = t;
        if (COARSE) p.ws.csums[blockIdx.x] = t2;
    }
    if (COARSE && blockIdx.x == 0) {
        __syncthreads();
        uint32_t carry = 0;
        for (int v0 = 0; v0 < p.num_views; v0 += GS_BLOCK) {
            const int v = v0 + (int)threadIdx.x;
            uint32_t sv = 0;
            if (v < p.num_views) {
                const gsevt_view &V = p.views[v];
                sv = (uint32_t)(((V.tiles_x + GS_SUPER - 1) / GS_SUPER) * ((V.tiles_y + GS_SUPER - 1) / GS_SUPER));
            }
            const uint32_t ex = block_excl_scan(sv, wsum);
            if (v < p.num_views) p.ws.soffs[v] = carry + ex;
            if (threadIdx.x == GS_BLOCK - 1) wsum2[0] = ex + sv;
            __syncthreads();
            carry += wsum2[0];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            p.ws.soffs[p.num_views] = carry;
            // more super-tiles than the layout provides ids for: k_duplicate_coarse clamps
            // the ids (results are wrong but every access stays in bounds)
            if (carry > p.super_bound) atomicOr(p.ws.status, GSEVT_STATUS_LAYOUT);
        }
    }
}

// Warp-cooperative duplication: each warp expands the pairs of its 32 depth-sorted slots
// into one contiguous output range, lane k writing pair k, k + 32, ... of that range
// (coalesced); the owning slot of a pair is found by a shuffle binary search over the
// warp's exclusive prefix of tile counts.
__global__ void __launch_bounds__(GS_BLOCK) k_duplicate(BinParams p, const uint32_t *sorted_vals)
{
    __shared__ uint32_t wtot[GS_BLOCK / 32];
    if (gs_sort_timed_out(p.ws.status)) return;  // the depth order is incomplete (uniform)
    const uint32_t nvis = p.ws.status[5];
    const uint32_t i = blockIdx.x * GS_BLOCK + threadIdx.x;
    if (blockIdx.x * GS_BLOCK >= nvis) return;  // uniform per block
    const int lane = threadIdx.x & 31;
    uint32_t vg = 0;
    int4 bin = make_int4(0, 0, 0, 0);
    if (i < nvis) {
        vg = sorted_vals[i];
        bin = p.ws.bin[vg];
    }
    const uint32_t cnt = (uint32_t)bin.x;
    const uint32_t off = p.ws.toffs[blockIdx.x] + block_excl_scan(cnt, wtot);
    int x0 = 0, y0 = 0, rw = 1, toff = 0, tpx = 1;
    if (cnt > 0) {
        const gsevt_view &V = p.views[find_view_by_vg(p.views, p.num_views, vg)];
        x0 = bin.y & 0xffff;
        y0 = (bin.y >> 16) & 0xffff;
        rw = (bin.z & 0xffff) - x0;
        toff = V.tile_offset;
        tpx = V.tiles_x;
    }
    // warp-level exclusive prefix of the counts and the warp's output base
    uint32_t winc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, winc, o);
        if (lane >= o) winc += y;
    }
    const uint32_t wex = winc - cnt;
    const uint32_t wtotal = __shfl_sync(0xffffffffu, winc, 31);
    const uint32_t wbase = __shfl_sync(0xffffffffu, off, 0);
    for (uint32_t c = 0; c < wtotal; c += 32) {
        const uint32_t k = c + lane;
        // owner: the largest lane s with wex_s <= k (empty slots resolve to a later lane)
        int s = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const uint32_t e = __shfl_sync(0xffffffffu, wex, s + step);
            if (e <= k) s += step;
        }
        const uint32_t q = k - __shfl_sync(0xffffffffu, wex, s);
        const int sx0 = __shfl_sync(0xffffffffu, x0, s), sy0 = __shfl_sync(0xffffffffu, y0, s);
        const int srw = __shfl_sync(0xffffffffu, rw, s), stoff = __shfl_sync(0xffffffffu, toff, s);
        const int stpx = __shfl_sync(0xffffffffu, tpx, s);
        const uint32_t svg = __shfl_sync(0xffffffffu, vg, s);
        const uint32_t idx = wbase + k;
        if (k < wtotal && idx < p.capacity) {
            const int y = sy0 + (int)(q / (uint32_t)srw), x = sx0 + (int)(q % (uint32_t)srw);
            p.ws.keys[0][idx] = (uint32_t)(stoff + y * stpx + x);
            p.ws.vals[0][idx] = svg;
        }
    }
}

// Coarse duplication for the batched tracker: in depth order, one (super-tile id, slot)
// pair per 4x4-tile super-tile of the slot's rectangle (row-major), written with the same
// warp-cooperative expansion as k_duplicate.
__global__ void __launch_bounds__(GS_BLOCK) k_duplicate_coarse(BinParams p, const uint32_t *sorted_vals)
{
    __shared__ uint32_t wtot[GS_BLOCK / 32];
    if (gs_sort_timed_out(p.ws.status)) return;  // the depth order is incomplete (uniform)
    const uint32_t nvis = p.ws.status[5];
    const uint32_t i = blockIdx.x * GS_BLOCK + threadIdx.x;
    if (blockIdx.x * GS_BLOCK >= nvis) return;  // uniform per block
    const int lane = threadIdx.x & 31;
    uint32_t vg = 0;
    int4 bin = make_int4(0, 0, 0, 0);
    if (i < nvis) {
        vg = sorted_vals[i];
        bin = make_int4(1, (int)p.ws.dkeys[1][i], (int)p.ws.dvals[1][i], 0);  // visible: touches >= 1 tile
    }
    int sx0 = 0, sy0 = 0, srw = 1, soff = 0, stx = 1;
    uint32_t cnt = 0;
    if (bin.x > 0) {
        const int v = find_view_by_vg(p.views, p.num_views, vg);
        const gsevt_view &V = p.views[v];
        int sx1, sy1;
        super_rect(bin, sx0, sy0, sx1, sy1);
        srw = sx1 - sx0;
        cnt = (uint32_t)(srw * (sy1 - sy0));
        soff = (int)p.ws.soffs[v];
        stx = (V.tiles_x + GS_SUPER - 1) / GS_SUPER;
    }
    const uint32_t off = p.ws.coffs[blockIdx.x] + block_excl_scan(cnt, wtot);
    uint32_t winc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, winc, o);
        if (lane >= o) winc += y;
    }
    const uint32_t wex = winc - cnt;
    const uint32_t wtotal = __shfl_sync(0xffffffffu, winc, 31);
    const uint32_t wbase = __shfl_sync(0xffffffffu, off, 0);
    for (uint32_t c = 0; c < wtotal; c += 32) {
        const uint32_t k = c + lane;
        int s = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const uint32_t e = __shfl_sync(0xffffffffu, wex, s + step);
            if (e <= k) s += step;
        }
        const uint32_t q = k - __shfl_sync(0xffffffffu, wex, s);
        const int ssx0 = __shfl_sync(0xffffffffu, sx0, s), ssy0 = __shfl_sync(0xffffffffu, sy0, s);
        const int ssrw = __shfl_sync(0xffffffffu, srw, s), ssoff = __shfl_sync(0xffffffffu, soff, s);
        const int sstx = __shfl_sync(0xffffffffu, stx, s);
        const uint32_t svg = __shfl_sync(0xffffffffu, vg, s);
        const uint32_t idx = wbase + k;
        if (k < wtotal && idx < p.capacity) {
            const int y = ssy0 + (int)(q / (uint32_t)ssrw), x = ssx0 + (int)(q % (uint32_t)ssrw);
            // ids past the layout's count (flagged by k_sorted_sums) are clamped in range
            p.ws.keys[0][idx] = min((uint32_t)(ssoff + y * sstx + x), p.super_bound - 1u);
            p.ws.vals[0][idx] = svg;
        }
    }
}

// Tiles of super-tile (sx, sy) covered by a tile rectangle, as a 16-bit mask (bit
// 4 ly + lx for local tile (lx, ly)).
__device__ __forceinline__ uint32_t cover_mask(uint32_t lo, uint32_t hi, int X, int Y)
{
    const int x0 = max((int)(lo & 0xffff) - X, 0), x1 = min((int)(hi & 0xffff) - X, GS_SUPER);
    const int y0 = max((int)(lo >> 16) - Y, 0), y1 = min((int)(hi >> 16) - Y, GS_SUPER);
    if (x0 >= x1 || y0 >= y1) return 0u;
    const uint32_t row = ((1u << x1) - 1u) & ~((1u << x0) - 1u);
    uint32_t m = 0;
#pragma unroll
    for (int ly = 0; ly < GS_SUPER; ++ly)
        if (ly >= y0 && ly < y1) m |= row << (GS_SUPER * ly);
    return m;
}

// One block per super-tile (16 warps, two blocks per SM); warp w takes the w-th
// contiguous sixteenth of the super-tile's depth-ordered coarse list: up to 16 groups of
// 32 entries loaded at once and held in registers for both passes, or, for longer lists,
// four groups at a time in each pass (their loads in flight together).  Pass 1 counts, per warp and
// tile, the entries whose rectangle covers the tile; the block then claims a
// contiguous region of the fine list with one atomic add and lays its 16 tile lists out
// in it; pass 2 rescans the same entries and writes each one into the lists of the tiles
// it covers, at (tile start + earlier warps' count + running count + rank in the ballot).
// Order within a tile is the coarse list order, i.e. depth order with ties in slot order
// - the order of the full stable (tile | depth) sort.  Tile ranges are written for every
// tile of the super-tile; their placement in the fine list follows the order in which
// blocks claim regions, which does not affect any tile's content.
#define FILTER_TILES (GS_SUPER * GS_SUPER)
#define FILTER_WARPS 16
#define FILTER_ILP 4
// entries per lane a warp holds in registers across the two passes (segments of at most
// 32 * FILTER_REG entries are loaded once, all loads in flight together)
#define FILTER_REG 16
template <int G>
__device__ __forceinline__ void filter_load(const uint32_t *cvals, const int4 *bin, uint32_t g, uint32_t b1,
                                            int lane, int X, int Y, uint32_t (&vg)[G], uint32_t (&m)[G])
{
#pragma unroll
    for (int k = 0; k < G; ++k) {
        const uint32_t i = g + 32 * k + lane;
        vg[k] = i < b1 ? cvals[i] : 0xffffffffu;
    }
#pragma unroll
    for (int k = 0; k < G; ++k) {
        m[k] = 0;
        if (vg[k] != 0xffffffffu) {
            const int4 b = bin[vg[k]];
            m[k] = cover_mask((uint32_t)b.y, (uint32_t)b.z, X, Y);
        }
    }
}

// Pass 1 for the first `groups` (warp-uniform) of G groups of 32 entries: per-tile counts
// (lane t adds tile t's count to cnt).  Each lane spreads its 16-bit mask over four words,
// one byte per tile (x * 0x00204081 moves bit i of a nibble to bit 8 i), so four warp-wide
// integer sums count all 16 tiles at once (a group contributes at most 32 per byte).
template <int G>
__device__ __forceinline__ void filter_count(const uint32_t (&m)[G], int groups, int lane, uint32_t &cnt)
{
#pragma unroll
    for (int k = 0; k < G; ++k) {
        if (k < groups) {
            uint32_t packed[4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
                packed[r] = __reduce_add_sync(0xffffffffu, (((m[k] >> (4 * r)) & 0xfu) * 0x00204081u) & 0x01010101u);
            cnt += (packed[(lane >> 2) & 3] >> (8 * (lane & 3))) & 0xffu;
        }
    }
}

// Pass 2 for the first `groups` (warp-uniform) of G groups: each entry into the lists of
// the tiles it covers (pos: the warp-uniform running position of each tile's list).
template <int G>
__device__ __forceinline__ void filter_write(const uint32_t (&vg)[G], const uint32_t (&m)[G], int groups,
                                             uint32_t lt, uint32_t (&pos)[FILTER_TILES], uint32_t *fine_vals,
                                             uint32_t capacity)
{
#pragma unroll
    for (int k = 0; k < G; ++k) {
        if (k < groups) {
#pragma unroll
            for (int t = 0; t < FILTER_TILES; ++t) {
                const bool hit = (m[k] >> t) & 1u;
                const uint32_t bal = __ballot_sync(0xffffffffu, hit);
                const uint32_t at = pos[t] + __popc(bal & lt);
                if (hit && at < capacity) fine_vals[at] = vg[k];
                pos[t] += __popc(bal);
            }
        }
    }
}

__global__ void __launch_bounds__(FILTER_WARPS * 32, 2) k_filter_tiles(const gsevt_view *views, int num_views,
                                                                  Workspace ws, const uint32_t *cvals,
                                                                  uint32_t *fine_vals, uint32_t capacity)
{
    __shared__ uint32_t s_cnt[FILTER_WARPS][FILTER_TILES + 1];  // [warp][tile]
    __shared__ uint32_t s_start[FILTER_TILES];
    const uint32_t sid = blockIdx.x;
    if (gs_sort_timed_out(ws.status)) return;  // the super-tile lists are incomplete (uniform)
    if (sid >= ws.soffs[num_views]) return;  // uniform per block
    int lo = 0, hi = num_views - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ws.soffs[mid] <= sid) lo = mid; else hi = mid - 1;
    }
    const gsevt_view &V = views[lo];
    const int stx = (V.tiles_x + GS_SUPER - 1) / GS_SUPER;
    const uint32_t local = sid - ws.soffs[lo];
    const int X = (int)(local % (uint32_t)stx) * GS_SUPER, Y = (int)(local / (uint32_t)stx) * GS_SUPER;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint2 sr = ws.sranges[sid];
    const uint32_t len = sr.y - sr.x, seg = (len + FILTER_WARPS - 1) / FILTER_WARPS;
    const uint32_t b0 = sr.x + min(len, (uint32_t)w * seg), b1 = sr.x + min(len, (uint32_t)(w + 1) * seg);
    const uint32_t lt = (1u << lane) - 1u;

    // pass 1: per-tile counts of this warp's entries (lane t holds tile t's count).  A
    // segment of at most 32 FILTER_REG entries (the same length for every warp of the block)
    // is loaded once and kept in registers for pass 2; longer ones are loaded in steps of
    // FILTER_ILP groups in each pass.
    const bool in_regs = seg <= 32u * FILTER_REG;  // uniform over the block
    const int rgroups = (int)((b1 - b0 + 31) / 32);
    uint32_t rvg[FILTER_REG], rm[FILTER_REG];
    uint32_t cnt = 0;
    if (in_regs) {
        filter_load<FILTER_REG>(cvals, ws.bin, b0, b1, lane, X, Y, rvg, rm);
        filter_count<FILTER_REG>(rm, rgroups, lane, cnt);
    } else {
        for (uint32_t g = b0; g < b1; g += 32 * FILTER_ILP) {
            uint32_t vg[FILTER_ILP], m[FILTER_ILP];
            filter_load<FILTER_ILP>(cvals, ws.bin, g, b1, lane, X, Y, vg, m);
            filter_count<FILTER_ILP>(m, FILTER_ILP, lane, cnt);
        }
    }
    if (lane < FILTER_TILES) s_cnt[w][lane] = cnt;
    __syncthreads();
    // per tile: exclusive prefix over warps; tile totals -> region of this super-tile
    if (w == 0) {
        uint32_t tot = 0;
        if (lane < FILTER_TILES) {
            for (int q = 0; q < FILTER_WARPS; ++q) {
                const uint32_t c = s_cnt[q][lane];
                s_cnt[q][lane] = tot;
                tot += c;
            }
        }
        uint32_t inc = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        uint32_t base = 0;
        if (lane == FILTER_TILES - 1) base = atomicAdd(ws.status + 7, inc);
        base = __shfl_sync(0xffffffffu, base, FILTER_TILES - 1);
        const uint32_t total = __shfl_sync(0xffffffffu, inc, FILTER_TILES - 1);
        // a region past the fine-list capacity (the key count has flagged the overflow)
        // gets empty ranges, so that no reader goes past the buffer
        const bool fits = (uint64_t)base + total <= (uint64_t)capacity;
        if (lane < FILTER_TILES) {
            const uint32_t start = base + inc - tot;
            s_start[lane] = start;
            const int tx = X + (lane % GS_SUPER), ty = Y + (lane / GS_SUPER);
            if (tx < V.tiles_x && ty < V.tiles_y)
                ws.ranges[V.tile_offset + ty * V.tiles_x + tx] = fits ? make_uint2(start, start + tot) : make_uint2(0, 0);
        }
    }
    __syncthreads();
    // pass 2: write (starts and running counts are warp-uniform)
    uint32_t pos[FILTER_TILES];
#pragma unroll
    for (int t = 0; t < FILTER_TILES; ++t) pos[t] = s_start[t] + s_cnt[w][t];
    if (in_regs) {
        filter_write<FILTER_REG>(rvg, rm, rgroups, lt, pos, fine_vals, capacity);
    } else {
        for (uint32_t g = b0; g < b1; g += 32 * FILTER_ILP) {
            uint32_t vg[FILTER_ILP], m[FILTER_ILP];
            filter_load<FILTER_ILP>(cvals, ws.bin, g, b1, lane, X, Y, vg, m);
            filter_write<FILTER_ILP>(vg, m, FILTER_ILP, lt, pos, fine_vals, capacity);
        }
    }
}

__global__ void k_ranges(const uint32_t *keys, const uint32_t *count_word, uint32_t capacity, uint2 *ranges,
                         const uint32_t *status)
{
    if (gs_sort_timed_out(status)) return;  // the keys' order is incomplete
    uint32_t K = min(*count_word, capacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
        uint32_t t = keys[i];
        if (i == 0 || keys[i - 1] != t) ranges[t].x = i;
        if (i == K - 1 || keys[i + 1] != t) ranges[t].y = i + 1;
    }
}

// Exclusive scan of n block sums into offs, the total into *total (overflow flagged above
// `capacity`, 0: no check): one block for small n, else the three-launch scan with its
// chunk sums in the sort-count table.
int scan_sums(const uint32_t *sums, uint32_t *offs, int n, uint32_t *total, const Workspace &ws, uint32_t capacity,
              bool clear_cursor, cudaStream_t s)
{
    const int nparts = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    if (n <= SCAN_SMALL || (size_t)nparts * 8 > (size_t)(GS_COOP_GP + 1) * 256 * 4) {
        if (clear_cursor) cudaMemsetAsync(ws.status + 7, 0, 4, s);
        k_scan_blocks<<<1, 1024, 0, s>>>(sums, offs, n, total, ws.status, capacity);
    } else {
        unsigned long long *part = (unsigned long long *)ws.sort_hist;
        k_scan_part<<<nparts, 1024, 0, s>>>(sums, n, part);
        k_scan_top<<<1, 1024, 0, s>>>(part, nparts, total, ws.status, capacity, clear_cursor ? 1 : 0);
        k_scan_final<<<nparts, 1024, 0, s>>>(sums, n, part, offs);
    }
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

BinParams make_params(const gsevt_frame *f, const Workspace &ws)
{
    BinParams p;
    p.views = f->views;
    p.num_views = f->L.num_views;
    p.maps = f->maps;
    p.ws = ws;
    p.capacity = f->L.key_capacity;
    p.rgb = f->L.channels == 3;
    p.super_bound = gs_super_bound(f->L);
    return p;
}

}  // namespace

// After preprocess: visible-slot compaction, depth sort, key offsets in depth order.
// Leaves the key count in status[1] (and flags overflow) and N_vis in status[5].  With
// coarse (the batched tracker), *binned (if given) says whether the depth sort's launch
// also built the super-tile lists, so that gs_launch_bin_coarse only filters them.
int gs_launch_depth_order(const gsevt_frame *f, const Workspace &ws, cudaStream_t s, bool coarse, bool *binned)
{
    if (binned) *binned = false;
    const gsevt_layout &L = f->L;
    const uint32_t nb = gs_sorted_blocks(L);
    if (L.num_scan_blocks <= 0 || L.num_vg <= 0) {
        cudaMemsetAsync(ws.status + 1, 0, 4, s);
        cudaMemsetAsync(ws.status + 5, 0, 4, s);
        cudaMemsetAsync(ws.status + 6, 0, 4, s);
        GS_CUDA_CHECK();
        return GSEVT_OK;
    }
    BinParams p = make_params(f, ws);
    // the cooperative sort compacts the visible slots in its first pass; otherwise the
    // visible-slot scan and compaction kernels run first
    GsCompact cmp = {};
    const bool fuse_compact = ws.coop_ok && gs_coop_depth_sort((uint32_t)L.num_vg, (uint32_t)L.num_scan_blocks);
    if (fuse_compact) {
        cmp.views = f->views;
        cmp.num_views = L.num_views;
        cmp.maps = f->maps;
        cmp.bin = ws.bin;
        cmp.gradA = ws.gradA;
        cmp.gradB = ws.gradB;
        cmp.gradC = L.channels == 3 ? ws.gradC : nullptr;
        cmp.num_scan_blocks = (uint32_t)L.num_scan_blocks;
        cmp.enabled = 1;
    } else {
        if (int st = scan_sums(ws.vis_sums, ws.vis_offs, L.num_scan_blocks, ws.status + 5, ws, 0, false, s)) return st;
        k_compact<<<L.num_scan_blocks, GS_BLOCK, 0, s>>>(p);
        GS_CUDA_CHECK();
    }
    GsCoarseBin cb = {};
    if (coarse && binned && gs_super_bits(L) <= 8 && L.total_tiles > 0) {
        cb.views = f->views;
        cb.num_views = L.num_views;
        cb.bin = ws.bin;
        cb.soffs = ws.soffs;
        cb.sranges = ws.sranges;
        cb.cvals = ws.vals[1];
        cb.capacity = (uint32_t)L.key_capacity;
        cb.super_bound = gs_super_bound(L);
        cb.rec_a = ws.keys[0];  // the pair key buffers are free in this path
        cb.rec_b = ws.keys[1];
        cb.enabled = 1;
    }
    bool fused = false;
    int st = gs_launch_depth_sort(ws, (uint32_t)L.num_vg, fuse_compact ? &cmp : nullptr, cb.enabled ? &cb : nullptr,
                                  &fused, s);
    if (st) return st;
    if (fused) {
        *binned = true;
        return GSEVT_OK;
    }
    if (coarse) {
        k_sorted_sums<true><<<nb, GS_BLOCK, 0, s>>>(p, ws.dvals[0]);
        if ((int)nb <= SCAN_SMALL) {
            k_scan_blocks2<<<1, 1024, 0, s>>>(ws.tsums, ws.toffs, ws.status + 1, ws.csums, ws.coffs, ws.status + 6,
                                              (int)nb, ws.status, L.key_capacity);
        } else {
            if (int st = scan_sums(ws.tsums, ws.toffs, (int)nb, ws.status + 1, ws, L.key_capacity, true, s)) return st;
            if (int st = scan_sums(ws.csums, ws.coffs, (int)nb, ws.status + 6, ws, L.key_capacity, false, s)) return st;
        }
    } else {
        k_sorted_sums<false><<<nb, GS_BLOCK, 0, s>>>(p, ws.dvals[0]);
        if (int st = scan_sums(ws.tsums, ws.toffs, (int)nb, ws.status + 1, ws, L.key_capacity, false, s)) return st;
    }
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

// Key duplication in depth order, stable sort by tile, tile ranges.
int gs_launch_bin(const gsevt_frame *f, const Workspace &ws, uint32_t max_keys, cudaStream_t s)
{
    const gsevt_layout &L = f->L;
    cudaMemsetAsync(ws.ranges, 0, (size_t)L.total_tiles * sizeof(uint2), s);
    GS_CUDA_CHECK();
    if (L.num_vg <= 0 || max_keys == 0) return GSEVT_OK;
    BinParams p = make_params(f, ws);
    k_duplicate<<<gs_sorted_blocks(L), GS_BLOCK, 0, s>>>(p, ws.dvals[0]);
    GS_CUDA_CHECK();
    int buf = 0;
    uint32_t *k[2] = {ws.keys[0], ws.keys[1]};
    uint32_t *v[2] = {ws.vals[0], ws.vals[1]};
    int st = gs_launch_sort_t<uint32_t>(k, v, ws.status + 1, L.key_capacity, gs_tile_bits(L), max_keys,
                                       ws.pair_kpt, ws, &buf, s, nullptr, 0);
    if (st) return st;
    if (buf != gs_tile_sort_buffer(L)) return GSEVT_ERR_ARG;
    int blocks = (int)std::min<uint32_t>((max_keys + 255) / 256, 152u * 16u);
    k_ranges<<<blocks, 256, 0, s>>>(ws.keys[buf], ws.status + 1, L.key_capacity, ws.ranges, ws.status);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

// Batched-tracker binning through 4x4-tile super-tiles (after gs_launch_depth_order with
// coarse = true, which also resets the fine-list region cursor): coarse duplication in depth order, stable sort of the coarse pairs by
// super-tile, super-tile ranges, and the per-super-tile filter that writes the fine
// lists and the tile ranges.  The fine lists and ranges equal those of
// gs_launch_bin (depth order within a tile, ties in slot order); only the values are
// produced (the blend reads no keys).  The fine list is returned through *fine_vals.
int gs_launch_bin_coarse(const gsevt_frame *f, const Workspace &ws, uint32_t max_keys, uint32_t **fine_vals,
                         cudaStream_t s, bool binned)
{
    const gsevt_layout &L = f->L;
    *fine_vals = ws.vals[0];
    const uint32_t nsup = gs_super_bound(L);
    const int bits = gs_super_bits(L);
    // up to 256 super-tiles the sort is one pass and writes the super-tile ranges itself
    const bool one_pass = bits <= 8;
    if (L.num_vg <= 0 || max_keys == 0 || L.total_tiles <= 0) {
        cudaMemsetAsync(ws.ranges, 0, (size_t)L.total_tiles * sizeof(uint2), s);
        GS_CUDA_CHECK();
        return GSEVT_OK;
    }
    if (binned) {
        // the depth sort's launch built the super-tile lists in vals[1] and their ranges
        k_filter_tiles<<<nsup, FILTER_WARPS * 32, 0, s>>>(f->views, L.num_views, ws, ws.vals[1], ws.vals[0],
                                                         L.key_capacity);
        GS_CUDA_CHECK();
        *fine_vals = ws.vals[0];
        return GSEVT_OK;
    }
    BinParams p = make_params(f, ws);
    if (!one_pass) cudaMemsetAsync(ws.sranges, 0, (size_t)nsup * 8, s);
    k_duplicate_coarse<<<gs_sorted_blocks(L), GS_BLOCK, 0, s>>>(p, ws.dvals[0]);
    GS_CUDA_CHECK();
    int buf = 0;
    uint32_t *k[2] = {ws.keys[0], ws.keys[1]};
    uint32_t *v[2] = {ws.vals[0], ws.vals[1]};
    int st = gs_launch_sort_t<uint32_t>(k, v, ws.status + 6, L.key_capacity, bits, max_keys, ws.pair_kpt, ws,
                                        &buf, s, one_pass ? ws.sranges : nullptr, one_pass ? nsup : 0u);
    if (st) return st;
    if (!one_pass) {
        int blocks = (int)std::min<uint32_t>((max_keys + 255) / 256, 152u * 16u);
        k_ranges<<<blocks, 256, 0, s>>>(ws.keys[buf], ws.status + 6, L.key_capacity, ws.sranges, ws.status);
    }
    k_filter_tiles<<<nsup, FILTER_WARPS * 32, 0, s>>>(f->views, L.num_views, ws, ws.vals[buf], ws.vals[buf ^ 1],
                                                     L.key_capacity);
    GS_CUDA_CHECK();
    *fine_vals = ws.vals[buf ^ 1];
    return GSEVT_OK;
}
