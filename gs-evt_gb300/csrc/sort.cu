// LSD radix sorts of (32-bit key, 32-bit value) pairs, 8-bit digits, stable.
//
// Two implementations with identical results: a sort whose capacity fits 8192 keys per
// SM runs all its passes in one cooperative launch (k_sort_coop, below the onesweep
// kernels; the batched tracker's depth sort also bins the sorted slots through
// super-tiles in that launch); larger sorts run the onesweep passes described next.
//
// Method: Adinets & Merrill, "Onesweep: A Faster Least Significant Digit Radix Sort
// for GPUs" (2022).  One histogram kernel reads the keys once and counts the digits of
// every pass; each pass is then a single kernel in which a block
//   1. takes a tile ticket from an atomic counter (tickets are handed out in launch
//      order, so every earlier tile belongs to a block that is already running),
//   2. ranks its 256 x KPT keys stably with warp-level match/ballot multisplit,
//   3. publishes its per-digit counts to a look-back table and walks back over the
//      earlier tiles (decoupled look-back) to get its exclusive per-digit prefix,
//   4. scatters keys and values through shared memory to their global positions.
// A pass whose digit is constant over all keys (its histogram holds every key in one
// bin) is the identity permutation and runs as a plain copy.
// Look-back entries are single 64-bit words {epoch:32 | flag:2 | count:30}; the epoch
// changes every pass, so the table never needs clearing between passes or sorts (it
// must be zero-filled once, when the workspace is created).  Every wait on a
// predecessor is bounded by the layout's spin limit (GS_SPIN_LIMIT polls by default); on
// expiry the block records GSEVT_STATUS_SORT_TIMEOUT and continues with a partial prefix,
// which only moves its scatter positions down (they stay inside [0, K)), so a fault can
// never hang the GPU; the kernels that consume the order skip their work afterwards.
// Stability: ranks follow (warp, key slot, lane) order, which is the input order.
#include <atomic>

#include "common.cuh"

namespace {

#define FLAG_AGG 1ull
#define FLAG_PREFIX 2ull

template <typename KT>
__global__ void k_sort_hist(const KT *keys, const uint32_t *count, uint32_t capacity, int passes, uint32_t *hist,
                            uint32_t *status)
{
    __shared__ uint32_t sh[GS_MAX_PASSES][256];
    if (blockIdx.x == 0 && threadIdx.x == 0) gs_sort_reserve_epochs(status, passes);
    for (int i = threadIdx.x; i < GS_MAX_PASSES * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    uint32_t K = min(*count, capacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
        KT k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(k >> (8 * p)) & 255], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}


template <typename KT>
struct PassParams {
    const KT *kin;
    const uint32_t *vin;
    KT *kout;
    uint32_t *vout;
    const uint32_t *hist;       // this pass's 256 digit counts
    uint32_t *counter;          // this pass's tile ticket counter
    unsigned long long *lookback;
    uint32_t *status;
    const uint32_t *count;      // number of keys (device word)
    uint32_t capacity;
    int pass;
    uint2 *ranges;              // single-pass sorts: [start, end) of keys 0..nranges-1, or null
    uint32_t nranges;
    uint32_t spin_limit;        // polls of the look-back wait before it gives up
};

template <typename KT, int SORT_KPT>
__global__ void __launch_bounds__(GS_BLOCK) k_sort_pass(PassParams<KT> p)
{
    constexpr uint32_t SORT_TILE = GS_BLOCK * SORT_KPT;
    __shared__ KT skeys[SORT_TILE];
    __shared__ uint32_t svals[SORT_TILE];
    __shared__ uint32_t whist[GS_BLOCK / 32][256];
    __shared__ uint32_t dstart[256];
    __shared__ uint32_t gbase[256];
    __shared__ uint32_t s_tile;
    __shared__ uint32_t wscan[GS_BLOCK / 32];

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint32_t K = min(*p.count, p.capacity);
    const uint32_t ntiles = (K + SORT_TILE - 1) / SORT_TILE;
    if (p.ranges && blockIdx.x == 0) {
        // a single-pass sort's digit is the whole key: key d occupies bucket d of the
        // output, [exclusive prefix of the histogram, + its count)
        const uint32_t c = p.hist[tid];
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wscan[w] = inc;
        __syncthreads();
        uint32_t wb = 0;
        for (int i = 0; i < w; ++i) wb += wscan[i];
        if ((uint32_t)tid < p.nranges) p.ranges[tid] = make_uint2(wb + inc - c, wb + inc);
        __syncthreads();
    }
    // A pass whose digit is the same for every key is the identity permutation of a
    // stable sort: copy keys and values, with no ranking or look-back.
    if (__syncthreads_or(p.hist[tid] == K)) {
        const uint32_t stride = gridDim.x * GS_BLOCK;
        for (uint32_t i0 = blockIdx.x * GS_BLOCK + tid; i0 < K; i0 += 4 * stride) {
            KT kk[4];
            uint32_t vv[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t i = i0 + k * stride;
                if (i < K) { kk[k] = p.kin[i]; vv[k] = p.vin[i]; }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t i = i0 + k * stride;
                if (i < K) { p.kout[i] = kk[k]; p.vout[i] = vv[k]; }
            }
        }
        return;
    }
    // Persistent over tiles: a block takes the next ticket after finishing its tile, so a
    // grid sized for the resident blocks covers any key count; every ticket below a
    // block's own belongs to a running or finished block, so look-back never waits on a
    // block that has not started.
    for (;;) {
    if (tid == 0) s_tile = atomicAdd(p.counter, 1u);
    for (int i = tid; i < (GS_BLOCK / 32) * 256; i += GS_BLOCK) (&whist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) return;
    const uint32_t base = tile * SORT_TILE;
    const uint32_t count = min((uint32_t)SORT_TILE, K - base);
    const int shift = 8 * p.pass;
    const unsigned long long epoch = (unsigned long long)(p.status[4] + (uint32_t)p.pass);

    KT key[SORT_KPT];
    uint32_t val[SORT_KPT];
    uint32_t rank[SORT_KPT];
    int dig[SORT_KPT];
#pragma unroll
    for (int k = 0; k < SORT_KPT; ++k) {
        uint32_t li = (uint32_t)(w * 32 * SORT_KPT + k * 32 + lane);
        bool ok = li < count;
        key[k] = ok ? p.kin[base + li] : (KT)0;
        val[k] = ok ? p.vin[base + li] : 0u;
        dig[k] = ok ? (int)((key[k] >> shift) & 255) : 256;
    }
    const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < SORT_KPT; ++k) {
        int d = dig[k];
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = 0;
        int leader = __ffs(peers) - 1;
        if (d < 256) before = whist[w][d];
        __syncwarp();
        if (d < 256 && lane == leader) whist[w][d] = before + __popc(peers);
        __syncwarp();
        rank[k] = before + __popc(peers & lt_mask);
    }
    __syncthreads();
    // per digit: exclusive offsets across warps and the tile total
    const int d = tid;  // GS_BLOCK == 256 digits
    uint32_t total = 0;
#pragma unroll
    for (int i = 0; i < GS_BLOCK / 32; ++i) {
        uint32_t t = whist[i][d];
        whist[i][d] = total;
        total += t;
    }
    // publish the tile aggregate (or the inclusive prefix for tile 0)
    volatile unsigned long long *lb = (volatile unsigned long long *)p.lookback;
    if (tile == 0) lb[d] = (epoch << 32) | (FLAG_PREFIX << 30) | total;
    else lb[(size_t)tile * 256 + d] = (epoch << 32) | (FLAG_AGG << 30) | total;
    // decoupled look-back
    uint32_t excl = 0;
    if (tile > 0) {
        int t = (int)tile - 1;
        uint32_t spins = 0;
        while (t >= 0) {
            unsigned long long e = lb[(size_t)t * 256 + d];
            unsigned long long fl = (e >> 30) & 3ull;
            if ((e >> 32) != epoch || fl == 0) {
                if (++spins > p.spin_limit) {
                    atomicOr(p.status, GSEVT_STATUS_SORT_TIMEOUT);
                    break;
                }
                __nanosleep(32);
                continue;
            }
            excl += (uint32_t)(e & 0x3fffffffull);
            if (fl == FLAG_PREFIX) break;
            --t;
        }
        lb[(size_t)tile * 256 + d] = (epoch << 32) | (FLAG_PREFIX << 30) | (excl + total);
    }
    // global digit offset: exclusive scan of the pass histogram + tile prefix
    uint32_t hcount = p.hist[d];
    uint32_t inc = hcount, inc_t = total;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        uint32_t yt = __shfl_up_sync(0xffffffffu, inc_t, o);
        if (lane >= o) { inc += y; inc_t += yt; }
    }
    __shared__ uint32_t wscan_t[GS_BLOCK / 32];
    if (lane == 31) { wscan[w] = inc; wscan_t[w] = inc_t; }
    __syncthreads();
    uint32_t wb = 0, wbt = 0;
    for (int i = 0; i < w; ++i) { wb += wscan[i]; wbt += wscan_t[i]; }
    gbase[d] = (wb + inc - hcount) + excl;
    dstart[d] = wbt + inc_t - total;
    __syncthreads();
    // scatter into shared memory in block-sorted order
#pragma unroll
    for (int k = 0; k < SORT_KPT; ++k) {
        if (dig[k] < 256) {
            uint32_t pos = dstart[dig[k]] + whist[w][dig[k]] + rank[k];
            skeys[pos] = key[k];
            svals[pos] = val[k];
        }
    }
    __syncthreads();
    for (uint32_t i = tid; i < count; i += GS_BLOCK) {
        KT kk = skeys[i];
        int dd = (int)((kk >> shift) & 255);
        uint32_t pos = gbase[dd] + (i - dstart[dd]);
        p.kout[pos] = kk;
        p.vout[pos] = svals[i];
    }
    __syncthreads();  // shared memory is reused by the next tile
    }
}

// ------------------------------------------------------------- cooperative ---------
// Sorts of at most G x GS_COOP_TILE keys with two or more passes run every pass in one
// cooperative launch of G = (SMs x resident blocks) 1024-thread blocks.  Block b owns the
// contiguous run [b TS, (b + 1) TS) of the keys, TS = ceil(K / G), the same run in every
// pass (for the depth sort with the compaction in pass 0, that pass's run is a range of
// 256-slot scan blocks instead, of which the visible slots are the keys).  A pass:
//   1. the block ranks its run stably (warp w takes the w-th 32nd of the run in rounds of
//      32 keys; the lanes holding the same digit are found with nine ballots, so ranks
//      follow the input order) and writes its 256 digit counts into column b of a
//      digit-major table [256][GS_COOP_GP];
//   2. grid barrier; meanwhile the block orders its keys by digit in shared memory (the
//      values were staged there in input order);
//   3. block b scans rows b, b + G, ... of the table in place (exclusive prefix over the
//      blocks) and writes each row's total;
//   4. grid barrier; thread d reads row d's prefix at column b and the row totals, whose
//      exclusive scan over the digits places the block's digit runs; the runs are written
//      out, and a third barrier ends the pass before the next one reads them.
// There is no histogram kernel, no per-pass launch and no look-back chain, and no block
// reads more of the table than its own column and the rows it scans.  A pass whose digit
// is constant is the identity permutation here as well.  Barriers are an arrival counter
// (release add, acquire loads); every wait is bounded by the layout's spin limit, after
// which the block records GSEVT_STATUS_SORT_TIMEOUT and returns at once.  A block that
// passes a barrier has seen every block arrive there, so no block had given up earlier
// and the data it reads is complete; the blocks still running then give up at the next
// barrier, which the returned block never reaches.  Every scatter is also bounded by the
// capacity.  Data written by other blocks
// in an earlier phase is read with ld.global.cg (L2), never through a stale L1 line.
// Optional tail of the depth sort in the batched tracker (gs_launch_depth_order with
// coarse binning): after the last pass the same grid bins the depth-sorted slots through
// 4x4-tile super-tiles.  Block b takes its run of sorted slots again; each warp expands its
// 32nd of the run into (super-tile, slot) pairs, slot by slot in depth order and row-major
// within a slot (the expansion of k_duplicate_coarse), ranks them stably per super-tile
// with ballots and records each pair's id, rank and slot (sweep 1); after the same table
// scan as a sort pass it writes every recorded pair straight to its place in the
// super-tile-sorted list (sweep 2; a warp whose records overflowed its share of the
// scratch expands its pairs again).  That is the order of the stable sort of the
// depth-ordered pairs by super-tile id, with no histogram or sort pass in between.  Block 0 also
// numbers the views' super-tiles (soffs) and writes every super-tile's range; the fine
// pair count and the coarse count land in status[1] and status[6].
typedef GsCoarseBin CoopBin;

struct CoopParams {
    uint32_t *keys[2];
    uint32_t *vals[2];
    uint32_t *cnt;          // [256][GS_COOP_GP] per-block digit counts, then [256] row totals
    uint32_t *barrier;      // arrival counter, zero at launch
    uint32_t *status;
    const uint32_t *count;  // number of keys (device word)
    uint32_t capacity;
    uint32_t spin_limit;    // polls of a barrier wait before it gives up
    int passes;
    CoopBin bin;
    GsCompact cmp;
};

__device__ __forceinline__ void coop_arrive(uint32_t *ctr)
{
    __syncthreads();
    if (threadIdx.x == 0) asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(ctr) : "memory");
}

// Waits (thread 0, bounded) until `target` arrivals; returns false, uniformly over the
// block, when the wait ran out (the status bit is then set and the block must return).
__device__ __forceinline__ bool coop_wait(const uint32_t *ctr, uint32_t target, uint32_t *status, uint32_t limit)
{
    __shared__ int s_go;
    if (threadIdx.x == 0) {
        uint32_t spins = 0, v;
        int go = 1;
        for (;;) {
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
            if (v >= target) break;
            if (++spins > limit) {
                atomicOr(status, GSEVT_STATUS_SORT_TIMEOUT);
                go = 0;
                break;
            }
        }
        s_go = go;
    }
    __syncthreads();
    return s_go != 0;
}

// exclusive scan of one value per thread over threads 0-255 (the digits); every thread
// of the block must call it
__device__ __forceinline__ uint32_t coop_digit_scan(uint32_t v, uint32_t *wsc)
{
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    uint32_t inc = v;
    if (tid < 256) {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsc[w] = inc;
    }
    __syncthreads();
    uint32_t base = 0;
    if (tid < 256)
        for (int i = 0; i < w; ++i) base += wsc[i];
    __syncthreads();  // wsc is reused by the next scan
    return base + inc - v;
}

// Stable in-warp ranking of one 8-bit id per lane (valid lanes only): the lanes with the
// same validity and id are found with nine ballots; returns the lane's rank among them
// plus the warp's running count for the id, which the group's first lane advances.
__device__ __forceinline__ uint32_t coop_warp_rank(bool valid, uint32_t id, uint32_t *wcount, int lane)
{
    uint32_t peers = __ballot_sync(0xffffffffu, valid);
    if (!valid) peers = ~peers;
#pragma unroll
    for (int bit = 0; bit < 8; ++bit) {
        const uint32_t m = __ballot_sync(0xffffffffu, (id >> bit) & 1u);
        peers &= ((id >> bit) & 1u) ? m : ~m;
    }
    const int leader = __ffs(peers) - 1;
    uint32_t before = 0;
    if (valid) before = wcount[id];
    __syncwarp();
    if (valid && lane == leader) wcount[id] = before + __popc(peers);
    __syncwarp();
    return before + __popc(peers & ((1u << lane) - 1u));
}

// Views the fused super-tile binning handles (their tables are staged in shared memory).
#define COOP_MAX_VIEWS 64

// The (super-tile id, slot) pairs of one warp's 32nd of a block's run of depth-sorted
// slots, in order (slot by slot, row-major within a slot), 32 at a time: f(valid, id, slot)
// is called by every lane for every batch.  The run's slots and tile rectangles are in
// shared memory (s_vg, s_lo, s_hi), as are the views' slot offsets, super-tile offsets
// and super-tile row lengths.
template <typename F>
__device__ __forceinline__ void coop_coarse_pairs(const uint32_t *s_vg, const uint32_t *s_lo, const uint32_t *s_hi,
                                                  const uint32_t *s_vgoff, const uint32_t *s_soff,
                                                  const int *s_stx, int num_views, uint32_t super_bound,
                                                  uint32_t nb, uint32_t span, int w, int lane, F f)
{
    for (uint32_t g0 = 0; g0 < span; g0 += 32) {  // uniform over the warp
        const uint32_t li = (uint32_t)w * span + g0 + (uint32_t)lane;
        uint32_t vg = 0, c = 0, mg = 0;
        int sx0 = 0, sy0 = 0, srw = 1, soff = 0, stx = 1;
        if (g0 + (uint32_t)lane < span && li < nb) {
            vg = s_vg[li];
            const uint32_t lo4 = s_lo[li], hi4 = s_hi[li];
            int lo = 0, hi = num_views - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_vgoff[mid] <= vg) lo = mid; else hi = mid - 1;
            }
            sx0 = (int)(lo4 & 0xffffu) / GS_SUPER;
            sy0 = (int)(lo4 >> 16) / GS_SUPER;
            const int sx1 = ((int)(hi4 & 0xffffu) - 1) / GS_SUPER + 1;
            const int sy1 = ((int)(hi4 >> 16) - 1) / GS_SUPER + 1;
            srw = sx1 - sx0;
            c = (uint32_t)(srw * (sy1 - sy0));  // visible slots touch at least one tile
            soff = (int)s_soff[lo];
            stx = s_stx[lo];
            // q / srw = umulhi(q, floor((2^32 - 1) / srw) + 1), exact for q < 2^16 and
            // 2 <= srw <= 2^16 (here q < 256: at most 256 super-tiles)
            mg = srw > 1 ? 0xffffffffu / (uint32_t)srw + 1u : 0u;
        }
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        const uint32_t ex = inc - c;
        const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
        for (uint32_t k0 = 0; k0 < total; k0 += 32) {
            const uint32_t k = k0 + (uint32_t)lane;
            // owner: the largest lane s with ex_s <= k (empty slots resolve to a later lane)
            int o = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const uint32_t e = __shfl_sync(0xffffffffu, ex, o + step);
                if (e <= k) o += step;
            }
            const uint32_t qq = k - __shfl_sync(0xffffffffu, ex, o);
            const int osx0 = __shfl_sync(0xffffffffu, sx0, o), osy0 = __shfl_sync(0xffffffffu, sy0, o);
            const int osrw = __shfl_sync(0xffffffffu, srw, o), osoff = __shfl_sync(0xffffffffu, soff, o);
            const int ostx = __shfl_sync(0xffffffffu, stx, o);
            const uint32_t ovg = __shfl_sync(0xffffffffu, vg, o), omg = __shfl_sync(0xffffffffu, mg, o);
            const bool valid = k < total;
            uint32_t id = 0;
            if (valid) {
                const uint32_t qy = osrw > 1 ? __umulhi(qq, omg) : qq;
                const int y = osy0 + (int)qy, x = osx0 + (int)(qq - qy * (uint32_t)osrw);
                // ids past the layout's count (flagged by block 0) are clamped in range
                id = min((uint32_t)(osoff + y * ostx + x), super_bound - 1u);
            }
            f(valid, id, ovg);
        }
    }
}

#define COOP_WARPS (GS_COOP_THREADS / 32)
__global__ void __launch_bounds__(GS_COOP_THREADS, 1) k_sort_coop(CoopParams p)
{
    extern __shared__ uint32_t coop_smem[];
    // block-sorted keys and values, and the values staged in input order
    uint32_t *skeys = coop_smem, *svals = coop_smem + GS_COOP_TILE, *sin = coop_smem + 2 * GS_COOP_TILE;
    __shared__ uint32_t whist[COOP_WARPS][256];
    __shared__ uint32_t qall[4][256];
    __shared__ uint32_t gbase[256], dstart[256];
    __shared__ uint32_t wsc[8];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int d = tid & 255, q = tid >> 8;  // digit and quarter (four threads per digit)
    const uint32_t G = gridDim.x, b = blockIdx.x;
    // with the compaction fused into pass 0 the key count is only known after that pass
    uint32_t K = p.cmp.enabled ? 1u : min(*p.count, p.capacity);
    if (p.bin.enabled && b == 0 && tid == 0) {
        // super-tile numbering of the views; the fine-list cursor of the filter that follows
        uint32_t carry = 0;
        for (int v = 0; v < p.bin.num_views; ++v) {
            const gsevt_view &V = p.bin.views[v];
            p.bin.soffs[v] = carry;
            carry += (uint32_t)(((V.tiles_x + GS_SUPER - 1) / GS_SUPER) * ((V.tiles_y + GS_SUPER - 1) / GS_SUPER));
        }
        p.bin.soffs[p.bin.num_views] = carry;
        if (carry > p.bin.super_bound) atomicOr(p.status, GSEVT_STATUS_LAYOUT);
        p.status[7] = 0u;
    }
    if (K == 0) {  // uniform over the grid: no slot is visible, every super-tile list is empty
        if (p.bin.enabled && b == 0) {
            for (uint32_t i = tid; i < p.bin.super_bound; i += GS_COOP_THREADS) p.bin.sranges[i] = make_uint2(0u, 0u);
            if (tid == 0) p.status[6] = 0u;
        }
        return;
    }
    if (K > G * (uint32_t)GS_COOP_TILE || G > GS_COOP_GP || G * COOP_WARPS < 256) {
        // the launcher sizes the grid for the capacity, so this is unreachable
        if (b == 0 && tid == 0) atomicOr(p.status, GSEVT_STATUS_KEY_OVERFLOW);
        return;
    }
    uint32_t *row_tot = p.cnt + 256 * GS_COOP_GP;
    __shared__ uint32_t s_total[2];
    // this block's run of keys: [t0, t0 + nb), nb <= GS_COOP_TILE; with the compaction in
    // pass 0, that pass's run is instead scan blocks [sb0, sb0 + nsb) of the slot space
    // (256 slots each, at most GS_COOP_TILE), of which the visible ones are its keys
    uint32_t TS = (K + G - 1) / G;
    uint32_t t0 = min(K, b * TS);
    uint32_t nb = min(K, t0 + TS) - t0;
    uint32_t sb0 = 0;
    if (p.cmp.enabled) {
        const uint32_t per = (p.cmp.num_scan_blocks + G - 1) / G;
        sb0 = min(p.cmp.num_scan_blocks, b * per);
        nb = (min(p.cmp.num_scan_blocks, sb0 + per) - sb0) * (uint32_t)GS_BLOCK;
        t0 = 0;
    }
    uint32_t span = (nb + COOP_WARPS - 1) / COOP_WARPS;  // keys of each warp (<= 32 GS_COOP_KPT)
    int rounds = (int)((span + 31) / 32);
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t nbar = 0;
    for (int pass = 0; pass < p.passes; ++pass) {
        const bool compact = p.cmp.enabled && pass == 0;  // uniform
        const bool odd = (pass & 1) != 0;  // selects, not a dynamic index into the parameters
        const uint32_t *kin = odd ? p.keys[1] : p.keys[0], *vin = odd ? p.vals[1] : p.vals[0];
        uint32_t *kout = odd ? p.keys[0] : p.keys[1], *vout = odd ? p.vals[0] : p.vals[1];
        const int shift = 8 * pass;
        for (int i = tid; i < COOP_WARPS * 256; i += GS_COOP_THREADS) (&whist[0][0])[i] = 0;
        // keys into registers, values staged in shared memory in input order
        uint32_t key[GS_COOP_KPT], rank[GS_COOP_KPT];
        uint32_t ok = 0;
        if (compact) {
            // slot li of the run: scan block sb0 + li / 256, thread li % 256 of it; a key
            // when the slot exists and touches a tile (the visibility test of k_compact)
#pragma unroll
            for (int k = 0; k < GS_COOP_KPT; ++k) {
                const uint32_t o = (uint32_t)(k * 32 + lane), li = (uint32_t)w * span + o;
                bool v = false;
                key[k] = 0u;
                rank[k] = 0u;
                if (o < span && li < nb) {
                    const int sb = (int)(sb0 + li / GS_BLOCK);
                    int lo = 0, hi = p.cmp.num_views - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (p.cmp.views[mid].sb_offset <= sb) lo = mid; else hi = mid - 1;
                    }
                    const gsevt_view &V = p.cmp.views[lo];
                    const int g = (sb - V.sb_offset) * GS_BLOCK + (int)(li % GS_BLOCK);
                    if (g < p.cmp.maps[V.map].n) {
                        const uint32_t vg = (uint32_t)V.vg_offset + (uint32_t)g;
                        const int4 b4 = p.cmp.bin[vg];
                        // the adjoint blend accumulates into these with atomics; they are
                        // cleared for every slot, so that a zero gradient also marks the
                        // slots the adjoint never reached (the cached twist adjoint skips them)
                        p.cmp.gradA[vg] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        p.cmp.gradB[vg] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        if (p.cmp.gradC) p.cmp.gradC[vg] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        if (b4.x > 0) {
                            v = true;
                            key[k] = (uint32_t)b4.w;
                            sin[li] = vg;
                        }
                    }
                }
                ok |= (uint32_t)v << k;
            }
        } else {
#pragma unroll
            for (int k = 0; k < GS_COOP_KPT; ++k) {
                const uint32_t o = (uint32_t)(k * 32 + lane), li = (uint32_t)w * span + o;
                const bool v = o < span && li < nb;
                key[k] = v ? __ldcg(kin + t0 + li) : 0u;
                if (v) sin[li] = __ldcg(vin + t0 + li);
                rank[k] = 0u;
                ok |= (uint32_t)v << k;
            }
        }
        __syncthreads();
        // stable ranks within each warp's keys, per-warp digit counts
#pragma unroll
        for (int k = 0; k < GS_COOP_KPT; ++k) {
            if (k < rounds) {  // uniform over the block
                const bool valid = ((ok >> k) & 1u) != 0;
                const uint32_t dg = (key[k] >> shift) & 255u;
                // lanes with the same validity and the same eight digit bits
                uint32_t peers = __ballot_sync(0xffffffffu, valid);
                if (!valid) peers = ~peers;
#pragma unroll
                for (int bit = 0; bit < 8; ++bit) {
                    const uint32_t m = __ballot_sync(0xffffffffu, (dg >> bit) & 1u);
                    peers &= ((dg >> bit) & 1u) ? m : ~m;
                }
                const int leader = __ffs(peers) - 1;
                uint32_t before = 0;
                if (valid) before = whist[w][dg];
                __syncwarp();
                if (valid && lane == leader) whist[w][dg] = before + __popc(peers);
                __syncwarp();
                rank[k] = before + __popc(peers & lt);
            }
        }
        __syncthreads();
        // per digit: exclusive offsets over the warps (each quarter of the threads takes
        // eight warps) and the block's count
        {
            uint32_t s = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) s += whist[8 * q + i][d];
            qall[q][d] = s;
        }
        __syncthreads();
        uint32_t pre = 0, tot = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint32_t v = qall[i][d];
            pre += i < q ? v : 0u;
            tot += v;
        }
        {
            uint32_t run = pre;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const uint32_t v = whist[8 * q + i][d];
                whist[8 * q + i][d] = run;
                run += v;
            }
        }
        if (q == 0) p.cnt[(size_t)d * GS_COOP_GP + b] = tot;
        coop_arrive(p.barrier);
        ++nbar;
        // while the other blocks arrive: this block's keys in digit order in shared memory
        {
            const uint32_t ds = coop_digit_scan(tot, wsc);
            if (tid < 256) dstart[d] = ds;
            if (tid == 255) s_total[0] = ds + tot;  // this block's keys
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < GS_COOP_KPT; ++k) {
            if ((ok >> k) & 1u) {
                const uint32_t dg = (key[k] >> shift) & 255u;
                const uint32_t pos = dstart[dg] + whist[w][dg] + rank[k];
                skeys[pos] = key[k];
                svals[pos] = sin[(uint32_t)w * span + (uint32_t)(k * 32 + lane)];
            }
        }
        if (!coop_wait(p.barrier, nbar * G, p.status, p.spin_limit)) return;
        // rows b, b + G, ... of the table: exclusive prefix over the blocks, in place, and
        // the row total (warp i takes row b + i G; lane l holds columns l, l + 32, ...)
        {
            const uint32_t r = b + (uint32_t)w * G;
            if (r < 256) {
                uint32_t *row = p.cnt + (size_t)r * GS_COOP_GP;
                uint32_t v[GS_COOP_GP / 32];
#pragma unroll
                for (int c = 0; c < GS_COOP_GP / 32; ++c) {
                    const uint32_t col = (uint32_t)(c * 32 + lane);
                    v[c] = col < G ? __ldcg(row + col) : 0u;
                }
                uint32_t run = 0;
#pragma unroll
                for (int c = 0; c < GS_COOP_GP / 32; ++c) {
                    const uint32_t col = (uint32_t)(c * 32 + lane);
                    uint32_t inc = v[c];
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
                        if (lane >= o) inc += y;
                    }
                    if (col < G) row[col] = run + inc - v[c];
                    run += __shfl_sync(0xffffffffu, inc, 31);
                }
                if (lane == 0) row_tot[r] = run;
            }
        }
        coop_arrive(p.barrier);
        ++nbar;
        if (!coop_wait(p.barrier, nbar * G, p.status, p.spin_limit)) return;
        uint32_t A = 0, E = 0;
        if (tid < 256) {
            E = __ldcg(p.cnt + (size_t)d * GS_COOP_GP + b);
            A = __ldcg(row_tot + d);
        }
        {
            const uint32_t ga = coop_digit_scan(A, wsc);
            if (tid < 256) gbase[d] = ga + E;
            if (tid == 255) s_total[1] = ga + A;  // all blocks' keys
        }
        __syncthreads();
        const uint32_t nwrite = s_total[0];
        for (uint32_t i = tid; i < nwrite; i += GS_COOP_THREADS) {
            const uint32_t kk = skeys[i];
            const uint32_t dg = (kk >> shift) & 255u;
            const uint32_t pos = gbase[dg] + (i - dstart[dg]);
            if (pos < p.capacity) {
                kout[pos] = kk;
                vout[pos] = svals[i];
            }
        }
        if (compact) {
            // the visible slots are now keys [0, K) of buffer 1: the runs of the later passes
            K = min(s_total[1], p.capacity);
            if (b == 0 && tid == 0) p.status[5] = K;  // N_vis
            TS = (K + G - 1) / G;
            t0 = min(K, b * TS);
            nb = min(K, t0 + TS) - t0;
            span = (nb + COOP_WARPS - 1) / COOP_WARPS;
            rounds = (int)((span + 31) / 32);
        }
        if (pass + 1 < p.passes) {
            coop_arrive(p.barrier);
            ++nbar;
            if (!coop_wait(p.barrier, nbar * G, p.status, p.spin_limit)) return;
        }
    }
    if (K == 0) {  // no visible slot (uniform; only reachable with the compaction in pass 0)
        if (p.bin.enabled && b == 0) {
            for (uint32_t i = tid; i < p.bin.super_bound; i += GS_COOP_THREADS) p.bin.sranges[i] = make_uint2(0u, 0u);
            if (tid == 0) p.status[6] = 0u;
        }
        return;
    }
    if (!p.bin.enabled) return;
    // ---- coarse binning of the sorted slots (the tail described above CoopBin) ----
    __shared__ uint32_t s_vgoff[COOP_MAX_VIEWS], s_soff[COOP_MAX_VIEWS];
    __shared__ int s_stx[COOP_MAX_VIEWS];
    coop_arrive(p.barrier);
    ++nbar;
    for (int i = tid; i < COOP_WARPS * 256; i += GS_COOP_THREADS) (&whist[0][0])[i] = 0;
    if (!coop_wait(p.barrier, nbar * G, p.status, p.spin_limit)) return;
    const int nviews = min(p.bin.num_views, COOP_MAX_VIEWS);  // the launcher checks the count
    if (tid < nviews) {
        const gsevt_view &V = p.bin.views[tid];
        s_vgoff[tid] = (uint32_t)V.vg_offset;
        s_soff[tid] = __ldcg(p.bin.soffs + tid);
        s_stx[tid] = (V.tiles_x + GS_SUPER - 1) / GS_SUPER;
    }
    // the block's run of sorted slots and their tile rectangles, into shared memory
    // (the sort's staging buffers are free now); all loads of the run in flight together
    uint32_t *s_vg = skeys, *s_lo = svals, *s_hi = sin;
    const uint32_t *sorted = (p.passes & 1) ? p.vals[1] : p.vals[0];
    uint32_t fine = 0;
    for (uint32_t i = tid; i < nb; i += GS_COOP_THREADS) {
        const uint32_t vg = __ldcg(sorted + t0 + i);
        const int4 b4 = p.bin.bin[vg];
        s_vg[i] = vg;
        s_lo[i] = (uint32_t)b4.y;
        s_hi[i] = (uint32_t)b4.z;
        fine += (uint32_t)b4.x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) fine += __shfl_xor_sync(0xffffffffu, fine, o);
    if (lane == 0 && fine) atomicAdd(p.status + 1, fine);
    __syncthreads();
    // sweep 1: pairs per (warp, super-tile); each pair's id, rank in its warp and slot are
    // also recorded in the warp's share of the scratch buffers, so that sweep 2 only has to
    // place them (a warp whose pairs overflow its share expands them again instead)
    __shared__ uint32_t s_nw[COOP_WARPS];
    const uint32_t rw_cap = p.bin.capacity / G / COOP_WARPS;
    const size_t rbase = ((size_t)b * COOP_WARPS + (size_t)w) * rw_cap;
    uint32_t nrec = 0;
    coop_coarse_pairs(s_vg, s_lo, s_hi, s_vgoff, s_soff, s_stx, nviews, p.bin.super_bound, nb, span, w, lane,
                      [&](bool valid, uint32_t id, uint32_t slot) {
                          const uint32_t r = coop_warp_rank(valid, id, whist[w], lane);
                          const uint32_t j = nrec + (uint32_t)lane;  // valid lanes are a prefix
                          if (valid && j < rw_cap) {
                              p.bin.rec_a[rbase + j] = (id << 24) | r;
                              p.bin.rec_b[rbase + j] = slot;
                          }
                          nrec += __popc(__ballot_sync(0xffffffffu, valid));
                      });
    if (lane == 0) s_nw[w] = nrec;
    __syncthreads();
    {
        uint32_t s4 = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) s4 += whist[8 * q + i][d];
        qall[q][d] = s4;
    }
    __syncthreads();
    uint32_t pre = 0, tot = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint32_t v = qall[i][d];
        pre += i < q ? v : 0u;
        tot += v;
    }
    {
        uint32_t run = pre;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const uint32_t v = whist[8 * q + i][d];
            whist[8 * q + i][d] = run;
            run += v;
        }
    }
    if (q == 0) p.cnt[(size_t)d * GS_COOP_GP + b] = tot;
    coop_arrive(p.barrier);
    ++nbar;
    if (!coop_wait(p.barrier, nbar * G, p.status, p.spin_limit)) return;
    {
        const uint32_t r = b + (uint32_t)w * G;
        if (r < 256) {
            uint32_t *row = p.cnt + (size_t)r * GS_COOP_GP;
            uint32_t v[GS_COOP_GP / 32];
#pragma unroll
            for (int c = 0; c < GS_COOP_GP / 32; ++c) {
                const uint32_t col = (uint32_t)(c * 32 + lane);
                v[c] = col < G ? __ldcg(row + col) : 0u;
            }
            uint32_t run = 0;
#pragma unroll
            for (int c = 0; c < GS_COOP_GP / 32; ++c) {
                const uint32_t col = (uint32_t)(c * 32 + lane);
                uint32_t inc = v[c];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += y;
                }
                if (col < G) row[col] = run + inc - v[c];
                run += __shfl_sync(0xffffffffu, inc, 31);
            }
            if (lane == 0) row_tot[r] = run;
        }
    }
    coop_arrive(p.barrier);
    ++nbar;
    if (!coop_wait(p.barrier, nbar * G, p.status, p.spin_limit)) return;
    uint32_t A = 0, E = 0;
    if (tid < 256) {
        E = __ldcg(p.cnt + (size_t)d * GS_COOP_GP + b);
        A = __ldcg(row_tot + d);
    }
    const uint32_t ga = coop_digit_scan(A, wsc);
    if (tid < 256) {
        gbase[d] = ga + E;
        if (b == 0) {
            // clamped to the capacity: past it no pair is written (overflow is flagged below),
            // and the filter must not read there
            if ((uint32_t)d < p.bin.super_bound)
                p.bin.sranges[d] = make_uint2(min(ga, p.bin.capacity), min(ga + A, p.bin.capacity));
            if (d == 255) {
                const uint32_t coarse = ga + A;
                p.status[6] = coarse;
                if (coarse > p.bin.capacity) atomicOr(p.status, GSEVT_STATUS_KEY_OVERFLOW);
            }
        }
    }
    if (b == 0 && tid == 0) {
        // every block added its fine count before the last barrier
        if (__ldcg(p.status + 1) > p.bin.capacity) atomicOr(p.status, GSEVT_STATUS_KEY_OVERFLOW);
    }
    __syncthreads();
    // sweep 2: every pair to its place in its super-tile's list (gbase: the super-tile's
    // start plus the pairs of earlier blocks; whist: the pairs of earlier warps of the block)
    const uint32_t nw = s_nw[w];  // uniform over the warp
    if (nw <= rw_cap) {
        for (uint32_t j = (uint32_t)lane; j < nw; j += 32) {
            const uint32_t a = __ldcg(p.bin.rec_a + rbase + j), slot = __ldcg(p.bin.rec_b + rbase + j);
            const uint32_t id = a >> 24;
            const uint32_t pos = gbase[id] + whist[w][id] + (a & 0xffffffu);
            if (pos < p.bin.capacity) p.bin.cvals[pos] = slot;
        }
    } else {
        coop_coarse_pairs(s_vg, s_lo, s_hi, s_vgoff, s_soff, s_stx, nviews, p.bin.super_bound, nb, span, w, lane,
                          [&](bool valid, uint32_t id, uint32_t slot) {
                              const uint32_t r = coop_warp_rank(valid, id, whist[w], lane);
                              if (valid) {
                                  const uint32_t pos = gbase[id] + r;
                                  if (pos < p.bin.capacity) p.bin.cvals[pos] = slot;
                              }
                          });
    }
}
#undef COOP_WARPS

// grid of the cooperative sort on each device: 0 not prepared, -1 unavailable (set once
// per device by gs_sort_prepare, read by every launch; atomic so that workspaces set up
// from several host threads are safe)
std::atomic<int> g_coop_grid[64];

int coop_grid_query(int dev)
{
    int coop = 0, sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return -1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    const int smem = 3 * GS_COOP_TILE * 4;
    if (cudaFuncSetAttribute(k_sort_coop, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return -1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sort_coop, GS_COOP_THREADS, smem) != cudaSuccess)
        return -1;
    // at most GS_COOP_GP table columns; at least 8 blocks, so 256 / G rows fit 32 warps
    const int g = std::min(sms * per_sm, GS_COOP_GP);
    return g >= 8 ? g : -1;
}

// Launches the cooperative sort when this device has it prepared and the capacity fits
// its grid; returns false (nothing launched) otherwise.  *st receives the launch status.
int coop_grid_here()
{
    int dev = 0;
    return (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) ? g_coop_grid[dev].load(std::memory_order_relaxed)
                                                                        : -1;
}

bool launch_coop(uint32_t *const keys[2], uint32_t *const vals[2], const uint32_t *count, uint32_t capacity,
                 int passes, const Workspace &ws, cudaStream_t s, const GsCoarseBin *bin, int *st,
                 const GsCompact *cmp = nullptr)
{
    const int g = coop_grid_here();
    if (!ws.coop_ok || g <= 0 || (uint64_t)capacity > (uint64_t)g * GS_COOP_TILE) return false;
    if (cmp && (uint64_t)cmp->num_scan_blocks * GS_BLOCK > (uint64_t)g * GS_COOP_TILE) return false;
    cudaMemsetAsync(ws.sort_counter, 0, 4, s);
    CoopParams cp;
    cp.keys[0] = keys[0];
    cp.keys[1] = keys[1];
    cp.vals[0] = vals[0];
    cp.vals[1] = vals[1];
    cp.cnt = ws.sort_hist;
    cp.barrier = ws.sort_counter;
    cp.status = ws.status;
    cp.count = count;
    cp.capacity = capacity;
    cp.spin_limit = ws.spin_limit;
    cp.passes = passes;
    cp.cmp = {};
    if (cmp) {
        cp.cmp = *cmp;
        cp.cmp.enabled = 1;
    }
    cp.bin = {};
    if (bin && bin->super_bound >= 1 && bin->super_bound <= 256 && bin->num_views >= 1 &&
        bin->num_views <= COOP_MAX_VIEWS) {
        cp.bin = *bin;
        cp.bin.enabled = 1;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)g);
    cfg.blockDim = dim3(GS_COOP_THREADS);
    cfg.dynamicSmemBytes = 3 * GS_COOP_TILE * 4;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    *st = GSEVT_OK;
    if (cudaLaunchKernelEx(&cfg, k_sort_coop, cp) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        *st = GSEVT_ERR_CUDA;
    return true;
}

}  // namespace

template <typename KT>
int gs_launch_sort_t(KT *const keys[2], uint32_t *const vals[2], const uint32_t *count, uint32_t capacity,
                     int bits, uint32_t max_keys, int kpt, const Workspace &ws, int *out_buf, cudaStream_t s,
                     uint2 *ranges, uint32_t nranges);

bool gs_coop_depth_sort(uint32_t capacity, uint32_t num_scan_blocks)
{
    const int g = coop_grid_here();
    return g > 0 && capacity > 0 && (uint64_t)capacity <= (uint64_t)g * GS_COOP_TILE &&
           (uint64_t)num_scan_blocks * GS_BLOCK <= (uint64_t)g * GS_COOP_TILE;
}

int gs_launch_depth_sort(const Workspace &ws, uint32_t capacity, const GsCompact *cmp, const GsCoarseBin *bin,
                         bool *binned, cudaStream_t s)
{
    *binned = false;
    uint32_t *dk[2] = {ws.dkeys[0], ws.dkeys[1]};
    uint32_t *dv[2] = {ws.dvals[0], ws.dvals[1]};
    int st = 0;
    if (capacity > 0 && launch_coop(dk, dv, ws.status + 5, capacity, 4, ws, s, bin, &st, cmp)) {
        *binned = st == GSEVT_OK && bin && bin->super_bound >= 1 && bin->super_bound <= 256 && bin->num_views >= 1 &&
                  bin->num_views <= COOP_MAX_VIEWS;
        return st;
    }
    if (cmp) return GSEVT_ERR_ARG;  // the compaction runs only inside the cooperative sort
    int buf = 0;
    st = gs_launch_sort_t<uint32_t>(dk, dv, ws.status + 5, capacity, 32, capacity, ws.depth_kpt, ws, &buf, s,
                                    nullptr, 0);
    if (st) return st;
    return buf == 0 ? GSEVT_OK : GSEVT_ERR_ARG;  // 4 passes: the result is back in buffer 0
}

// Sets up the cooperative sort on the current device (function attributes and its grid);
// called outside stream capture, e.g. when a workspace is initialised.  A sort launched
// on a device that was never prepared (or that lacks cooperative launches) runs the
// onesweep passes.
void gs_sort_prepare()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { cudaGetLastError(); return; }
    if (g_coop_grid[dev].load(std::memory_order_relaxed) == 0)
        g_coop_grid[dev].store(coop_grid_query(dev), std::memory_order_relaxed);
    cudaGetLastError();
}

// Sorts keys[0]/vals[0] (count in *count, a device word) on the low `bits` bits; the
// result is in buffer index (passes & 1), returned through *out_buf.  max_keys bounds
// the grid (a host-known count, or the capacity when the count is only known on the
// device).  The look-back table must hold gs_sort_tiles(capacity, kpt) * 256 entries.
// ranges: for a single-pass sort (bits <= 8), also write the [start, end) range of
// every key below nranges (no separate range pass); null otherwise.
template <typename KT>
int gs_launch_sort_t(KT *const keys[2], uint32_t *const vals[2], const uint32_t *count, uint32_t capacity,
                     int bits, uint32_t max_keys, int kpt, const Workspace &ws, int *out_buf, cudaStream_t s,
                     uint2 *ranges, uint32_t nranges)
{
    if (kpt != 4 && kpt != 8 && kpt != 12) return GSEVT_ERR_ARG;
    int passes = (bits + 7) / 8;
    if (passes < 1) passes = 1;
    if (passes > GS_MAX_PASSES || passes * 8 > (int)(8 * sizeof(KT)) + 7) return GSEVT_ERR_ARG;
    if (ranges && (passes != 1 || nranges > 256)) return GSEVT_ERR_ARG;
    *out_buf = passes & 1;
    if (max_keys > capacity) max_keys = capacity;
    if (max_keys == 0) return GSEVT_OK;
    if (sizeof(KT) == 4 && passes >= 2 && !ranges) {
        int st = 0;
        if (launch_coop((uint32_t *const *)keys, vals, count, capacity, passes, ws, s, nullptr, &st)) return st;
    }
    cudaMemsetAsync(ws.sort_hist, 0, GS_MAX_PASSES * 256 * 4, s);
    cudaMemsetAsync(ws.sort_counter, 0, GS_MAX_PASSES * 4, s);
    GS_CUDA_CHECK();
    // ~4096 keys per block, at most two blocks per SM: each block flushes up to 256 bins per
    // pass to the global histogram with atomics, so fewer, fuller blocks flush less
    int hblocks = (int)std::min<uint32_t>((max_keys + 4095) / 4096, 152u * 2u);
    k_sort_hist<KT><<<hblocks, 256, 0, s>>>(keys[0], count, capacity, passes, ws.sort_hist, ws.status);
    GS_CUDA_CHECK();
    // resident blocks per SM of the pass kernel (registers / shared memory bound)
    const uint32_t per_sm = kpt == 4 ? 6u : (kpt == 8 ? 4u : 3u);
    uint32_t tiles = std::min(gs_sort_tiles(max_keys, kpt), 152u * per_sm);
    for (int pass = 0; pass < passes; ++pass) {
        PassParams<KT> p;
        int src = pass & 1;
        p.kin = keys[src];
        p.vin = vals[src];
        p.kout = keys[src ^ 1];
        p.vout = vals[src ^ 1];
        p.hist = ws.sort_hist + 256 * pass;
        p.counter = ws.sort_counter + pass;
        p.lookback = ws.sort_lookback;
        p.status = ws.status;
        p.count = count;
        p.capacity = capacity;
        p.pass = pass;
        p.ranges = ranges;
        p.nranges = nranges;
        p.spin_limit = ws.spin_limit;
        if (kpt == 4) k_sort_pass<KT, 4><<<tiles, GS_BLOCK, 0, s>>>(p);
        else if (kpt == 8) k_sort_pass<KT, 8><<<tiles, GS_BLOCK, 0, s>>>(p);
        else k_sort_pass<KT, 12><<<tiles, GS_BLOCK, 0, s>>>(p);
        GS_CUDA_CHECK();
    }
    return GSEVT_OK;
}

template int gs_launch_sort_t<uint32_t>(uint32_t *const keys[2], uint32_t *const vals[2], const uint32_t *count,
                                        uint32_t capacity, int bits, uint32_t max_keys, int kpt,
                                        const Workspace &ws, int *out_buf, cudaStream_t s, uint2 *ranges,
                                        uint32_t nranges);
