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
#include "common.cuh"

template <typename KT>
int gs_launch_sort_t(KT *const keys[2], uint32_t *const vals[2], const uint32_t *count, uint32_t capacity,
                     int bits, uint32_t max_keys, const Workspace &ws, int *out_buf, cudaStream_t s);

namespace {

// exclusive scan of n block sums (one block of 1024 threads); total into *total and an
// overflow flag when the total exceeds `capacity` (0: no check)
__global__ void __launch_bounds__(1024) k_scan_blocks(const uint32_t *sums, uint32_t *offs, int n, uint32_t *total,
                                                      uint32_t *status, uint32_t capacity)
{
    __shared__ unsigned long long part[1024];
    int t = threadIdx.x;
    int per = (n + 1023) / 1024;
    int b = t * per, e = min(n, b + per);
    unsigned long long s = 0;
    for (int i = b; i < e; ++i) s += sums[i];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        unsigned long long v = t >= o ? part[t - o] : 0ull;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    unsigned long long run = t > 0 ? part[t - 1] : 0ull;
    for (int i = b; i < e; ++i) {
        offs[i] = (uint32_t)min(run, 0xffffffffull);
        run += sums[i];
    }
    if (t == 1023) {
        unsigned long long tot = part[1023];
        *total = (uint32_t)min(tot, 0xffffffffull);
        if (capacity && tot > capacity) atomicOr(&status[0], GSEVT_STATUS_KEY_OVERFLOW);
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
    if (vis) {
        p.ws.dkeys[0][c] = (uint32_t)bin.w;
        p.ws.dvals[0][c] = (uint32_t)vg;
    }
}

// tiles touched per block of 256 depth-sorted visible slots
__global__ void __launch_bounds__(GS_BLOCK) k_sorted_sums(BinParams p, const uint32_t *sorted_vals)
{
    __shared__ uint32_t wsum[GS_BLOCK / 32];
    const uint32_t nvis = p.ws.status[5];
    const uint32_t i = blockIdx.x * GS_BLOCK + threadIdx.x;
    uint32_t cnt = 0;
    if (i < nvis) cnt = (uint32_t)p.ws.bin[sorted_vals[i]].x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < GS_BLOCK / 32; ++w) t += wsum[w];
        p.ws.tsums[blockIdx.x] = t;
    }
}

// Warp-cooperative duplication: each warp expands the pairs of its 32 depth-sorted slots
// into one contiguous output range, lane k writing pair k, k + 32, ... of that range
// (coalesced); the owning slot of a pair is found by a shuffle binary search over the
// warp's exclusive prefix of tile counts.
__global__ void __launch_bounds__(GS_BLOCK) k_duplicate(BinParams p, const uint32_t *sorted_vals)
{
    __shared__ uint32_t wtot[GS_BLOCK / 32];
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
        p.ws.gradA[vg] = make_float4(0, 0, 0, 0);
        p.ws.gradB[vg] = make_float4(0, 0, 0, 0);
        if (p.rgb) p.ws.gradC[vg] = make_float4(0, 0, 0, 0);
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

__global__ void k_ranges(const uint32_t *keys, const uint32_t *status, uint32_t capacity, uint2 *ranges)
{
    uint32_t K = min(status[1], capacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
        uint32_t t = keys[i];
        if (i == 0 || keys[i - 1] != t) ranges[t].x = i;
        if (i == K - 1 || keys[i + 1] != t) ranges[t].y = i + 1;
    }
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
    return p;
}

}  // namespace

// After preprocess: visible-slot compaction, depth sort, key offsets in depth order.
// Leaves the key count in status[1] (and flags overflow) and N_vis in status[5].
int gs_launch_depth_order(const gsevt_frame *f, const Workspace &ws, cudaStream_t s)
{
    const gsevt_layout &L = f->L;
    const uint32_t nb = gs_sorted_blocks(L);
    if (L.num_scan_blocks <= 0 || L.num_vg <= 0) {
        cudaMemsetAsync(ws.status + 1, 0, 4, s);
        cudaMemsetAsync(ws.status + 5, 0, 4, s);
        GS_CUDA_CHECK();
        return GSEVT_OK;
    }
    BinParams p = make_params(f, ws);
    k_scan_blocks<<<1, 1024, 0, s>>>(ws.vis_sums, ws.vis_offs, L.num_scan_blocks, ws.status + 5, ws.status, 0);
    k_compact<<<L.num_scan_blocks, GS_BLOCK, 0, s>>>(p);
    GS_CUDA_CHECK();
    int buf = 0;
    uint32_t *dk[2] = {ws.dkeys[0], ws.dkeys[1]};
    uint32_t *dv[2] = {ws.dvals[0], ws.dvals[1]};
    int st = gs_launch_sort_t<uint32_t>(dk, dv, ws.status + 5, (uint32_t)L.num_vg, 32, (uint32_t)L.num_vg, ws, &buf, s);
    if (st) return st;
    if (buf != 0) return GSEVT_ERR_ARG;  // 4 passes: the result is back in buffer 0
    k_sorted_sums<<<nb, GS_BLOCK, 0, s>>>(p, ws.dvals[0]);
    k_scan_blocks<<<1, 1024, 0, s>>>(ws.tsums, ws.toffs, (int)nb, ws.status + 1, ws.status, L.key_capacity);
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
    int st = gs_launch_sort_t<uint32_t>(k, v, ws.status + 1, L.key_capacity, gs_tile_bits(L), max_keys, ws, &buf, s);
    if (st) return st;
    if (buf != gs_tile_sort_buffer(L)) return GSEVT_ERR_ARG;
    int blocks = (int)std::min<uint32_t>((max_keys + 255) / 256, 152u * 16u);
    k_ranges<<<blocks, 256, 0, s>>>(ws.keys[buf], ws.status, L.key_capacity, ws.ranges);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}
