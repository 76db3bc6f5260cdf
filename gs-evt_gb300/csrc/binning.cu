// Key scan, key duplication and tile ranges.
//
// k_scan_blocks: exclusive scan of the per-(view, block) touched-tile sums written by
//   the preprocess kernel (one block; at most a few hundred thousand entries), total
//   key count into status[1], overflow flag when it exceeds the key capacity.
// k_duplicate: per (view, block) of 256 Gaussians, block-local exclusive scan of the
//   touched counts plus the block offset; each visible Gaussian writes one
//   (key, value) per tile of its rect in row-major order:
//   key = (global tile << 32) | float bits of depth, value = (view, Gaussian) slot.
//   The same pass zeroes the slot's gradient records for the adjoint.
// k_ranges: [start, end) of every global tile in the sorted keys.
#include "common.cuh"

namespace {

__global__ void __launch_bounds__(1024) k_scan_blocks(const uint32_t *sums, uint32_t *offs, int n,
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
    // Hillis-Steele inclusive scan over the 1024 partial sums
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
        status[1] = (uint32_t)min(tot, 0xffffffffull);
        if (tot > capacity) atomicOr(&status[0], GSEVT_STATUS_KEY_OVERFLOW);
    }
}

struct DupParams {
    const gsevt_view *views;
    int num_views;
    const gsevt_map *maps;
    Workspace ws;
    uint32_t capacity;
    int rgb;
};

__device__ __forceinline__ int find_view_by_sb(const gsevt_view *views, int num_views, int sb)
{
    int lo = 0, hi = num_views - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (views[mid].sb_offset <= sb) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(GS_BLOCK) k_duplicate(DupParams p)
{
    __shared__ uint32_t wtot[GS_BLOCK / 32];
    int sb = blockIdx.x;
    int v = find_view_by_sb(p.views, p.num_views, sb);
    const gsevt_view &V = p.views[v];
    int n = p.maps[V.map].n;
    int gb = sb - V.sb_offset;
    int g = gb * GS_BLOCK + threadIdx.x;
    int4 bin = make_int4(0, 0, 0, 0);
    size_t vg = (size_t)V.vg_offset + g;
    if (g < n) bin = p.ws.bin[vg];
    uint32_t cnt = (uint32_t)bin.x;
    // block exclusive scan of cnt
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wtot[w] = inc;
    __syncthreads();
    uint32_t wbase = 0;
    for (int i = 0; i < w; ++i) wbase += wtot[i];
    uint32_t off = p.ws.scan_offs[sb] + wbase + inc - cnt;
    if (cnt == 0) return;
    p.ws.gradA[vg] = make_float4(0, 0, 0, 0);
    p.ws.gradB[vg] = make_float4(0, 0, 0, 0);
    if (p.rgb) p.ws.gradC[vg] = make_float4(0, 0, 0, 0);
    int x0 = bin.y & 0xffff, y0 = (bin.y >> 16) & 0xffff;
    int x1 = bin.z & 0xffff, y1 = (bin.z >> 16) & 0xffff;
    unsigned long long db = (unsigned long long)(uint32_t)bin.w;
    uint32_t k = off;
    for (int y = y0; y < y1; ++y)
        for (int x = x0; x < x1; ++x) {
            if (k < p.capacity) {
                unsigned long long tile = (unsigned long long)(uint32_t)(V.tile_offset + y * V.tiles_x + x);
                p.ws.keys[0][k] = (tile << 32) | db;
                p.ws.vals[0][k] = (uint32_t)vg;
            }
            ++k;
        }
}

__global__ void k_ranges(const unsigned long long *keys, const uint32_t *status, uint32_t capacity,
                         uint2 *ranges)
{
    uint32_t K = min(status[1], capacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
        uint32_t t = (uint32_t)(keys[i] >> 32);
        if (i == 0 || (uint32_t)(keys[i - 1] >> 32) != t) ranges[t].x = i;
        if (i == K - 1 || (uint32_t)(keys[i + 1] >> 32) != t) ranges[t].y = i + 1;
    }
}

}  // namespace

int gs_launch_scan(const gsevt_frame *f, const Workspace &ws, cudaStream_t s)
{
    if (f->L.num_scan_blocks <= 0) {
        cudaMemsetAsync(ws.status + 1, 0, 4, s);
        GS_CUDA_CHECK();
        return GSEVT_OK;
    }
    k_scan_blocks<<<1, 1024, 0, s>>>(ws.scan_sums, ws.scan_offs, f->L.num_scan_blocks, ws.status,
                                      f->L.key_capacity);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

int gs_launch_duplicate(const gsevt_frame *f, const Workspace &ws, cudaStream_t s)
{
    if (f->L.num_scan_blocks <= 0) return GSEVT_OK;
    DupParams p;
    p.views = f->views;
    p.num_views = f->L.num_views;
    p.maps = f->maps;
    p.ws = ws;
    p.capacity = f->L.key_capacity;
    p.rgb = f->L.channels == 3;
    k_duplicate<<<f->L.num_scan_blocks, GS_BLOCK, 0, s>>>(p);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

int gs_launch_ranges(const gsevt_frame *f, const Workspace &ws, const unsigned long long *sorted_keys,
                     uint32_t max_keys, cudaStream_t s)
{
    cudaMemsetAsync(ws.ranges, 0, (size_t)f->L.total_tiles * sizeof(uint2), s);
    GS_CUDA_CHECK();
    if (max_keys == 0) return GSEVT_OK;
    int blocks = (int)std::min<uint32_t>((max_keys + 255) / 256, 152u * 16u);
    k_ranges<<<blocks, 256, 0, s>>>(sorted_keys, ws.status, f->L.key_capacity, ws.ranges);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}
