// Shared definitions of the gsevt CUDA library (sm_103a).
//
// Every translation unit is compiled with -fmad=false: a multiply followed by an add
// is rounded twice unless an explicit fmaf() is written, so the forward arithmetic
// reproduces the operation order of the CPU oracle bit for bit (keys, sort order,
// tile ranges, radii and images compare exactly).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "gsevt.h"

#define GS_BLOCK 256
// keys per thread of a sort pass (template instances 4, 8 and 12 exist)
#ifndef GS_SORT_KPT_TILES
#define GS_SORT_KPT_TILES 12
#endif
#ifndef GS_SORT_KPT_DEPTH
#define GS_SORT_KPT_DEPTH 12
#endif
#define GS_MAX_PASSES 8
#define GS_SPIN_LIMIT (1u << 22)
// cooperative sort (all passes of a sort in one launch, one block per SM): threads per
// block, keys per thread at most, keys per block at most, and the padded column count
// of its digit-major count table (an upper bound on the grid)
#define GS_COOP_THREADS 1024
#define GS_COOP_KPT 8
#define GS_COOP_TILE (GS_COOP_THREADS * GS_COOP_KPT)
#define GS_COOP_GP 160

// ----------------------------------------------------------------- exp ----------
// The blends evaluate a Gaussian's weight in base 2: with the conic (cx, cy, cz) scaled
// once per record to K = (-log2(e)/2 cx, -log2(e) cy, -log2(e)/2 cz), the exponent
// y = Kx dx^2 + Ky dx dy + Kz dy^2 is log2(e) times the published power
// -(cx dx^2 + cz dy^2)/2 - cy dx dy, and the weight is 2^y.  The FP32 operation order (three
// products for K, then gs_power2) is the CPU oracle's, so every decision and image bit is
// shared with it; so is the transmittance update T (1 - alpha), one fused multiply-add
// fmaf(-T, alpha, T) in the blends and the oracle.
#define GS_KHALF (-0x1.715476p-1f)  // -log2(e) / 2, rounded to FP32
#define GS_KFULL (-0x1.715476p+0f)  // -log2(e)

__host__ __device__ __forceinline__ uint32_t gs_float_bits(float x)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    union { float f; uint32_t u; } cv;
    cv.f = x;
    return cv.u;
#endif
}

__host__ __device__ __forceinline__ float gs_bits_float(uint32_t u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    union { uint32_t u; float f; } cv;
    cv.u = u;
    return cv.f;
#endif
}

// Deterministic 2^y for y <= 0: k = rint(y), r = y - k (exact, |r| <= 1/2), 2^r = 1 + r c(r)
// with c a degree-5 near-minimax polynomial (Lawson fit, oracle/fit_exp.py fit_exp2;
// Horner with fused multiply-adds) and an exact power-of-two scale: below one ulp of 2^y.
// The same value as or_exp2f in the CPU oracle for every float (which states it with
// rintf and a multiply by 2^k).  y below -126 (and NaN) is raised to -126: a weight of
// 2^-126 fails the blends' alpha test exactly as 0 would, one instruction cheaper than a
// branch.
//
// No conversion instruction (they issue at a fraction of the FP32 rate, and the blends
// evaluate this once per pixel and candidate): t = y + 1.5 2^23 lies in [2^23, 2^24),
// where the float spacing is 1, so the addition rounds y to the nearest integer, ties to
// even, exactly as rint; k = t - 1.5 2^23 is exact, and the low bits of t hold k in two's
// complement: bits(t) = bits(1.5 2^23) + k, whence bits(t) << 23 = k << 23 (mod 2^32;
// bits(1.5 2^23) has no set bit below bit 22).  The scale by 2^k is then an addition to
// the exponent field of p, which equals the product p 2^k while that product is normal:
// for y >= -126, k = -126 only with r >= 0, where p >= 1.  (For y > 0 the result is
// unspecified; every caller discards the weight of a positive exponent.)
__host__ __device__ __forceinline__ float gs_exp2f(float y)
{
    y = fmaxf(y, -126.0f);
    const float t = y + 0x1.8p23f;
    const float k = t - 0x1.8p23f;
    const float r = y - k;
    float p = 0x1.41fbb8p-13f;
    p = fmaf(p, r, 0x1.5f3e56p-10f);
    p = fmaf(p, r, 0x1.3b2d4ep-7f);
    p = fmaf(p, r, 0x1.c6aee8p-5f);
    p = fmaf(p, r, 0x1.ebfbdcp-3f);
    p = fmaf(p, r, 0x1.62e43p-1f);
    p = fmaf(p, r, 1.0f);
    return gs_bits_float(gs_float_bits(p) + (gs_float_bits(t) << 23));
}

// The base-2 exponent coefficients of a record's conic {cx, cy, cz, opacity} (opacity kept).
__host__ __device__ __forceinline__ float4 gs_log2_conic(float4 B)
{
    return make_float4(GS_KHALF * B.x, GS_KFULL * B.y, GS_KHALF * B.z, B.w);
}

// The base-2 exponent at pixel offset d = mean - pixel, dx (Kx dx + Ky dy) + Kz dy^2: two
// fused multiply-adds and three products (Kx dx is shared by the pixels of one column).
__host__ __device__ __forceinline__ float gs_power2(float4 K, float dx, float dy)
{
    return fmaf(fmaf(K.y, dy, K.x * dx), dx, (K.z * dy) * dy);
}

// ------------------------------------------------------------ workspace ---------
// Pair loss scalars.  With d = I_next - I_last, s = |d|, n = d / s and e the event
// frame: cross = d . e (|d| . |e| in unsigned mode), e2 = e . e, L = |n - e|.  The
// per-pixel image gradient is dL/dd = (g - n ndotg) / s with g = (n - e) / L
// (sign(d) (|n| - |e|) / L in unsigned mode) and ndotg = n . g = (1 - cross / s) / L.
struct LossScal {
    double s, cross, e2, L;
    float inv_s, ndotg, inv_L, pad;
};

struct Workspace {
    uint32_t *status;     // [0] status bits, [1] num keys, [2] last sort epoch, [4] sort epoch base,
                          // [5] number of visible (view, Gaussian) slots, [6] number of coarse
                          // (super-tile, slot) pairs, [7] fine-list region cursor
    int4 *bin;            // [num_vg] {touched, rect lo (x0 | y0<<16), rect hi, depth bits}
    float4 *rec;          // [num_vg][2] the blend record of each slot, 32 bytes:
                          // {mean x, mean y, depth, grey}, {conic x, y, z, opacity}
    float4 *recC;         // [num_vg] {r, g, b, 0} (channels == 3)
    float4 *gradA;        // [num_vg] dL/d{mean x, mean y, conic x, conic y}
    float4 *gradB;        // [num_vg] dL/d{conic z, opacity, grey or r, depth}
    float4 *gradC;        // [num_vg] dL/d{g, b, -, -} (channels == 3)
    uint32_t *vis_sums;   // [num_scan_blocks] visible slots per (view, block)
    uint32_t *vis_offs;   // [num_scan_blocks]
    uint32_t *dkeys[2];   // [num_vg] depth bits of the visible slots (depth sort)
    uint32_t *dvals[2];   // [num_vg] their (view, Gaussian) slots
    uint32_t *tsums;      // [sorted blocks] touched tiles per block of depth-sorted slots
    uint32_t *toffs;      // [sorted blocks]
    uint32_t *keys[2];    // [key_capacity] global tile id of each (tile, Gaussian) pair
    uint32_t *vals[2];    // [key_capacity] its (view, Gaussian) slot
    uint32_t *sort_hist;      // [GS_MAX_PASSES][256]; the cooperative sort's [256][GS_COOP_GP] + [256]
    uint32_t *sort_counter;   // [GS_MAX_PASSES]
    unsigned long long *sort_lookback;  // [sort tiles][256]  {epoch:32 | flag:2 | count:30}
    uint2 *ranges;        // [total_tiles]
    double *loss_part;    // [loss_blocks][4]
    LossScal *loss_scal;  // [num_pairs] norms of the pair loss and the per-pixel gradient factors
    uint32_t *loss_done;  // [num_pairs]
    double *xi_part;      // [num_scan_blocks][6] float pairs (hi, lo) of the block's twist sums
    double *xi;           // [num_views][6]
    // super-tile binning (batched tracker): 4x4-tile super-tiles, numbered per view
    uint32_t *csums;      // [sorted blocks] super-tiles touched per block of depth-sorted slots
    uint32_t *coffs;      // [sorted blocks]
    uint32_t *soffs;      // [num_views + 1] first super-tile of each view; [num_views] = total
    uint2 *sranges;       // [gs_super_bound] [start, end) of every super-tile in the sorted coarse pairs
    float4 *fcache;       // [num_vg][6] forward intermediates of each visible slot for the
                          // twist-only adjoint (frames with render pairs; else absent)
    size_t bytes;
    uint32_t spin_limit;  // polls of a bounded wait before it gives up (the layout's, or GS_SPIN_LIMIT)
    int depth_kpt;        // keys per thread of the onesweep depth sort (4, 8 or 12)
    int pair_kpt;         // keys per thread of the onesweep pair sorts (4, 8 or 12)
    int coop_ok;          // the cooperative sort may be used
};

// keys per thread of a tuning field: 4, 8 or 12 (anything else: the default)
inline int gs_kpt_choice(int32_t v, int dflt) { return (v == 4 || v == 8 || v == 12) ? (int)v : dflt; }

#define GS_WS_REGIONS 34
#define GS_FCACHE 6       // float4 words per slot in fcache
#define GS_SUPER 4   // tiles per super-tile side

__host__ __device__ inline size_t gs_align(size_t x) { return (x + 255) & ~(size_t)255; }

inline uint32_t gs_sort_tiles(uint32_t cap, int kpt) { return (cap + GS_BLOCK * kpt - 1) / (GS_BLOCK * kpt); }
inline uint32_t gs_sorted_blocks(const gsevt_layout &L) { return ((uint32_t)(L.num_vg > 0 ? L.num_vg : 1) + GS_BLOCK - 1) / GS_BLOCK; }
// look-back entries of the onesweep sorts: enough for the smallest keys-per-thread choice (4),
// so that a tuning change never needs a larger workspace
inline uint32_t gs_lookback_tiles(const gsevt_layout &L)
{
    uint32_t cap = L.key_capacity > 0 ? L.key_capacity : 1;
    uint32_t vg = L.num_vg > 0 ? (uint32_t)L.num_vg : 1;
    return std::max(gs_sort_tiles(cap, 4), gs_sort_tiles(vg, 4));
}
inline int gs_tile_bits(const gsevt_layout &L) { return L.sort_bits - 32; }
// number of super-tile ids: the layout's exact count, else an upper bound
// (ceil(tx/4) ceil(ty/4) <= floor(tx ty / 4) + 1 per view)
inline uint32_t gs_super_bound(const gsevt_layout &L)
{
    if (L.super_tiles > 0) return (uint32_t)L.super_tiles;
    return (uint32_t)(L.total_tiles > 0 ? L.total_tiles : 0) / 4 + (uint32_t)(L.num_views > 0 ? L.num_views : 0) + 1;
}
inline int gs_super_bits(const gsevt_layout &L)
{
    uint32_t n = gs_super_bound(L), b = 1;
    while ((1u << b) < n && b < 31) ++b;
    return (int)b;
}
inline int gs_tile_sort_buffer(const gsevt_layout &L) { return ((gs_tile_bits(L) + 7) / 8) & 1; }

// Reserves the look-back epochs of a sort's passes: status[4] = first epoch of this sort,
// status[2] = last epoch used so far.  One thread, before any pass of the sort runs.
__device__ __forceinline__ void gs_sort_reserve_epochs(uint32_t *status, int passes)
{
    const uint32_t e = status[2];
    status[4] = e + 1;
    status[2] = e + (uint32_t)passes;
}

// Carves the workspace in a fixed order; with base == nullptr it only sizes it.
inline Workspace gs_carve(const gsevt_layout &L, void *base)
{
    Workspace w;
    char *p = (char *)base;
    size_t off = 0;
    auto take = [&](size_t bytes) -> void * {
        void *r = base ? (void *)(p + off) : nullptr;
        off += gs_align(bytes > 0 ? bytes : 1);
        return r;
    };
    size_t vg = (size_t)(L.num_vg > 0 ? L.num_vg : 1);
    bool rgb = L.channels == 3;
    w.status = (uint32_t *)take(64);
    w.bin = (int4 *)take(vg * 16);
    w.rec = (float4 *)take(vg * 32);
    w.recC = rgb ? (float4 *)take(vg * 16) : nullptr;
    w.gradA = (float4 *)take(vg * 16);
    w.gradB = (float4 *)take(vg * 16);
    w.gradC = rgb ? (float4 *)take(vg * 16) : nullptr;
    w.vis_sums = (uint32_t *)take((size_t)L.num_scan_blocks * 4);
    w.vis_offs = (uint32_t *)take((size_t)L.num_scan_blocks * 4);
    w.dkeys[0] = (uint32_t *)take(vg * 4);
    w.dkeys[1] = (uint32_t *)take(vg * 4);
    w.dvals[0] = (uint32_t *)take(vg * 4);
    w.dvals[1] = (uint32_t *)take(vg * 4);
    w.tsums = (uint32_t *)take((size_t)gs_sorted_blocks(L) * 4);
    w.toffs = (uint32_t *)take((size_t)gs_sorted_blocks(L) * 4);
    size_t cap = (size_t)(L.key_capacity > 0 ? L.key_capacity : 1);
    w.keys[0] = (uint32_t *)take(cap * 4);
    w.keys[1] = (uint32_t *)take(cap * 4);
    w.vals[0] = (uint32_t *)take(cap * 4);
    w.vals[1] = (uint32_t *)take(cap * 4);
    w.sort_hist = (uint32_t *)take((size_t)std::max(GS_MAX_PASSES, GS_COOP_GP + 1) * 256 * 4);
    w.sort_counter = (uint32_t *)take(GS_MAX_PASSES * 4);
    w.sort_lookback = (unsigned long long *)take((size_t)gs_lookback_tiles(L) * 256 * 8);
    w.ranges = (uint2 *)take((size_t)L.total_tiles * 8);
    w.loss_part = (double *)take((size_t)L.loss_blocks * 4 * 8);
    w.loss_scal = (LossScal *)take((size_t)L.num_pairs * sizeof(LossScal));
    w.loss_done = (uint32_t *)take((size_t)L.num_pairs * 4);
    w.xi_part = (double *)take((size_t)L.num_scan_blocks * 6 * 8);
    w.xi = (double *)take((size_t)L.num_views * 6 * 8);
    w.csums = (uint32_t *)take((size_t)gs_sorted_blocks(L) * 4);
    w.coffs = (uint32_t *)take((size_t)gs_sorted_blocks(L) * 4);
    w.soffs = (uint32_t *)take((size_t)(L.num_views + 1) * 4);
    w.sranges = (uint2 *)take((size_t)gs_super_bound(L) * 8);
    w.fcache = (L.num_pairs > 0 && !rgb) ? (float4 *)take(vg * GS_FCACHE * 16) : nullptr;
    w.bytes = off;
    w.spin_limit = L.spin_limit ? L.spin_limit : GS_SPIN_LIMIT;
    w.depth_kpt = gs_kpt_choice(L.tuning.depth_sort_kpt, GS_SORT_KPT_DEPTH);
    w.pair_kpt = gs_kpt_choice(L.tuning.pair_sort_kpt, GS_SORT_KPT_TILES);
    w.coop_ok = L.tuning.coop_sort != 1;
    return w;
}

// ------------------------------------------------------------- helpers ----------
// True once a bounded wait of this frame's sorts ran out (GSEVT_STATUS_SORT_TIMEOUT).
// The kernels that consume a sort's order then do nothing, so an index that a sort left
// unwritten is never followed.  The word only changes inside the sort kernels, which
// precede every reader on the stream, so all threads of a block read the same value.
__device__ __forceinline__ bool gs_sort_timed_out(const uint32_t *status)
{
    return (__ldcg(status) & GSEVT_STATUS_SORT_TIMEOUT) != 0u;
}

__device__ __forceinline__ int gs_find_map(const gsevt_map *maps, int num_maps, int block)
{
    int m = 0;
    for (int i = 1; i < num_maps; ++i)
        if (maps[i].block_offset <= block) m = i;
    return m;
}

// view containing global tile id `tile` (views ordered by tile_offset)
__device__ __forceinline__ int gs_find_view_by_tile(const gsevt_view *views, int num_views, int tile)
{
    int lo = 0, hi = num_views - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (views[mid].tile_offset <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Unevaluated float pair hi + lo, added with Knuth's TwoSum (exact error of each FP32
// addition; every operation rounds separately because the library is built with
// -fmad=false): about 48 significant bits at FP32 cost.
struct FP2 {
    float hi = 0.0f, lo = 0.0f;
    __device__ void add(float xh, float xl)
    {
        const float t = hi + xh, z = t - hi;
        const float e = (hi - (t - z)) + (xh - z);
        hi = t;
        lo = lo + (e + xl);
        const float u = hi + lo;  // renormalise
        lo = lo - (u - hi);
        hi = u;
    }
    __device__ void add(const FP2 &x) { add(x.hi, x.lo); }
};

// warp sum of one float per lane as a float pair, combined in lane order (every lane
// gets the same result)
__device__ __forceinline__ FP2 warp_sum_fp2(float v)
{
    FP2 sm;
    sm.hi = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float hi = __shfl_xor_sync(0xffffffffu, sm.hi, o), lo = __shfl_xor_sync(0xffffffffu, sm.lo, o);
        FP2 other;
        other.hi = hi;
        other.lo = lo;
        FP2 a = ((threadIdx.x & o) == 0) ? sm : other;
        const FP2 b = ((threadIdx.x & o) == 0) ? other : sm;
        a.add(b);
        sm = a;
    }
    return sm;
}

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

#define GS_CUDA_CHECK()                                         \
    do {                                                        \
        cudaError_t _e = cudaGetLastError();                    \
        if (_e != cudaSuccess) return GSEVT_ERR_CUDA;           \
    } while (0)

// First statement of every entry point that enqueues work: clears an error that an
// earlier, unrelated runtime call of the caller left pending, so that GS_CUDA_CHECK
// reports only failures of this call's own launches and copies.  (A sticky error, which
// means the context is lost, is still reported by the next check.)
#define GS_ENTRY() ((void)cudaGetLastError())

// Prepares the cooperative sort on the current device (sort.cu); outside stream capture.
void gs_sort_prepare();

// Super-tile binning fused into the cooperative depth sort (sort.cu, batched tracker).
struct GsCoarseBin {
    const gsevt_view *views;
    int num_views;
    const int4 *bin;       // per slot {tiles touched, rect lo, rect hi, depth bits}
    uint32_t *soffs;       // [num_views + 1] first super-tile of each view
    uint2 *sranges;        // [super_bound] [start, end) of each super-tile's list
    uint32_t *cvals;       // [capacity] the super-tile lists (slots)
    uint32_t capacity;     // pair capacity (fine and coarse)
    uint32_t super_bound;  // super-tile ids available (<= 256)
    uint32_t *rec_a;       // [capacity] scratch: each pair's super-tile id and rank in its warp
    uint32_t *rec_b;       // [capacity] scratch: each pair's slot
    int enabled;
};
// Visible-slot compaction fused into the first pass of the cooperative depth sort: the
// pass reads every (view, Gaussian) slot's bin record itself, keeps the visible ones in
// slot order, clears their gradient records and writes N_vis to status[5].
struct GsCompact {
    const gsevt_view *views;
    int num_views;
    const gsevt_map *maps;
    const int4 *bin;
    float4 *gradA, *gradB, *gradC;  // gradC null without RGB
    uint32_t num_scan_blocks;
    int enabled;
};
// True when the cooperative sort runs a depth sort of this capacity on the current device
// (and, for the compaction, of this many scan blocks).
bool gs_coop_depth_sort(uint32_t capacity, uint32_t num_scan_blocks);
// Stable depth sort of the N_vis visible slots (count in status[5]) in dkeys/dvals, the
// result in buffer 0.  With `cmp` (only when gs_coop_depth_sort holds) the launch also
// compacts the visible slots itself.  With `bin` (super_bound <= 256) and a frame the cooperative sort
// takes, the same launch also writes the super-tile lists, their ranges, soffs and the
// pair counts (status[1], status[6]), and *binned is set.
int gs_launch_depth_sort(const Workspace &ws, uint32_t capacity, const GsCompact *cmp, const GsCoarseBin *bin,
                         bool *binned, cudaStream_t s);
