// Per-tile front-to-back alpha blending and its adjoint.
//
// One block per 16x16 tile (global tile ids cover every view of the frame, so views of
// different sizes share the launch): 256 threads, one pixel each, or 128 threads with two
// pixels each (the grey forward and the tracker adjoint of the batched step, below).  The
// tile's depth-sorted Gaussians are staged through shared memory in batches of one record
// per thread (32 bytes each, or 48 with RGB); a batch is loaded with cp.async (16-byte
// global->shared copies that bypass registers) while the block is still blending the
// previous one.  A pixel
// stops when its transmittance would fall below 1e-4; the block stops when
// __syncthreads_count says every pixel has stopped.
//
// Blending (the published 3DGS rule): alpha = min(0.99, o * exp(power)), skipped when
// power > 0 or alpha < 1/255; C += c alpha T (one fused multiply-add); T *= 1 - alpha.
// exp(power) is evaluated in base 2 as gs_exp2f(y) with y = gs_power2(K, d) = log2(e) power
// (K the record's conic scaled by gs_log2_conic), so the per-pixel decisions and sums are
// bit-identical to the CPU oracle, which uses the same operation order.
//
// Adjoint: the same front-to-back traversal with the same decisions (no per-pixel
// contributor lists are stored); with P_i the running prefix of c alpha T up to and
// including Gaussian i and C the stored pixel value (Gaussians plus T_final bg),
//   dC/dalpha_i = T_i c_i - (C - P_i) / (1 - alpha_i).
// The power's gradient enters the 2D mean and conic gradients linearly in the conic, so a
// pixel contributes the five moments dpow (dx, dy, dx^2, dx dy, dy^2) and the conic is
// applied once per Gaussian and tile.  Per-Gaussian contributions are reduced across the
// warp in FP32 (shuffles; the tracker adjoint reduces two candidates' terms per butterfly),
// summed per tile in shared memory and added to the global per-slot gradients once per
// tile.
//
// Warp-level culling (both directions): each batch Gaussian gets a conservative pixel
// box and quadratic form of its alpha support (gauss_box); a warp ballots which of them
// reach its pixel block, 8x4 or 8x8 (box overlap, then the exact ellipse-rectangle test of
// ellipse_hits) and walks only those, in depth order, two at a time.  Gaussians that fail
// both cannot pass the per-pixel alpha test, so the decisions and results are unchanged.
// Every lane evaluates each candidate; the per-pixel decisions are predicates, not
// divergent branches.  The default forms of the grey forward (k_blend_fwd_px2) and of the
// tracker adjoint (k_blend_bwd_px2) give each lane two pixels (128 threads and 8x8-pixel
// warps per tile): the two pixels share the record loads and loop control, and in the
// adjoint one warp reduction serves 64 pixels.
//
// Staging (gsevt_tuning.blend_staging): either every thread copies its candidate's 32-byte
// record with two 16-byte cp.async, or (the grey tracker blends, staging 2) one warp stages
// the whole batch with TMA: the records form a 2-D tensor of num_vg rows of 8 floats, and
// each cp.async.bulk.tensor ... tile::gather4 copies four rows chosen by slot id into one
// 128-byte aligned group of the batch buffer, completing on the buffer's mbarrier (every
// wait on it is bounded; one that runs out sets GSEVT_STATUS_STAGE_TIMEOUT, and a block
// that stops early still waits, again bounded, for the copies it issued).
#include <cuda.h>

#include <atomic>
#include <cstring>

#include "common.cuh"

namespace {

struct BlendParams {
    const gsevt_view *views;
    int num_views;
    const gsevt_pair *pairs;
    Workspace ws;
    const uint32_t *vals;  // sorted values (view, Gaussian) slots
    int rgb;
    int total_pixels;
    float *image, *final_T, *depth, *alpha;
    int32_t *n_contrib, *n_touched;
    const float *dL_dimage, *dL_ddepth, *dL_dalpha;
    int stage_all_warps;  // TMA staging: every warp issues its candidates' copies (staging 3)
    // persistent launches: the tiles in the order blocks take them, and the queue head
    const uint32_t *order;
    uint32_t *queue;
    int num_tiles;
    int ordered;  // two-pixel blends: block b takes tile order[b] (longest lists first)
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// One staged Gaussian: the slot's 32-byte blend record.
struct Rec {
    float4 A;  // {mean x, mean y, depth, grey}
    float4 B;  // {conic x, y, z, opacity}
};

template <bool RGB> struct alignas(128) Batch {
    Rec r[GS_BLOCK];  // first member: 128-byte aligned for the tensor-copy groups
    float4 C[RGB ? GS_BLOCK : 1];
    float4 box[GS_BLOCK];  // {xmin, xmax, ymin, ymax}: outside it the Gaussian fails the alpha test
    float4 ell[GS_BLOCK];  // {a, b, c, -tau}: quadratic form of the alpha support and its bound
    uint32_t id[GS_BLOCK];
};

// Conservative pixel box of a Gaussian's alpha support.  A pixel blends the Gaussian
// only if alpha = min(0.99, o exp(power)) >= 1/255, i.e. -power <= tau = ln(255 o).  With
// M the conic, -power = d^T M d / 2 in exact arithmetic; the FP32 evaluation (gs_power2:
// three products for K, three in the exponent and two fused multiply-adds) deviates by
// less than 1e-6 tr(M) |d|^2, so
// every pixel that can pass satisfies Q(d) = d^T (M/2 - 1e-6 tr(M) I) d <= tau + 1e-4 (the
// slack also covers gs_exp2f's and logf's rounding).  The box of that ellipse, widened by 0.1 % + 0.5 px,
// therefore never excludes a pixel whose per-pixel test would pass, so culling against it
// leaves every blending decision - and the result bits - unchanged.
// Also returns, through *ell, Q's coefficients {a, b, c} (Q = a dx^2 + 2 b dx dy + c dy^2;
// all zero when Q is ill-conditioned, which disables the ellipse test) and -tau with tau
// = ln(255 o) (1 + 1e-4) + 1e-3 (1e30 when no pixel can pass), the ellipse test's bound.
__device__ __forceinline__ float4 gauss_box(float4 A, float4 B, float4 *ell)
{
    const float o = B.w;
    *ell = make_float4(0.0f, 0.0f, 0.0f, 1e30f);
    if (!(o >= (1.0f / 255.0f) * 0.999f)) return make_float4(1e30f, -1e30f, 1e30f, -1e30f);
    const float tau = logf(255.0f * o) * 1.0001f + 1e-3f;
    ell->w = -tau;
    const float g = 1e-6f * (fabsf(B.x) + fabsf(B.z));
    const float a = 0.5f * B.x - g, b = 0.5f * B.y, c = 0.5f * B.z - g;
    const float det = a * c - b * b;
    if (!(a > 0.0f && c > 0.0f && det > 0.0f && tau > -1e29f && tau < 1e29f))
        return make_float4(-1e30f, 1e30f, -1e30f, 1e30f);  // no culling
    // |b| <= 0.995 sqrt(ac): the FP32 rounding of Q stays below 1.4e-4 Q (see ellipse_hits)
    if (b * b <= 0.99f * (a * c)) { ell->x = a; ell->y = b; ell->z = c; }
    const float hx = sqrtf(fmaxf(tau, 0.0f) * c / det) * 1.001f + 0.5f;
    const float hy = sqrtf(fmaxf(tau, 0.0f) * a / det) * 1.001f + 0.5f;
    return make_float4(A.x - hx, A.x + hx, A.y - hy, A.y + hy);
}

// Does the Gaussian's support ellipse Q(mean - p) <= tau reach the pixel rectangle
// [x0, x1] x [y0, y1]?  Exact minimum of the convex Q over the rectangle: zero when the
// mean is inside, else on an edge that faces the mean (at most two), where the
// one-dimensional minimum is clamped to the edge.  Any pixel that passes the alpha test
// has Q <= tau, so min Q <= tau; the FP32 value computed here exceeds min Q by at most
// 1.4e-4 Q (|b| <= 0.995 sqrt(ac) bounds a dx^2 + c dy^2 by 400 Q) plus a second-order
// term from the rounded edge minimiser, both far below the slack of the comparison
// (tau * 1.001 + 0.01).  So this never rejects a Gaussian a pixel of the rectangle blends.
// Both edge minima are evaluated and selected (no divergent branches).
__device__ __forceinline__ bool ellipse_hits(float mx, float my, float4 E, float x0, float x1, float y0, float y1)
{
    const bool inx = mx >= x0 && mx <= x1, iny = my >= y0 && my <= y1;
    const float a = E.x, b = E.y, c = E.z;
    // the x-facing edge
    const float dxa = mx - (mx < x0 ? x0 : x1);
    const float dya = fminf(fmaxf(-__fdividef(b * dxa, c), my - y1), my - y0);
    const float qa = (a * dxa) * dxa + 2.0f * ((b * dxa) * dya) + (c * dya) * dya;
    // the y-facing edge
    const float dyb = my - (my < y0 ? y0 : y1);
    const float dxb = fminf(fmaxf(-__fdividef(b * dyb, a), mx - x1), mx - x0);
    const float qb = (a * dxb) * dxb + 2.0f * ((b * dxb) * dyb) + (c * dyb) * dyb;
    const float q = fminf(inx ? 1e30f : qa, iny ? 1e30f : qb);
    return (inx && iny) || q <= -E.w * 1.001f + 0.01f;
}

// Which of the batch's candidates c0 + lane reach the warp's pixel rectangle (box overlap
// and the ellipse test, both evaluated for every lane).  BT: a batch type with the
// members r, box and ell.
template <class BT>
__device__ __forceinline__ bool warp_hit(const BT &cur, int c0, int n, int lane, float sx0, float sx1,
                                         float sy0, float sy1)
{
    const int ci = min(c0 + lane, n - 1);
    const float4 bx = cur.box[ci], A = cur.r[ci].A;
    const bool box = bx.y >= sx0 && bx.x <= sx1 && bx.w >= sy0 && bx.z <= sy1;
    const bool ell = ellipse_hits(A.x, A.y, cur.ell[ci], sx0, sx1, sy0, sy1);
    return (c0 + lane < n) & box & ell;
}

// Issue the copies of batch `r` of the tile range into buffer `buf`.
template <bool RGB>
__device__ __forceinline__ void load_batch(const BlendParams &p, Batch<RGB> &buf, uint2 range, int r)
{
    uint32_t idx = range.x + (uint32_t)r * GS_BLOCK + threadIdx.x;
    if (idx < range.y) {
        uint32_t vg = __ldg(p.vals + idx);
        buf.id[threadIdx.x] = vg;
        cp_async16(&buf.r[threadIdx.x].A, p.ws.rec + 2 * (size_t)vg);
        cp_async16(&buf.r[threadIdx.x].B, p.ws.rec + 2 * (size_t)vg + 1);
        if (RGB) cp_async16(&buf.C[threadIdx.x], p.ws.recC + vg);
    }
    cp_async_commit();
}

// ---- TMA staging ----
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *m, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(m)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect(uint64_t *m, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(m)), "r"(bytes) : "memory");
}

// Bounded wait for the phase of parity `parity` to complete; false when `limit` polls ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *m, uint32_t parity, uint32_t limit)
{
    const uint32_t a = smem_addr(m);
    for (uint32_t i = 0; i <= limit; ++i) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(ok) : "r"(a), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

// Four rows (r0..r3) of the 2-D record tensor, x = 0, into 128 contiguous bytes at dst.
__device__ __forceinline__ void tma_gather4(void *dst, const CUtensorMap *tm, uint32_t r0, uint32_t r1, uint32_t r2,
                                            uint32_t r3, uint64_t *m)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cta.global.tile::gather4.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
                 ::"r"(smem_addr(dst)), "l"(tm), "r"(0), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(smem_addr(m))
                 : "memory");
}

// Stages batch r of the tile range into buf with tile::gather4 copies, called by every
// thread.  The issuing warps (warp 0 alone with staging 2; every warp for its own 32
// candidates with staging 3) give each lane a group g of four candidates: the lane reads
// their slot ids, stores them in buf.id, and (after the warp's lane 0 has announced the
// warp's bytes on the mbarrier) copies their four records with one gather4 into the
// 128-byte group buf.r[4g .. 4g + 3].  Rows past the range repeat the batch's first slot
// (copied but never read); an issuing warp without rows still arrives, with no bytes.
template <bool RGB>
__device__ __forceinline__ void tma_load_batch(const BlendParams &p, Batch<RGB> &buf, uint2 range, int r,
                                               uint64_t *mbar, const CUtensorMap *tm)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (!p.stage_all_warps && w != 0) return;
    const uint32_t base = range.x + (uint32_t)r * GS_BLOCK;
    const uint32_t n = min((uint32_t)GS_BLOCK, range.y - base);  // >= 1
    const uint32_t groups = (n + 3) / 4;
    // this warp's groups: [g0, g1)
    const uint32_t g0 = p.stage_all_warps ? 8u * (uint32_t)w : 0u;
    const uint32_t g1 = min(groups, p.stage_all_warps ? g0 + 8u : 64u);
    const uint32_t first = __ldg(p.vals + base);
    uint32_t rows[2][4];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t g = g0 + (uint32_t)(lane + 32 * h);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t c = 4 * g + (uint32_t)k;
            const bool own = g < g1 && c < n;
            rows[h][k] = own ? __ldg(p.vals + base + c) : first;
            if (own) buf.id[c] = rows[h][k];
        }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive_expect(mbar, (g1 > g0 ? g1 - g0 : 0u) * 128u);
    __syncwarp();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t g = g0 + (uint32_t)(lane + 32 * h);
        if (g < g1) tma_gather4(&buf.r[4 * g], tm, rows[h][0], rows[h][1], rows[h][2], rows[h][3], mbar);
    }
}

// Before a block exits: wait (bounded) for the batch it issued but did not consume (at
// most one, batch `waited`, when the block stopped early), so that no tensor copy still
// targets its shared memory.
__device__ __forceinline__ void tma_drain(uint64_t *mbar, uint32_t &phase, int issued, int waited, uint32_t limit,
                                          uint32_t *status)
{
    if (issued > waited) {
        const int b = waited & 1;
        if (!mbar_wait(&mbar[b], (phase >> b) & 1u, limit) && threadIdx.x == 0)
            atomicOr(status, GSEVT_STATUS_STAGE_TIMEOUT);
        phase ^= 1u << b;
    }
}

// Pixel of thread t: warps tile the 16x16 tile as 2 x 4 blocks of 8x4 pixels, so a warp's
// footprint is nearly square (fewer Gaussians overlap it than a 16x2 strip).
__device__ __forceinline__ void warp_pixel(int tid, int tx, int ty, int &px, int &py, float &sx0, float &sx1,
                                           float &sy0, float &sy1)
{
    const int w = tid >> 5, l = tid & 31;
    const int bx = tx * GSEVT_TILE + (w & 1) * 8, by = ty * GSEVT_TILE + (w >> 1) * 4;
    px = bx + (l & 7);
    py = by + (l >> 3);
    sx0 = (float)bx;
    sx1 = (float)(bx + 7);
    sy0 = (float)by;
    sy1 = (float)(by + 3);
}

// One candidate of the forward blend for one lane.  Every lane evaluates it and the
// decisions are predicates (selects instead of divergent branches; stopped lanes change
// nothing).  A candidate is skipped when y > 0 or alpha < 1/255; the pixel stops
// before a candidate that would take T below 1e-4.
template <bool EXTRAS, bool RGB>
__device__ __forceinline__ void fwd_candidate(const Batch<RGB> &cur, const BlendParams &p, int j, int r, float pxf,
                                              float pyf, float &T, float &C0, float &C1, float &C2, float &D,
                                              float &Aacc, int &last, bool &done)
{
    const float4 A = cur.r[j].A, B = cur.r[j].B;
    const float dx = A.x - pxf, dy = A.y - pyf;
    const float y = gs_power2(gs_log2_conic(B), dx, dy);
    const float alpha = fminf(0.99f, B.w * gs_exp2f(y));
    const float test_T = fmaf(-T, alpha, T);  // T (1 - alpha), one rounding
    const bool pass = !done && !(y > 0.0f) && !(alpha < 1.0f / 255.0f);
    const bool stop = pass && test_T < 0.0001f;
    const bool use = pass && !stop;
    done = done || stop;
    if (RGB) {
        const float4 Cc = cur.C[j];
        C0 = use ? fmaf(Cc.x * alpha, T, C0) : C0;
        C1 = use ? fmaf(Cc.y * alpha, T, C1) : C1;
        C2 = use ? fmaf(Cc.z * alpha, T, C2) : C2;
    } else {
        C0 = use ? fmaf(A.w * alpha, T, C0) : C0;
    }
    if (EXTRAS) {
        D = use ? fmaf(A.z * alpha, T, D) : D;
        Aacc = use ? fmaf(alpha, T, Aacc) : Aacc;
        if (use && p.n_touched && test_T > 0.5f) atomicAdd(p.n_touched + cur.id[j], 1);
        last = use ? r * GS_BLOCK + j + 1 : last;
    }
    T = use ? test_T : T;
}

// EXTRAS: the frame wants depth, alpha, contributor counts or n_touched (each still
// checked at run time); without it only the image and the final transmittance are
// accumulated (the batched tracker's case).
// Blends one tile (all threads of the block).  V is the tile's view; with TMA, `phase`
// carries the buffers' mbarrier parities from tile to tile.
template <bool EXTRAS, bool RGB, bool TMA>
__device__ __forceinline__ void fwd_tile(const BlendParams &p, const CUtensorMap *tm, int tile, Batch<RGB> (&sb)[2],
                                         const gsevt_view &V, uint64_t *mbar, uint32_t &phase)
{
    const int lt = tile - V.tile_offset;
    const int tx = lt % V.tiles_x, ty = lt / V.tiles_x;
    int px, py;
    float sx0, sx1, sy0, sy1;
    warp_pixel(threadIdx.x, tx, ty, px, py, sx0, sx1, sy0, sy1);
    const bool inside = px < V.width && py < V.height;
    const float pxf = (float)px, pyf = (float)py;
    const uint2 range = p.ws.ranges[tile];
    const int todo = (int)(range.y - range.x);
    const int rounds = (todo + GS_BLOCK - 1) / GS_BLOCK;
    float T = 1.0f, C0 = 0.0f, C1 = 0.0f, C2 = 0.0f, D = 0.0f, Aacc = 0.0f;
    int last = 0;
    bool done = !inside;
    const int lane = threadIdx.x & 31;
    int issued = 0, waited = 0;  // TMA: batches issued / waited for
    if (rounds > 0) {
        if (TMA) {
            tma_load_batch(p, sb[0], range, 0, &mbar[0], tm);
            issued = 1;
        } else {
            load_batch(p, sb[0], range, 0);
        }
    }
    for (int r = 0; r < rounds; ++r) {
        Batch<RGB> &cur = sb[r & 1];
        if (TMA) {
            if (r + 1 < rounds) {
                tma_load_batch(p, sb[(r + 1) & 1], range, r + 1, &mbar[(r + 1) & 1], tm);
                issued = r + 2;
            }
            if (!mbar_wait(&mbar[r & 1], (phase >> (r & 1)) & 1u, p.ws.spin_limit) && threadIdx.x == 0)
                atomicOr(p.ws.status, GSEVT_STATUS_STAGE_TIMEOUT);
            phase ^= 1u << (r & 1);
            waited = r + 1;
        } else if (r + 1 < rounds) {
            load_batch(p, sb[(r + 1) & 1], range, r + 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        if (__syncthreads_count(done) == GS_BLOCK) break;
        const int n = min(GS_BLOCK, todo - r * GS_BLOCK);
        if ((int)threadIdx.x < n) {
            float4 e;
            cur.box[threadIdx.x] = gauss_box(cur.r[threadIdx.x].A, cur.r[threadIdx.x].B, &e);
            cur.ell[threadIdx.x] = e;
        }
        __syncthreads();
        bool warp_done = false;
        for (int c0 = 0; c0 < n && !warp_done; c0 += 32) {
            // candidates of this warp among the next 32 Gaussians, in depth order
            const bool hit = warp_hit(cur, c0, n, lane, sx0, sx1, sy0, sy1);
            unsigned mask = __ballot_sync(0xffffffffu, hit);
            // candidates two at a time (one saturation vote and loop step per pair)
            while (mask) {
                if (__all_sync(0xffffffffu, done)) { warp_done = true; break; }
                fwd_candidate<EXTRAS, RGB>(cur, p, c0 + __ffs(mask) - 1, r, pxf, pyf, T, C0, C1, C2, D, Aacc, last, done);
                mask &= mask - 1;
                if (mask) {
                    fwd_candidate<EXTRAS, RGB>(cur, p, c0 + __ffs(mask) - 1, r, pxf, pyf, T, C0, C1, C2, D, Aacc, last,
                                               done);
                    mask &= mask - 1;
                }
            }
        }
        __syncthreads();  // the next iteration overwrites this buffer
    }
    if (TMA) {
        tma_drain(mbar, phase, issued, waited, p.ws.spin_limit, p.ws.status);
    } else {
        cp_async_wait<0>();  // no copy may still target shared memory when the block exits
    }
    if (inside) {
        const int pix = V.pix_offset + py * V.width + px;
        const size_t P = (size_t)p.total_pixels;
        if (RGB) {
            p.image[pix] = C0 + T * V.bg[0];
            p.image[P + pix] = C1 + T * V.bg[1];
            p.image[2 * P + pix] = C2 + T * V.bg[2];
        } else {
            const float bgg = (0.2989f * V.bg[0] + 0.587f * V.bg[1]) + 0.114f * V.bg[2];
            p.image[pix] = C0 + T * bgg;
        }
        p.final_T[pix] = T;
        if (EXTRAS) {
            if (p.depth) p.depth[pix] = D;
            if (p.alpha) p.alpha[pix] = Aacc;
            if (p.n_contrib) p.n_contrib[pix] = last;
        }
    }
}

// The next tile of a block, in thread 0: its own tile (one block per tile), or with
// PERSIST the next entry of the tile order (blocks stay resident and take tiles from one
// queue, longest lists first); -1 when there is none.
template <bool PERSIST>
__device__ __forceinline__ int next_tile(const BlendParams &p, int it)
{
    if (!PERSIST) return it == 0 ? (int)blockIdx.x : -1;
    const uint32_t q = atomicAdd(p.queue, 1u);
    return q < (uint32_t)p.num_tiles ? (int)p.order[q] : -1;
}

template <bool EXTRAS, bool RGB, bool TMA, bool PERSIST>
__global__ void __launch_bounds__(GS_BLOCK, RGB ? 5 : 6) k_blend_fwd(BlendParams p, const __grid_constant__ CUtensorMap tm)
{
    __shared__ Batch<RGB> sb[2];
    __shared__ gsevt_view V;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ int s_tile;
    if (gs_sort_timed_out(p.ws.status)) return;  // the tile lists are incomplete (uniform)
    if (TMA && threadIdx.x == 0) {
        // one arrival per issuing warp: warp 0 (staging 2) or every warp (staging 3)
        const uint32_t arrivals = p.stage_all_warps ? GS_BLOCK / 32 : 1;
        mbar_init(&mbar[0], arrivals);
        mbar_init(&mbar[1], arrivals);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    uint32_t phase = 0;  // TMA: parity of the next phase of each buffer's mbarrier (bit b)
    for (int it = 0;; ++it) {
        if (threadIdx.x == 0) {
            const int t = next_tile<PERSIST>(p, it);
            s_tile = t;
            if (t >= 0) V = p.views[gs_find_view_by_tile(p.views, p.num_views, t)];
        }
        __syncthreads();
        const int tile = s_tile;
        if (tile < 0) break;
        fwd_tile<EXTRAS, RGB, TMA>(p, &tm, tile, sb, V, mbar, phase);
        __syncthreads();  // V, s_tile and the batch buffers are reused by the next tile
    }
}

// Per-Gaussian gradient components accumulated per tile:
//   0,1 mean x,y (pixels)  2,3,4 conic x,y,z  5 opacity  6 colour (grey or r)  7 depth
//   8,9 colour g,b (RGB only).
// Modes: 0 tracker (grey, pose only: 0-4 and 6), 1 grey drop-in (0-7), 2 RGB drop-in (0-9).
template <int MODE> struct Comps {
    static constexpr int n = MODE == 0 ? 6 : (MODE == 1 ? 8 : 10);
};
// the component count rounded up to a power of two for the transposed reduction
template <int MODE>
__device__ __forceinline__ constexpr int comps_padded() { return MODE == 2 ? 16 : 8; }
template <int MODE>
__device__ __forceinline__ constexpr int comp_idx(int q) { return (MODE == 0 && q >= 5) ? 6 : q; }

// Transposed butterfly: reduces NV values (a power of two, 8 or 16) over the warp with
// NV - 1 + (5 - log2 NV) shuffles instead of 5 per value.  At each halving stage a lane
// keeps one half of its values and trades the other half with its partner; afterwards
// lane l holds the warp total of component (l >> (5 - log2 NV)) & (NV - 1).
template <int NV>
__device__ __forceinline__ float warp_reduce_transposed(float (&v)[NV], int lane)
{
    int m = NV;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        if (m > 1) {
            const bool hi = (lane & o) != 0;
            const int half = m >> 1;
#pragma unroll
            for (int k = 0; k < NV / 2; ++k) {
                if (k < half) {
                    const float send = hi ? v[k] : v[half + k];
                    const float keep = hi ? v[half + k] : v[k];
                    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
                }
            }
            m = half;
        } else {
            v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
        }
    }
    return v[0];
}

// Gradient of the pair loss w.r.t. pixel (px, py) of view V's grey image, whose value is
// Is (V belongs to a pair: V.pair >= 0).
__device__ __forceinline__ float pair_pixel_grad(const BlendParams &p, const gsevt_view &V, int px, int py, float Is)
{
    const gsevt_pair &pr = p.pairs[V.pair];
    const LossScal &sc = p.ws.loss_scal[V.pair];
    const float inv_s = sc.inv_s, ng = sc.ndotg, inv_L = sc.inv_L;
    const int lp = py * V.width + px;
    const int other = V.pair_role == 0 ? pr.next_view : pr.last_view;
    const float Io = p.image[p.views[other].pix_offset + lp];
    // log grey: dI of the logs, and dI/dI_self carries 1 / (I_self + eps)
    const bool lg = pr.log_grey != 0;
    const float ls = lg ? logf(Is + pr.log_eps) : Is, lo = lg ? logf(Io + pr.log_eps) : Io;
    const float dI = V.pair_role == 0 ? (lo - ls) : (ls - lo);
    const float e = (pr.unsigned_mode && pr.event_abs) ? pr.event_abs[lp] : pr.event[lp];
    const float n = dI * inv_s;
    float g;
    if (pr.unsigned_mode) {
        const float sg = (dI > 0.0f) ? 1.0f : (dI < 0.0f ? -1.0f : 0.0f);
        g = sg * (fabsf(n) - fabsf(e)) * inv_L;
    } else {
        g = (n - e) * inv_L;
    }
    float dd = (g - n * ng) * inv_s;
    if (lg) dd = __fdividef(dd, Is + pr.log_eps);
    return V.pair_role == 0 ? -dd : dd;
}

// One candidate of the tracker adjoint (grey, pair-loss gradient gC per pixel): the
// forward's decisions as predicates, the state update, and the six terms (the five
// power-gradient moments and the colour gradient), zero for a lane that does not blend it.
// A: the record's {mean x, mean y, depth, grey}; K: its base-2 conic and opacity.
// S: the colour behind this candidate so far, the rendered pixel minus the front-to-back
// sum of the candidates blended before it (it starts at the pixel's value).
// tracker_pixel returns, for the pixel at row pyf and column offset dx = mean x - pixel x,
// the power gradient dpow, the row offset dy and the blend weight wgt (alpha T) of the
// candidate, all zero-weighted when the pixel does not blend it; tracker_candidate forms
// the six terms of one pixel from them, pair_terms those of the two pixels of a lane in
// the two-pixel adjoint, which share dx.
__device__ __forceinline__ bool tracker_pixel(const float4 A, const float4 K, float dx, float pyf, float gC,
                                              float &T, float &S, bool &done, float &dpow, float &dy, float &wgt)
{
    dy = A.y - pyf;
    const float y = gs_power2(K, dx, dy);
    // araw = o exp(power), whose derivative in the (natural) power is araw itself
    const float araw = K.w * gs_exp2f(y);
    const float alpha = fminf(0.99f, araw);
    const float test_T = fmaf(-T, alpha, T);  // T (1 - alpha), one rounding
    const bool pass = !done && !(y > 0.0f) && !(alpha < 1.0f / 255.0f);
    const bool stop = pass && test_T < 0.0001f;
    const bool contrib = pass && !stop;
    done = done || stop;
    wgt = contrib ? alpha * T : 0.0f;
    // gradient-only term: the 2-ulp fast reciprocal suffices
    const float inv1m = __fdividef(1.0f, 1.0f - alpha);
    S = contrib ? __fmaf_rn(-A.w, wgt, S) : S;
    const float dal = gC * __fmaf_rn(-S, inv1m, T * A.w);
    // below the 0.99 clamp alpha depends on the power
    dpow = (contrib && araw <= 0.99f) ? dal * araw : 0.0f;
    T = contrib ? test_T : T;
    return contrib;
}

__device__ __forceinline__ bool tracker_candidate(const float4 A, const float4 K, float pxf, float pyf, float gC,
                                                  float &T, float &S, bool &done, float (&g)[6])
{
    const float dx = A.x - pxf;
    float dpow, dy, wgt;
    const bool contrib = tracker_pixel(A, K, dx, pyf, gC, T, S, done, dpow, dy, wgt);
    const float mx = dpow * dx, my = dpow * dy;
    g[0] = mx;
    g[1] = my;
    g[2] = mx * dx;
    g[3] = mx * dy;
    g[4] = my * dy;
    g[5] = gC * wgt;
    return contrib;
}

// The six terms of a candidate summed over the two pixels of a lane (same column, so the
// same dx): sum dpow dx = dx (dpow0 + dpow1), sum dpow dx dx and sum dpow dx dy are dx
// times the first two sums; 12 operations instead of twelve products and six additions.
__device__ __forceinline__ void pair_terms(float dx, float dp0, float dy0, float w0, float gC0, float dp1, float dy1,
                                           float w1, float gC1, float (&g)[6])
{
    const float my0 = dp0 * dy0, my1 = dp1 * dy1;
    g[0] = (dp0 + dp1) * dx;
    g[1] = my0 + my1;
    g[2] = g[0] * dx;
    g[3] = g[1] * dx;
    g[4] = __fmaf_rn(my1, dy1, my0 * dy0);
    g[5] = __fmaf_rn(gC1, w1, gC0 * w0);
}

// Warp sums of the six terms of two candidates: the first stage trades candidate b of
// lanes 0-15 for candidate a of lanes 16-31, then each half-warp reduces its candidate's
// six values (padded to 8) transposed.  Lane l ends with the sum of term (l >> 1) & 7 of
// candidate (l >> 4) (a for lanes 0-15).
__device__ __forceinline__ float warp_reduce_pair6(const float (&a)[6], const float (&b)[6], int lane)
{
    const bool hi = (lane & 16) != 0;
    float v[8];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float send = hi ? a[k] : b[k];
        const float keep = hi ? b[k] : a[k];
        v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
    v[6] = v[7] = 0.0f;
    int m = 8;
#pragma unroll
    for (int o = 8; o >= 1; o >>= 1) {
        if (m > 1) {
            const bool up = (lane & o) != 0;
            const int half = m >> 1;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (k < half) {
                    const float send = up ? v[k] : v[half + k];
                    const float keep = up ? v[half + k] : v[k];
                    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
                }
            }
            m = half;
        } else {
            v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
        }
    }
    return v[0];
}

// The adjoint of one tile (all threads of the block); acc is zero on entry and on exit.
template <int MODE, bool TMA>
__device__ __forceinline__ void bwd_tile(const BlendParams &p, const CUtensorMap *tm, int tile,
                                         Batch<MODE == 2> (&sb)[2], float (*acc)[Comps<MODE>::n + 1],
                                         const gsevt_view &V, uint64_t *mbar, uint32_t &phase)
{
    constexpr bool RGB = MODE == 2;
    constexpr int NC = Comps<MODE>::n;
    const int lane = threadIdx.x & 31;
    const int lt = tile - V.tile_offset;
    const int tx = lt % V.tiles_x, ty = lt / V.tiles_x;
    int px, py;
    float sx0, sx1, sy0, sy1;
    warp_pixel(threadIdx.x, tx, ty, px, py, sx0, sx1, sy0, sy1);
    const bool inside = px < V.width && py < V.height;
    const float pxf = (float)px, pyf = (float)py;
    const uint2 range = p.ws.ranges[tile];
    const int todo = (int)(range.y - range.x);
    const int rounds = (todo + GS_BLOCK - 1) / GS_BLOCK;
    const size_t P = (size_t)p.total_pixels;
    const int pix = V.pix_offset + py * V.width + px;

    // per-pixel inputs
    // Cimg: the rendered pixel (Gaussians plus background); the colour behind the
    // Gaussian at hand is Cimg minus the front-to-back partial sum Pc
    float Cimg[3] = {0, 0, 0}, gC[3] = {0, 0, 0}, gD = 0.0f, gA = 0.0f, Dtot = 0.0f, Atot = 0.0f;
    if (inside) {
#pragma unroll
        for (int c = 0; c < (RGB ? 3 : 1); ++c) Cimg[c] = p.image[c * P + pix];
        if (MODE != 0) {
#pragma unroll
            for (int c = 0; c < (RGB ? 3 : 1); ++c) gC[c] = p.dL_dimage[c * P + pix];
            if (p.dL_ddepth) { gD = p.dL_ddepth[pix]; Dtot = p.depth[pix]; }
            if (p.dL_dalpha) { gA = p.dL_dalpha[pix]; Atot = p.alpha[pix]; }
        } else if (V.pair >= 0) {
            gC[0] = pair_pixel_grad(p, V, px, py, p.image[pix]);
        }
    }

    float T = 1.0f, Pc[3] = {0, 0, 0}, PD = 0.0f, PA = 0.0f;
    if (MODE == 0) Pc[0] = Cimg[0];  // the tracker adjoint tracks the suffix instead of the prefix
    bool done = !inside;
    int issued = 0, waited = 0;  // TMA: batches issued / waited for
    if (rounds > 0) {
        if (TMA) {
            tma_load_batch(p, sb[0], range, 0, &mbar[0], tm);
            issued = 1;
        } else {
            load_batch(p, sb[0], range, 0);
        }
    }
    for (int r = 0; r < rounds; ++r) {
        Batch<RGB> &cur = sb[r & 1];
        if (TMA) {
            if (r + 1 < rounds) {
                tma_load_batch(p, sb[(r + 1) & 1], range, r + 1, &mbar[(r + 1) & 1], tm);
                issued = r + 2;
            }
            if (!mbar_wait(&mbar[r & 1], (phase >> (r & 1)) & 1u, p.ws.spin_limit) && threadIdx.x == 0)
                atomicOr(p.ws.status, GSEVT_STATUS_STAGE_TIMEOUT);
            phase ^= 1u << (r & 1);
            waited = r + 1;
        } else if (r + 1 < rounds) {
            load_batch(p, sb[(r + 1) & 1], range, r + 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        if (__syncthreads_count(done) == GS_BLOCK) break;
        const int n = min(GS_BLOCK, todo - r * GS_BLOCK);
        if ((int)threadIdx.x < n) {
            float4 e;
            cur.box[threadIdx.x] = gauss_box(cur.r[threadIdx.x].A, cur.r[threadIdx.x].B, &e);
            cur.ell[threadIdx.x] = e;
        }
        __syncthreads();
        bool warp_done = false;
        for (int c0 = 0; c0 < n && !warp_done; c0 += 32) {
            const bool hit = warp_hit(cur, c0, n, lane, sx0, sx1, sy0, sy1);
            unsigned mask = __ballot_sync(0xffffffffu, hit);
            if constexpr (MODE == 0) {
                // the tracker adjoint takes its candidates two at a time: one 12-value warp
                // reduction and one shared-memory atomic instruction for the pair
                while (mask) {
                    if (__all_sync(0xffffffffu, done)) { warp_done = true; break; }
                    const int ja = c0 + __ffs(mask) - 1;
                    mask &= mask - 1;
                    const bool has_b = mask != 0u;
                    const int jb = has_b ? c0 + __ffs(mask) - 1 : ja;
                    if (has_b) mask &= mask - 1;
                    float ga[6], gb[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
                    // Pc[0] holds the suffix (the pixel minus the blended prefix) here
                    const bool ca = tracker_candidate(cur.r[ja].A, gs_log2_conic(cur.r[ja].B), pxf, pyf, gC[0], T,
                                                      Pc[0], done, ga);
                    bool cb = false;
                    if (has_b)
                        cb = tracker_candidate(cur.r[jb].A, gs_log2_conic(cur.r[jb].B), pxf, pyf, gC[0], T, Pc[0],
                                               done, gb);
                    if (__any_sync(0xffffffffu, ca || cb)) {
                        const float s = warp_reduce_pair6(ga, gb, lane);
                        const int q = (lane >> 1) & 7;
                        const bool second = (lane & 16) != 0;
                        if ((lane & 1) == 0 && q < NC && s != 0.0f && (has_b || !second))
                            atomicAdd(&acc[second ? jb : ja][q], s);
                    }
                }
            } else {
            while (mask) {
                if (__all_sync(0xffffffffu, done)) { warp_done = true; break; }
                const int j = c0 + __ffs(mask) - 1;
                mask &= mask - 1;
                // The forward's decisions as predicates (every lane evaluates the candidate;
                // a lane that does not blend it contributes zeros and keeps its state).
                const float4 A = cur.r[j].A, B = cur.r[j].B;
                const float dx = A.x - pxf, dy = A.y - pyf;
                const float y = gs_power2(gs_log2_conic(B), dx, dy);
                const float G = gs_exp2f(y);
                const float araw = B.w * G;
                const float alpha = fminf(0.99f, araw);
                const float test_T = fmaf(-T, alpha, T);  // T (1 - alpha), one rounding
                const bool pass = !done && !(y > 0.0f) && !(alpha < 1.0f / 255.0f);
                const bool stop = pass && test_T < 0.0001f;
                const bool contrib = pass && !stop;
                done = done || stop;
                float gv[10];
                float col[3];
                if (RGB) { const float4 Cc = cur.C[j]; col[0] = Cc.x; col[1] = Cc.y; col[2] = Cc.z; }
                else { col[0] = A.w; col[1] = col[2] = 0.0f; }
                const float wgt = contrib ? alpha * T : 0.0f;
                // gradient-only term: the 2-ulp fast reciprocal suffices
                const float inv1m = __fdividef(1.0f, 1.0f - alpha);
                float dal = 0.0f;
#pragma unroll
                for (int c = 0; c < (RGB ? 3 : 1); ++c) {
                    Pc[c] = contrib ? __fmaf_rn(col[c], wgt, Pc[c]) : Pc[c];
                    const float suffix = Cimg[c] - Pc[c];
                    dal = __fmaf_rn(gC[c], __fmaf_rn(-suffix, inv1m, T * col[c]), dal);
                }
                if (MODE != 0) {
                    PD = contrib ? __fmaf_rn(A.z, wgt, PD) : PD;
                    PA = contrib ? PA + wgt : PA;
                    dal = __fmaf_rn(gD, __fmaf_rn(-(Dtot - PD), inv1m, T * A.z), dal);
                    dal = __fmaf_rn(gA, __fmaf_rn(-(Atot - PA), inv1m, T), dal);
                }
                gv[7] = gD * wgt;
                gv[6] = gC[0] * wgt;
                gv[8] = gC[1] * wgt;
                gv[9] = gC[2] * wgt;
                // below the 0.99 clamp alpha depends on the power and the opacity
                const float dun = (contrib && araw <= 0.99f) ? dal : 0.0f;
                gv[5] = dun * G;
                // d power / d(mean, conic) is linear in the conic: accumulate the moments of
                // dpow over (dx, dy) and apply the conic once per Gaussian when the batch is
                // flushed
                const float dpow = dun * araw;
                const float mx = dpow * dx, my = dpow * dy;
                gv[0] = mx;
                gv[1] = my;
                gv[2] = mx * dx;
                gv[3] = mx * dy;
                gv[4] = my * dy;
                T = contrib ? test_T : T;
                if (__any_sync(0xffffffffu, contrib)) {
                    constexpr int NV = comps_padded<MODE>();
                    constexpr int SH = NV == 8 ? 2 : 1;  // 5 - log2(NV)
                    float red[NV];
#pragma unroll
                    for (int q = 0; q < NV; ++q) red[q] = q < NC ? gv[comp_idx<MODE>(q)] : 0.0f;
                    const float s = warp_reduce_transposed<NV>(red, lane);
                    const int q = (lane >> SH) & (NV - 1);
                    if ((lane & ((1 << SH) - 1)) == 0 && q < NC && s != 0.0f) atomicAdd(&acc[j][q], s);
                }
            }
            }
        }
        __syncthreads();
        // flush this batch's per-Gaussian sums to the global per-slot gradients
        if ((int)threadIdx.x < n) {
            const uint32_t vg = cur.id[threadIdx.x];
            // moments (sum dpow dx, dpow dy, dpow dx^2, dpow dx dy, dpow dy^2) to the
            // gradients of the 2D mean and the conic
            {
                const float4 B = cur.r[threadIdx.x].B;
                float *a = acc[threadIdx.x];
                const float mx = a[0], my = a[1], mxx = a[2], mxy = a[3], myy = a[4];
                a[0] = -(B.x * mx + B.y * my);
                a[1] = -(B.z * my + B.y * mx);
                a[2] = -0.5f * mxx;
                a[3] = -mxy;
                a[4] = -0.5f * myy;
            }
            float *dst[10] = {(float *)(p.ws.gradA + vg), (float *)(p.ws.gradA + vg) + 1, (float *)(p.ws.gradA + vg) + 2,
                              (float *)(p.ws.gradA + vg) + 3, (float *)(p.ws.gradB + vg), (float *)(p.ws.gradB + vg) + 1,
                              (float *)(p.ws.gradB + vg) + 2, (float *)(p.ws.gradB + vg) + 3,
                              RGB ? (float *)(p.ws.gradC + vg) : nullptr, RGB ? (float *)(p.ws.gradC + vg) + 1 : nullptr};
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                const float a = acc[threadIdx.x][q];
                if (a != 0.0f) atomicAdd(dst[comp_idx<MODE>(q)], a);
                acc[threadIdx.x][q] = 0.0f;
            }
        }
        __syncthreads();
    }
    if (TMA) tma_drain(mbar, phase, issued, waited, p.ws.spin_limit, p.ws.status);
    else cp_async_wait<0>();
}

// the tracker adjoint (MODE 0) keeps five blocks per SM (its shared memory allows five)
template <int MODE, bool TMA, bool PERSIST>
__global__ void __launch_bounds__(GS_BLOCK, MODE == 0 ? 5 : 1) k_blend_bwd(BlendParams p,
                                                                         const __grid_constant__ CUtensorMap tm)
{
    constexpr bool RGB = MODE == 2;
    constexpr int NC = Comps<MODE>::n;
    __shared__ Batch<RGB> sb[2];
    __shared__ float acc[GS_BLOCK][NC + 1];
    __shared__ gsevt_view V;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ int s_tile;
    if (gs_sort_timed_out(p.ws.status)) return;  // the tile lists are incomplete (uniform)
    if (TMA && threadIdx.x == 0) {
        // one arrival per issuing warp: warp 0 (staging 2) or every warp (staging 3)
        const uint32_t arrivals = p.stage_all_warps ? GS_BLOCK / 32 : 1;
        mbar_init(&mbar[0], arrivals);
        mbar_init(&mbar[1], arrivals);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = threadIdx.x; i < GS_BLOCK * (NC + 1); i += GS_BLOCK) (&acc[0][0])[i] = 0.0f;
    uint32_t phase = 0;  // TMA: parity of the next phase of each buffer's mbarrier (bit b)
    for (int it = 0;; ++it) {
        if (threadIdx.x == 0) {
            const int t = next_tile<PERSIST>(p, it);
            s_tile = t;
            if (t >= 0) V = p.views[gs_find_view_by_tile(p.views, p.num_views, t)];
        }
        __syncthreads();
        const int tile = s_tile;
        if (tile < 0) break;
        bwd_tile<MODE, TMA>(p, &tm, tile, sb, acc, V, mbar, phase);
        __syncthreads();  // V, s_tile and the batch buffers are reused by the next tile
    }
}

// ---- the tracker adjoint with two pixels per lane (gsevt_tuning.adjoint_pixels 0 or 2) ----
// One block of 128 threads per tile: warp w covers the 8x8 pixel block (w & 1, w >> 1) of
// the tile, lane l the pixels (l & 7, l >> 3) and (l & 7, (l >> 3) + 4) of it.  Each
// candidate is evaluated for both pixels (each with its own transmittance, prefix and
// stop state, in depth order as in the one-pixel adjoint), the two pixels' six terms are
// added in the lane, and one warp reduction serves 64 pixels instead of 32.  The price is
// the coarser warp culling (an 8x8 rectangle instead of two 8x4 ones) and half the warps
// per tile.  Batches of 128 records halve the shared memory of a block (21 KB), so eight
// blocks (32 warps, 64 registers a thread) are resident per SM against five blocks (40
// warps) of the one-pixel adjoint.
#define PX2_THREADS 128

struct alignas(128) Batch2 {
    Rec r[PX2_THREADS];
    float4 k[PX2_THREADS];  // the base-2 conic and opacity of each record (gs_log2_conic)
    float4 box[PX2_THREADS];
    float4 ell[PX2_THREADS];
    uint32_t id[PX2_THREADS];
};

__device__ __forceinline__ void load_batch2(const BlendParams &p, Batch2 &buf, uint2 range, int r)
{
    const uint32_t idx = range.x + (uint32_t)r * PX2_THREADS + threadIdx.x;
    if (idx < range.y) {
        const uint32_t vg = __ldg(p.vals + idx);
        buf.id[threadIdx.x] = vg;
        cp_async16(&buf.r[threadIdx.x].A, p.ws.rec + 2 * (size_t)vg);
        cp_async16(&buf.r[threadIdx.x].B, p.ws.rec + 2 * (size_t)vg + 1);
    }
    cp_async_commit();
}

// One candidate of the grey forward blend (no extras) for one pixel: the arithmetic of
// fwd_candidate<false, false>, so the image bits are the same.
__device__ __forceinline__ void grey_candidate(const float4 A, const float4 K, float pxf, float pyf, float &T,
                                               float &C, bool &done)
{
    const float dx = A.x - pxf, dy = A.y - pyf;
    const float y = gs_power2(K, dx, dy);
    const float alpha = fminf(0.99f, K.w * gs_exp2f(y));
    const float test_T = fmaf(-T, alpha, T);  // T (1 - alpha), one rounding
    const bool pass = !done && !(y > 0.0f) && !(alpha < 1.0f / 255.0f);
    const bool stop = pass && test_T < 0.0001f;
    const bool use = pass && !stop;
    done = done || stop;
    C = use ? fmaf(A.w * alpha, T, C) : C;
    T = use ? test_T : T;
}

// The grey forward blend of the batched step with two pixels per lane
// (gsevt_tuning.forward_pixels 0 or 2): the layout of k_blend_bwd_px2 (128 threads and 8x8-pixel
// warps per tile, batches of 128 records); every pixel runs the one-pixel forward's
// sequence of operations, so images and transmittances are bit-identical.
__global__ void __launch_bounds__(PX2_THREADS, 8) k_blend_fwd_px2(BlendParams p)
{
    __shared__ Batch2 sb[2];
    __shared__ gsevt_view V;
    if (gs_sort_timed_out(p.ws.status)) return;  // the tile lists are incomplete (uniform)
    const int tile = p.ordered ? (int)p.order[blockIdx.x] : (int)blockIdx.x;
    if (threadIdx.x == 0) V = p.views[gs_find_view_by_tile(p.views, p.num_views, tile)];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int lt = tile - V.tile_offset;
    const int tx = lt % V.tiles_x, ty = lt / V.tiles_x;
    const int bx = tx * GSEVT_TILE + (w & 1) * 8, by = ty * GSEVT_TILE + (w >> 1) * 8;
    const int px = bx + (lane & 7), py0 = by + (lane >> 3), py1 = py0 + 4;
    const float sx0 = (float)bx, sx1 = (float)(bx + 7), sy0 = (float)by, sy1 = (float)(by + 7);
    const float pxf = (float)px, py0f = (float)py0, py1f = (float)py1;
    const bool in0 = px < V.width && py0 < V.height, in1 = px < V.width && py1 < V.height;
    const uint2 range = p.ws.ranges[tile];
    const int todo = (int)(range.y - range.x);
    const int rounds = (todo + PX2_THREADS - 1) / PX2_THREADS;
    float T0 = 1.0f, T1 = 1.0f, C0 = 0.0f, C1 = 0.0f;
    bool d0 = !in0, d1 = !in1;
    if (rounds > 0) load_batch2(p, sb[0], range, 0);
    for (int r = 0; r < rounds; ++r) {
        Batch2 &cur = sb[r & 1];
        if (r + 1 < rounds) {
            load_batch2(p, sb[(r + 1) & 1], range, r + 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        if (__syncthreads_count(d0 && d1) == PX2_THREADS) break;
        const int n = min(PX2_THREADS, todo - r * PX2_THREADS);
        if ((int)threadIdx.x < n) {
            float4 e;
            const float4 B = cur.r[threadIdx.x].B;
            cur.box[threadIdx.x] = gauss_box(cur.r[threadIdx.x].A, B, &e);
            cur.ell[threadIdx.x] = e;
            cur.k[threadIdx.x] = gs_log2_conic(B);
        }
        __syncthreads();
        bool warp_done = false;
        for (int c0 = 0; c0 < n && !warp_done; c0 += 32) {
            const bool hit = warp_hit(cur, c0, n, lane, sx0, sx1, sy0, sy1);
            unsigned mask = __ballot_sync(0xffffffffu, hit);
            // candidates two at a time (one saturation vote and loop step per pair)
            while (mask) {
                if (__all_sync(0xffffffffu, d0 && d1)) { warp_done = true; break; }
                const int ja = c0 + __ffs(mask) - 1;
                mask &= mask - 1;
                const float4 Aa = cur.r[ja].A, Ka = cur.k[ja];
                grey_candidate(Aa, Ka, pxf, py0f, T0, C0, d0);
                grey_candidate(Aa, Ka, pxf, py1f, T1, C1, d1);
                if (mask) {
                    const int jb = c0 + __ffs(mask) - 1;
                    mask &= mask - 1;
                    const float4 Ab = cur.r[jb].A, Kb = cur.k[jb];
                    grey_candidate(Ab, Kb, pxf, py0f, T0, C0, d0);
                    grey_candidate(Ab, Kb, pxf, py1f, T1, C1, d1);
                }
            }
        }
        __syncthreads();  // the next iteration overwrites this buffer
    }
    cp_async_wait<0>();  // no copy may still target shared memory when the block exits
    const float bgg = (0.2989f * V.bg[0] + 0.587f * V.bg[1]) + 0.114f * V.bg[2];
    if (in0) {
        const int pix = V.pix_offset + py0 * V.width + px;
        p.image[pix] = C0 + T0 * bgg;
        p.final_T[pix] = T0;
    }
    if (in1) {
        const int pix = V.pix_offset + py1 * V.width + px;
        p.image[pix] = C1 + T1 * bgg;
        p.final_T[pix] = T1;
    }
}

__global__ void __launch_bounds__(PX2_THREADS, 8) k_blend_bwd_px2(BlendParams p)
{
    constexpr int NC = Comps<0>::n;
    __shared__ Batch2 sb[2];
    __shared__ float acc[PX2_THREADS][NC + 1];
    __shared__ gsevt_view V;
    if (gs_sort_timed_out(p.ws.status)) return;  // the tile lists are incomplete (uniform)
    const int tile = p.ordered ? (int)p.order[blockIdx.x] : (int)blockIdx.x;
    if (threadIdx.x == 0) V = p.views[gs_find_view_by_tile(p.views, p.num_views, tile)];
    for (int i = threadIdx.x; i < PX2_THREADS * (NC + 1); i += PX2_THREADS) (&acc[0][0])[i] = 0.0f;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int lt = tile - V.tile_offset;
    const int tx = lt % V.tiles_x, ty = lt / V.tiles_x;
    const int bx = tx * GSEVT_TILE + (w & 1) * 8, by = ty * GSEVT_TILE + (w >> 1) * 8;
    const int px = bx + (lane & 7), py0 = by + (lane >> 3), py1 = py0 + 4;
    const float sx0 = (float)bx, sx1 = (float)(bx + 7), sy0 = (float)by, sy1 = (float)(by + 7);
    const float pxf = (float)px, py0f = (float)py0, py1f = (float)py1;
    const bool in0 = px < V.width && py0 < V.height, in1 = px < V.width && py1 < V.height;
    float Cimg0 = 0.0f, gC0 = 0.0f, Cimg1 = 0.0f, gC1 = 0.0f;
    if (in0) {
        Cimg0 = p.image[V.pix_offset + py0 * V.width + px];
        if (V.pair >= 0) gC0 = pair_pixel_grad(p, V, px, py0, Cimg0);
    }
    if (in1) {
        Cimg1 = p.image[V.pix_offset + py1 * V.width + px];
        if (V.pair >= 0) gC1 = pair_pixel_grad(p, V, px, py1, Cimg1);
    }
    const uint2 range = p.ws.ranges[tile];
    const int todo = (int)(range.y - range.x);
    const int rounds = (todo + PX2_THREADS - 1) / PX2_THREADS;
    float T0 = 1.0f, T1 = 1.0f, S0 = Cimg0, S1 = Cimg1;  // transmittance and suffix per pixel
    bool d0 = !in0, d1 = !in1;
    if (rounds > 0) load_batch2(p, sb[0], range, 0);
    for (int r = 0; r < rounds; ++r) {
        Batch2 &cur = sb[r & 1];
        if (r + 1 < rounds) {
            load_batch2(p, sb[(r + 1) & 1], range, r + 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        if (__syncthreads_count(d0 && d1) == PX2_THREADS) break;
        const int n = min(PX2_THREADS, todo - r * PX2_THREADS);
        if ((int)threadIdx.x < n) {
            float4 e;
            const float4 B = cur.r[threadIdx.x].B;
            cur.box[threadIdx.x] = gauss_box(cur.r[threadIdx.x].A, B, &e);
            cur.ell[threadIdx.x] = e;
            cur.k[threadIdx.x] = gs_log2_conic(B);
        }
        __syncthreads();
        bool warp_done = false;
        for (int c0 = 0; c0 < n && !warp_done; c0 += 32) {
            const bool hit = warp_hit(cur, c0, n, lane, sx0, sx1, sy0, sy1);
            unsigned mask = __ballot_sync(0xffffffffu, hit);
            while (mask) {
                if (__all_sync(0xffffffffu, d0 && d1)) { warp_done = true; break; }
                const int ja = c0 + __ffs(mask) - 1;
                mask &= mask - 1;
                const bool has_b = mask != 0u;
                const int jb = has_b ? c0 + __ffs(mask) - 1 : ja;
                if (has_b) mask &= mask - 1;
                float ga[6], gb[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
                float p0, p1, y0, y1, w0, w1;
                const float4 Aa = cur.r[ja].A, Ka = cur.k[ja];
                const float dxa = Aa.x - pxf;
                const bool ca0 = tracker_pixel(Aa, Ka, dxa, py0f, gC0, T0, S0, d0, p0, y0, w0);
                const bool ca1 = tracker_pixel(Aa, Ka, dxa, py1f, gC1, T1, S1, d1, p1, y1, w1);
                pair_terms(dxa, p0, y0, w0, gC0, p1, y1, w1, gC1, ga);
                bool cb = false;
                if (has_b) {
                    const float4 Ab = cur.r[jb].A, Kb = cur.k[jb];
                    const float dxb = Ab.x - pxf;
                    const bool cb0 = tracker_pixel(Ab, Kb, dxb, py0f, gC0, T0, S0, d0, p0, y0, w0);
                    const bool cb1 = tracker_pixel(Ab, Kb, dxb, py1f, gC1, T1, S1, d1, p1, y1, w1);
                    pair_terms(dxb, p0, y0, w0, gC0, p1, y1, w1, gC1, gb);
                    cb = cb0 || cb1;
                }
                if (__any_sync(0xffffffffu, ca0 || ca1 || cb)) {
                    const float s = warp_reduce_pair6(ga, gb, lane);
                    const int q = (lane >> 1) & 7;
                    const bool second = (lane & 16) != 0;
                    if ((lane & 1) == 0 && q < NC && s != 0.0f && (has_b || !second))
                        atomicAdd(&acc[second ? jb : ja][q], s);
                }
            }
        }
        __syncthreads();
        // this batch's per-Gaussian sums to the global per-slot gradients (the moments to
        // the 2D mean and conic gradients, as in the one-pixel adjoint)
        if ((int)threadIdx.x < n) {
            const uint32_t vg = cur.id[threadIdx.x];
            const float4 B = cur.r[threadIdx.x].B;
            float *a = acc[threadIdx.x];
            const float mx = a[0], my = a[1], mxx = a[2], mxy = a[3], myy = a[4];
            a[0] = -(B.x * mx + B.y * my);
            a[1] = -(B.z * my + B.y * mx);
            a[2] = -0.5f * mxx;
            a[3] = -mxy;
            a[4] = -0.5f * myy;
            float *dst[7] = {(float *)(p.ws.gradA + vg), (float *)(p.ws.gradA + vg) + 1, (float *)(p.ws.gradA + vg) + 2,
                             (float *)(p.ws.gradA + vg) + 3, (float *)(p.ws.gradB + vg), (float *)(p.ws.gradB + vg) + 1,
                             (float *)(p.ws.gradB + vg) + 2};
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                const float v = a[q];
                if (v != 0.0f) atomicAdd(dst[comp_idx<0>(q)], v);
                a[q] = 0.0f;
            }
        }
        __syncthreads();
    }
    cp_async_wait<0>();  // no copy may still target shared memory when the block exits
}

// Orders the tiles for the persistent blends: descending list length in 33 buckets
// (bucket 1 + floor(log2 len), empty lists last), so that the blocks that finish last take
// short tiles.  One block; also clears the two queue heads (forward, adjoint).
__global__ void __launch_bounds__(1024) k_tile_order(const uint2 *ranges, int num_tiles, uint32_t *order,
                                                     uint32_t *queues)
{
    __shared__ uint32_t cnt[33], start[33];
    const int t = threadIdx.x;
    if (t < 33) cnt[t] = 0u;
    __syncthreads();
    for (int i = t; i < num_tiles; i += blockDim.x) {
        const uint32_t len = ranges[i].y - ranges[i].x;
        atomicAdd(&cnt[len ? 32 - __clz(len) : 0], 1u);
    }
    __syncthreads();
    if (t == 0) {
        uint32_t run = 0;
        for (int b = 32; b >= 0; --b) {
            start[b] = run;
            run += cnt[b];
        }
        queues[0] = queues[1] = 0u;
    }
    __syncthreads();
    for (int i = t; i < num_tiles; i += blockDim.x) {
        const uint32_t len = ranges[i].y - ranges[i].x;
        order[atomicAdd(&start[len ? 32 - __clz(len) : 0], 1u)] = (uint32_t)i;
    }
}

}  // namespace

static BlendParams make_params(const gsevt_frame *f, const Workspace &ws, const uint32_t *vals)
{
    BlendParams p;
    p.views = f->views;
    p.num_views = f->L.num_views;
    p.pairs = f->pairs;
    p.ws = ws;
    p.vals = vals;
    p.rgb = f->L.channels == 3;
    p.total_pixels = f->L.total_pixels;
    p.image = f->image;
    p.final_T = f->final_T;
    p.depth = f->depth;
    p.alpha = f->alpha;
    p.n_contrib = f->n_contrib;
    p.n_touched = f->n_touched;
    p.dL_dimage = p.dL_ddepth = p.dL_dalpha = nullptr;
    p.stage_all_warps = f->L.tuning.blend_staging == 3;
    p.order = ws.keys[0];  // free once the tile lists are built (batched step)
    p.queue = ws.status + 8;
    p.num_tiles = f->L.total_tiles;
    p.ordered = 0;
    return p;
}

// Longest-first blends (gsevt_tuning.blend_schedule 1, batched step only): the one-pixel
// blends run persistent, the two-pixel blends launch one block per tile in that order; the
// tile order and the queue heads live in the first pair-key buffer and status words 8-9.
bool gs_blend_persistent(const gsevt_frame *f)
{
    return f->L.tuning.blend_schedule == 1 && f->L.channels == 1 && (uint32_t)f->L.total_tiles <= f->L.key_capacity;
}

int gs_launch_tile_order(const gsevt_frame *f, const Workspace &ws, cudaStream_t s)
{
    k_tile_order<<<1, 1024, 0, s>>>(ws.ranges, f->L.total_tiles, ws.keys[0], ws.status + 8);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

// resident blocks of a kernel on the current device (for the persistent grids)
template <typename K>
static int resident_grid(K kernel, int tiles)
{
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                 cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, GS_BLOCK, 0) != cudaSuccess || per_sm < 1)
        return tiles;
    return std::min(tiles, sms * per_sm);
}

// The record tensor of a frame for the TMA staging path: num_vg rows of 8 floats (32 bytes),
// boxes of one row (what tile::gather4 copies four of).  false when the driver entry point or
// the encoding is unavailable, in which case the blends stage with cp.async.
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static bool record_tensor_map(const gsevt_frame *f, const Workspace &ws, CUtensorMap *tm)
{
    static std::atomic<EncodeTiledFn> encode{nullptr};
    static std::atomic<int> resolved{0};
    if (!resolved.load()) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            encode.store((EncodeTiledFn)fn);
        resolved.store(1);
    }
    EncodeTiledFn enc = encode.load();
    if (!enc || f->L.num_vg <= 0) return false;
    const cuuint64_t dims[2] = {8, (cuuint64_t)f->L.num_vg};
    const cuuint64_t strides[1] = {32};  // bytes between rows
    const cuuint32_t box[2] = {8, 1};
    const cuuint32_t estr[2] = {1, 1};
    return enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)ws.rec, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// TMA staging is used for the grey tracker blends when the frame's tuning asks for it.
static bool use_tma(const gsevt_frame *f, const Workspace &ws, CUtensorMap *tm)
{
    std::memset(tm, 0, sizeof(*tm));
    return (f->L.tuning.blend_staging == 2 || f->L.tuning.blend_staging == 3) && f->L.channels == 1 &&
           record_tensor_map(f, ws, tm);
}

int gs_launch_blend_fwd(const gsevt_frame *f, const Workspace &ws, const uint32_t *vals, cudaStream_t s,
                        bool persist)
{
    if (f->L.total_tiles <= 0) return GSEVT_OK;
    BlendParams p = make_params(f, ws, vals);
    if (f->n_touched) cudaMemsetAsync(f->n_touched, 0, (size_t)f->L.num_vg * 4, s);
    const int n = f->L.total_tiles;
    const bool extras = f->depth || f->alpha || f->n_contrib || f->n_touched;
    CUtensorMap tm;
    const bool tma = !extras && use_tma(f, ws, &tm);
    if (p.rgb) {
        if (extras) k_blend_fwd<true, true, false, false><<<n, GS_BLOCK, 0, s>>>(p, tm);
        else k_blend_fwd<false, true, false, false><<<n, GS_BLOCK, 0, s>>>(p, tm);
    } else if (extras) {
        k_blend_fwd<true, false, false, false><<<n, GS_BLOCK, 0, s>>>(p, tm);
    } else if (f->L.tuning.forward_pixels != 1) {
        p.ordered = persist ? 1 : 0;  // the tile order was built for this launch
        k_blend_fwd_px2<<<n, PX2_THREADS, 0, s>>>(p);
    } else if (persist) {
        p.queue = ws.status + 8;
        if (tma) {
            auto k = k_blend_fwd<false, false, true, true>;
            k<<<resident_grid(k, n), GS_BLOCK, 0, s>>>(p, tm);
        } else {
            auto k = k_blend_fwd<false, false, false, true>;
            k<<<resident_grid(k, n), GS_BLOCK, 0, s>>>(p, tm);
        }
    } else if (tma) {
        k_blend_fwd<false, false, true, false><<<n, GS_BLOCK, 0, s>>>(p, tm);
    } else {
        k_blend_fwd<false, false, false, false><<<n, GS_BLOCK, 0, s>>>(p, tm);
    }
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

int gs_launch_blend_bwd(const gsevt_frame *f, const Workspace &ws, const uint32_t *vals, const float *dL_dimage,
                        const float *dL_ddepth, const float *dL_dalpha, cudaStream_t s, bool persist)
{
    if (f->L.total_tiles <= 0) return GSEVT_OK;
    BlendParams p = make_params(f, ws, vals);
    p.dL_dimage = dL_dimage;
    p.dL_ddepth = dL_ddepth;
    p.dL_dalpha = dL_dalpha;
    CUtensorMap tm;
    const bool tma = !p.rgb && !dL_dimage && use_tma(f, ws, &tm);
    const int n = f->L.total_tiles;
    if (p.rgb) {
        k_blend_bwd<2, false, false><<<n, GS_BLOCK, 0, s>>>(p, tm);
    } else if (dL_dimage) {
        k_blend_bwd<1, false, false><<<n, GS_BLOCK, 0, s>>>(p, tm);
    } else if (f->L.tuning.adjoint_pixels != 1) {
        p.ordered = persist ? 1 : 0;
        k_blend_bwd_px2<<<n, PX2_THREADS, 0, s>>>(p);
    } else if (persist) {
        p.queue = ws.status + 9;
        if (tma) {
            auto k = k_blend_bwd<0, true, true>;
            k<<<resident_grid(k, n), GS_BLOCK, 0, s>>>(p, tm);
        } else {
            auto k = k_blend_bwd<0, false, true>;
            k<<<resident_grid(k, n), GS_BLOCK, 0, s>>>(p, tm);
        }
    } else if (tma) {
        k_blend_bwd<0, true, false><<<n, GS_BLOCK, 0, s>>>(p, tm);
    } else {
        k_blend_bwd<0, false, false><<<n, GS_BLOCK, 0, s>>>(p, tm);
    }
    GS_CUDA_CHECK();
    return GSEVT_OK;
}
