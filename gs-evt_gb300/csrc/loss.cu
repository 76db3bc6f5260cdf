// Normalised intensity-change loss of every render pair, in one launch.
//
// Replaces utils/render_camera/frame.py:86-94 (dI = I_next - I_last, n = dI/||dI||,
// or with the pair's log_grey the log-intensity change ln(I_next + eps) - ln(I_last + eps),
// |n|) and utils/tracker.py:93-103 (L = ||n - E|| or || |n| - |E| ||), which run as
// ~8 forward and ~10 backward torch kernels per iteration.  With s = ||dI||,
// c = sum(dI E) (signed) or sum(|dI| |E|) (unsigned) and e2 = sum(E^2),
//   L^2 = 1 - 2 c / s + e2,
// so one reduction pass gives L (FP32 over each thread's 8 pixels, float pairs with
// error-free additions within a block, FP64 across blocks); the per-pixel gradient
//   dL/dI_next = -dL/dI_last = (g - n (n.g)) / s,  n.g = (1 - c/s) / L,
// (times 1 / (I + eps) of the view's own pixel in log mode)
// is formed inside the blend adjoint without another pass, from 1/s, n.g and 1/L that
// the last block rounds to FP32 once per pair (no FP64 arithmetic per pixel).
// Each block reduces a slice of one pair into FP64 partials; the last block of the
// pair to finish (atomic ticket after a fence) adds the partials in a fixed order, so
// the scalars do not depend on block scheduling.
#include "common.cuh"

namespace {

// threads of a loss block and pixels per thread (GSEVT_LOSS_PIXELS_PER_BLOCK = their product)
#define LOSS_THREADS 512
#define LOSS_PIX_PER_THREAD 4
static_assert(LOSS_THREADS * LOSS_PIX_PER_THREAD == GSEVT_LOSS_PIXELS_PER_BLOCK, "loss block size");

__device__ __forceinline__ int find_pair(const gsevt_pair *pairs, int num_pairs, int block)
{
    int lo = 0, hi = num_pairs - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pairs[mid].block_offset <= block) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(LOSS_THREADS) k_loss(const gsevt_view *views, const gsevt_pair *pairs, int num_pairs,
                                                   const float *image, Workspace ws, double *loss_out)
{
    __shared__ FP2 part[LOSS_THREADS / 32][3];
    __shared__ double dpart[LOSS_THREADS / 32][3];
    __shared__ bool is_last;
    if (gs_sort_timed_out(ws.status)) return;  // no images were rendered (uniform)
    const int b = blockIdx.x;
    const int pi = find_pair(pairs, num_pairs, b);
    const gsevt_pair pr = pairs[pi];
    const gsevt_view &Vl = views[pr.last_view];
    const gsevt_view &Vn = views[pr.next_view];
    if (Vl.skip || Vn.skip) return;  // a finished problem: nothing rendered (uniform per pair)
    const int P = Vl.width * Vl.height;
    const int lb = b - pr.block_offset;
    // FP32 sums over this thread's 8 pixels, FP64 from the warp level up
    float s2 = 0.0f, cr = 0.0f, e2 = 0.0f;
    const int base = lb * LOSS_THREADS * LOSS_PIX_PER_THREAD;
    const bool lg = pr.log_grey != 0;
    const float eps = pr.log_eps;
#pragma unroll
    for (int k = 0; k < LOSS_PIX_PER_THREAD; ++k) {
        int i = base + k * LOSS_THREADS + threadIdx.x;
        if (i < P) {
            const float In = image[Vn.pix_offset + i], Il = image[Vl.pix_offset + i];
            float d = lg ? logf(In + eps) - logf(Il + eps) : In - Il;
            float e = (pr.unsigned_mode && pr.event_abs) ? __ldg(pr.event_abs + i) : __ldg(pr.event + i);
            s2 = fmaf(d, d, s2);
            e2 = fmaf(e, e, e2);
            cr = pr.unsigned_mode ? fmaf(fabsf(d), fabsf(e), cr) : fmaf(d, e, cr);
        }
    }
    // warp and block sums as float pairs (error-free FP32 additions; GB300's FP64 rate
    // would make double arithmetic the slow part), converted to FP64 once per block
    FP2 S2 = warp_sum_fp2(s2), CR = warp_sum_fp2(cr), E2 = warp_sum_fp2(e2);
    if ((threadIdx.x & 31) == 0) {
        part[threadIdx.x >> 5][0] = S2;
        part[threadIdx.x >> 5][1] = CR;
        part[threadIdx.x >> 5][2] = E2;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        FP2 t;
        for (int w = 0; w < LOSS_THREADS / 32; ++w) t.add(part[w][threadIdx.x]);
        ws.loss_part[(size_t)b * 4 + threadIdx.x] = (double)t.hi + (double)t.lo;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int t = atomicAdd(&ws.loss_done[pi], 1u);
        is_last = (t == (unsigned)pr.num_blocks - 1u);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // the last block of the pair adds the block partials: each thread a strided subset in
    // a fixed order, then a fixed-shape tree, so the result does not depend on scheduling
    const volatile double *lp = ws.loss_part;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int i = threadIdx.x; i < pr.num_blocks; i += LOSS_THREADS) {
        size_t q = (size_t)(pr.block_offset + i) * 4;
        a0 += lp[q];
        a1 += lp[q + 1];
        a2 += lp[q + 2];
    }
    a0 = warp_sum_d(a0);
    a1 = warp_sum_d(a1);
    a2 = warp_sum_d(a2);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        dpart[threadIdx.x >> 5][0] = a0;
        dpart[threadIdx.x >> 5][1] = a1;
        dpart[threadIdx.x >> 5][2] = a2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double S2t = 0, CRt = 0, E2t = 0;
        for (int w = 0; w < LOSS_THREADS / 32; ++w) { S2t += dpart[w][0]; CRt += dpart[w][1]; E2t += dpart[w][2]; }
        double s = sqrt(S2t);
        double L2 = 1.0 - 2.0 * CRt / s + E2t;
        double L = sqrt(L2 > 0.0 ? L2 : 0.0);
        LossScal &sc = ws.loss_scal[pi];
        sc.s = s;
        sc.cross = CRt;
        sc.e2 = E2t;
        sc.L = L;
        // factors of the per-pixel image gradient, rounded once here so the adjoint
        // blend's per-pixel prologue stays in FP32
        sc.inv_s = (float)(1.0 / s);
        sc.ndotg = (float)((1.0 - CRt / s) / L);
        sc.inv_L = (float)(1.0 / L);
        sc.pad = 0.0f;
        if (loss_out) loss_out[pi] = L;
        if (!(L == L) || !(s > 0.0)) atomicOr(ws.status, GSEVT_STATUS_NONFINITE);
        ws.loss_done[pi] = 0u;
    }
}

}  // namespace

int gs_loss_blocks_for(int pixels) { return (pixels + LOSS_THREADS * LOSS_PIX_PER_THREAD - 1) / (LOSS_THREADS * LOSS_PIX_PER_THREAD); }

int gs_launch_loss(const gsevt_frame *f, const Workspace &ws, double *loss_out, cudaStream_t s)
{
    if (f->L.num_pairs <= 0 || f->L.loss_blocks <= 0 || !f->pairs) return GSEVT_ERR_ARG;
    k_loss<<<f->L.loss_blocks, LOSS_THREADS, 0, s>>>(f->views, f->pairs, f->L.num_pairs, f->image, ws, loss_out);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}
