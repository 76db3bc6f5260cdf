// Twist-only adjoint of the batched tracker from the forward cache (see the kernel).
//
// This file is compiled with multiply-add contraction allowed (-fmad=true): it holds only
// gradient arithmetic, whose parity is a tolerance against the FP64 oracle gradient, and
// no forward value or decision that must match the oracle bit for bit.
#include "common.cuh"

namespace {

struct CachedParams {
    const gsevt_view *views;
    const gsevt_map *maps;
    int num_views;
    Workspace ws;
};

// Twist-only adjoint of the batched tracker from the forward cache: one thread per
// (view, Gaussian) slot, block b = (view, chunk b - sb_offset), no map attributes and no
// forward recomputation.  The chain is that of slot_backward for a grey frame without
// map gradients, with S T0^T, S T1^T and the direction term U taken from the cache.
__global__ void __launch_bounds__(GS_BLOCK) k_preprocess_bwd_cached(CachedParams p)
{
    __shared__ gsevt_view V;
    __shared__ int s_n;
    __shared__ float wpart[GS_BLOCK / 32][6];
    const int b = blockIdx.x;
    if (gs_sort_timed_out(p.ws.status)) return;  // no blend adjoint ran (uniform)
    if (threadIdx.x == 0) {
        int lo = 0, hi = p.num_views - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (p.views[mid].sb_offset <= b) lo = mid; else hi = mid - 1;
        }
        V = p.views[lo];
        s_n = p.maps[V.map].n;
    }
    __syncthreads();
    float xi[6] = {0, 0, 0, 0, 0, 0};
    const int g = (b - V.sb_offset) * GS_BLOCK + threadIdx.x;
    const size_t vg = (size_t)V.vg_offset + g;
    // The compaction cleared every slot's gradient, so a zero gradient marks a slot that is
    // not visible or that the blend adjoint never reached (behind saturated pixels); its
    // twist term is zero, and its forward cache (written for visible slots only) is not read.
    float4 GA = make_float4(0.0f, 0.0f, 0.0f, 0.0f), GB = GA;
    if (g < s_n) {
        GA = p.ws.gradA[vg];
        GB = p.ws.gradB[vg];
    }
    const bool live = GA.x != 0.0f || GA.y != 0.0f || GA.z != 0.0f || GA.w != 0.0f || GB.x != 0.0f ||
                      GB.y != 0.0f || GB.z != 0.0f || GB.w != 0.0f;
    if (live) {
        const float4 *c = p.ws.fcache + vg * GS_FCACHE;
        const float4 c0 = c[0], c1 = c[1], c2 = c[2], c3 = c[3], c4 = c[4], c5 = c[5];
        const float gCa = GA.z, gCb = GA.w, gCc = GB.x;
        const float a2 = c0.x, b2 = c0.y, c2_ = c0.z, det = c0.w;
        const float d2 = det * det;
        const float ga = (gCa * (-c2_ * c2_) + gCb * (b2 * c2_) + gCc * (-b2 * b2)) / d2;
        const float gb_ = (gCa * (2.0f * b2 * c2_) + gCb * (-(a2 * c2_ + b2 * b2)) + gCc * (2.0f * a2 * b2)) / d2;
        const float gc = (gCa * (-b2 * b2) + gCb * (a2 * b2) + gCc * (-a2 * a2)) / d2;
        const float Gs00 = ga, Gs01 = 0.5f * gb_, Gs11 = gc;
        const float T0S[3] = {c1.x, c1.y, c1.z}, T1S[3] = {c1.w, c2.x, c2.y};
        float gT0[3], gT1[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            gT0[j] = 2.0f * (Gs00 * T0S[j] + Gs01 * T1S[j]);
            gT1[j] = 2.0f * (Gs01 * T0S[j] + Gs11 * T1S[j]);
        }
        const float *R = V.R;
        const float J00 = c2.z, J02 = c2.w, J11 = c3.x, J12 = c3.y;
        float gJ00 = 0, gJ02 = 0, gJ11 = 0, gJ12 = 0;
        float gW[3][3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            gJ00 += gT0[j] * R[j];
            gJ02 += gT0[j] * R[6 + j];
            gJ11 += gT1[j] * R[3 + j];
            gJ12 += gT1[j] * R[6 + j];
            gW[0][j] = gT0[j] * J00;
            gW[1][j] = gT1[j] * J11;
            gW[2][j] = gT0[j] * J02 + gT1[j] * J12;
        }
        const float fx = (float)V.width / (2.0f * V.tanfovx), fy = (float)V.height / (2.0f * V.tanfovy);
        const float vx = c3.z, vy = c3.w, vz = c4.x;
        const float ivz = 1.0f / vz, ivz2 = ivz * ivz, ivz3 = ivz2 * ivz;
        const int flags = __float_as_int(c5.w);
        float gpc[3] = {0, 0, 0};
        gpc[2] += gJ00 * (-fx * ivz2) + gJ11 * (-fy * ivz2);
        if (!(flags & 1)) { gpc[0] += gJ02 * (-fx * ivz2); gpc[2] += gJ02 * (2.0f * fx * vx * ivz3); }
        else { gpc[2] += gJ02 * (-J02 * ivz); }
        if (!(flags & 2)) { gpc[1] += gJ12 * (-fy * ivz2); gpc[2] += gJ12 * (2.0f * fy * vy * ivz3); }
        else { gpc[2] += gJ12 * (-J12 * ivz); }
        const float gnx = GA.x * 0.5f * (float)V.width, gny = GA.y * 0.5f * (float)V.height;
        const float pw = c4.y;
        const float gh0 = gnx * pw, gh1 = gny * pw, gh3 = -(gnx * c4.z + gny * c4.w) * pw * pw;
#pragma unroll
        for (int j = 0; j < 3; ++j) gpc[j] += V.P[j] * gh0 + V.P[4 + j] * gh1 + V.P[12 + j] * gh3;
        gpc[2] += GB.w;
        const float gu[3] = {GB.z * c5.x, GB.z * c5.y, GB.z * c5.z};
        const float Rgu0 = R[0] * gu[0] + R[1] * gu[1] + R[2] * gu[2];
        const float Rgu1 = R[3] * gu[0] + R[4] * gu[1] + R[5] * gu[2];
        const float Rgu2 = R[6] * gu[0] + R[7] * gu[1] + R[8] * gu[2];
        xi[0] = gpc[0] + Rgu0;
        xi[1] = gpc[1] + Rgu1;
        xi[2] = gpc[2] + Rgu2;
        const float M12 = R[3] * gW[2][0] + R[4] * gW[2][1] + R[5] * gW[2][2];
        const float M21 = R[6] * gW[1][0] + R[7] * gW[1][1] + R[8] * gW[1][2];
        const float M20 = R[6] * gW[0][0] + R[7] * gW[0][1] + R[8] * gW[0][2];
        const float M02 = R[0] * gW[2][0] + R[1] * gW[2][1] + R[2] * gW[2][2];
        const float M01 = R[0] * gW[1][0] + R[1] * gW[1][1] + R[2] * gW[1][2];
        const float M10 = R[3] * gW[0][0] + R[4] * gW[0][1] + R[5] * gW[0][2];
        xi[3] = (vy * gpc[2] - vz * gpc[1]) + (M12 - M21);
        xi[4] = (vz * gpc[0] - vx * gpc[2]) + (M20 - M02);
        xi[5] = (vx * gpc[1] - vy * gpc[0]) + (M01 - M10);
    }
    // FP32 within the warp, the eight warp sums added as a float pair (error-free FP32
    // additions, no FP64 arithmetic) in warp order
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float sm = warp_sum(xi[k]);
        if ((threadIdx.x & 31) == 0) wpart[threadIdx.x >> 5][k] = sm;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        FP2 sm;
        for (int w = 0; w < GS_BLOCK / 32; ++w) sm.add(wpart[w][threadIdx.x], 0.0f);
        ((float2 *)p.ws.xi_part)[(size_t)b * 6 + threadIdx.x] = make_float2(sm.hi, sm.lo);
    }
}

}  // namespace

int gs_launch_preprocess_bwd_cached(const gsevt_frame *f, const Workspace &ws, cudaStream_t s)
{
    if (!ws.fcache) return GSEVT_ERR_ARG;
    CachedParams p;
    p.views = f->views;
    p.maps = f->maps;
    p.num_views = f->L.num_views;
    p.ws = ws;
    if (f->L.num_scan_blocks <= 0) return GSEVT_OK;
    k_preprocess_bwd_cached<<<f->L.num_scan_blocks, GS_BLOCK, 0, s>>>(p);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}
