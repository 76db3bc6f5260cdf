// Per-Gaussian preprocessing, forward and adjoint.
//
// Forward (k_preprocess_fwd): one thread per Gaussian of a map, looping over every view
// of that map, so the 232 B of attributes (position, opacity, cov3D, 48 SH
// coefficients) are read from HBM once per map and reused for all its views (the
// (t, t+dtau) pair, or all pose hypotheses).  Per (view, Gaussian) slot it writes the
// binning record, the two blend records and the per-(view, block) visible counts.
// The arithmetic follows the oracle's FP32 instance (oracle/or_math.inc) operation by
// operation: view transform, 1.3x guard-band Jacobian, EWA cov2D + 0.3, conic,
// radius = ceil(3 sqrt(lambda_max)), 16x16 tile rect, SH degree-3 colour + 0.5 clamped
// at 0, grey = 0.2989 R + 0.587 G + 0.114 B (utils/render_camera/frame.py:39-43).
//
// For batched-tracker frames the forward also bins each Gaussian only into the tiles its
// alpha support reaches (tighten_rect) and caches the per-slot intermediates of the
// twist-only adjoint (write_fcache).
//
// Adjoint (k_preprocess_bwd, drop-in): same per-Gaussian/per-view loop; recomputes the
// forward quantities, chains the blend adjoint's per-Gaussian 2D gradients through
// conic, cov2D, the Jacobian, the projection, depth and the SH view direction to (a) the
// left-twist gradient of each view (warp-reduced in FP32, block sums as float pairs,
// per-view sums in FP64) and (b) optionally the map gradients of the drop-in API.
// The batched tracker's twist-only adjoint from the cache is in preprocess_cached.cu.
#include "common.cuh"

namespace {

struct Pre {
    float pc[3], hom[4], pw, mean[2], cov2[3], det, conic[3], radius;
    int rect[4];
    float T0[3], T1[3], J[4];
    int clampx, clampy;
    float dir[3], dirlen, rgb_raw[3], rgb[3];
};

__device__ __forceinline__ void cov3d_from_sr(const float *s_in, const float *q, float mod, float *cov)
{
    float r = q[0], x = q[1], y = q[2], z = q[3];
    float s0 = mod * s_in[0], s1 = mod * s_in[1], s2 = mod * s_in[2];
    float R00 = 1.0f - 2.0f * ((y * y) + (z * z));
    float R01 = 2.0f * ((x * y) - (r * z));
    float R02 = 2.0f * ((x * z) + (r * y));
    float R10 = 2.0f * ((x * y) + (r * z));
    float R11 = 1.0f - 2.0f * ((x * x) + (z * z));
    float R12 = 2.0f * ((y * z) - (r * x));
    float R20 = 2.0f * ((x * z) - (r * y));
    float R21 = 2.0f * ((y * z) + (r * x));
    float R22 = 1.0f - 2.0f * ((x * x) + (y * y));
    float L00 = R00 * s0, L01 = R01 * s1, L02 = R02 * s2;
    float L10 = R10 * s0, L11 = R11 * s1, L12 = R12 * s2;
    float L20 = R20 * s0, L21 = R21 * s1, L22 = R22 * s2;
    cov[0] = ((L00 * L00) + (L01 * L01)) + (L02 * L02);
    cov[1] = ((L00 * L10) + (L01 * L11)) + (L02 * L12);
    cov[2] = ((L00 * L20) + (L01 * L21)) + (L02 * L22);
    cov[3] = ((L10 * L10) + (L11 * L11)) + (L12 * L12);
    cov[4] = ((L10 * L20) + (L11 * L21)) + (L12 * L22);
    cov[5] = ((L20 * L20) + (L21 * L21)) + (L22 * L22);
}

__device__ __forceinline__ void sh_rgb(int deg, const float *sh, float x, float y, float z, float *rgb)
{
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#define S(k) sh[(k) * 3 + c]
        float res = 0.28209479177387814f * S(0);
        if (deg > 0) {
            res = ((res - (0.4886025119029199f * y) * S(1)) + (0.4886025119029199f * z) * S(2))
                  - (0.4886025119029199f * x) * S(3);
            if (deg > 1) {
                float xx = x * x, yy = y * y, zz = z * z;
                float xy = x * y, yz = y * z, xz = x * z;
                res = res + (1.0925484305920792f * xy) * S(4);
                res = res + (-1.0925484305920792f * yz) * S(5);
                res = res + (0.31539156525252005f * ((2.0f * zz - xx) - yy)) * S(6);
                res = res + (-1.0925484305920792f * xz) * S(7);
                res = res + (0.5462742152960396f * (xx - yy)) * S(8);
                if (deg > 2) {
                    res = res + ((-0.5900435899266435f * y) * ((3.0f * xx) - yy)) * S(9);
                    res = res + ((2.890611442640554f * xy) * z) * S(10);
                    res = res + ((-0.4570457994644658f * y) * ((4.0f * zz - xx) - yy)) * S(11);
                    res = res + ((0.3731763325901154f * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy)) * S(12);
                    res = res + ((-0.4570457994644658f * x) * ((4.0f * zz - xx) - yy)) * S(13);
                    res = res + ((1.445305721320277f * z) * (xx - yy)) * S(14);
                    res = res + ((-0.5900435899266435f * x) * (xx - 3.0f * yy)) * S(15);
                }
            }
        }
#undef S
        rgb[c] = res + 0.5f;
    }
}

// Forward preprocessing of one Gaussian in one view (oracle: preprocess_one_f).
__device__ __forceinline__ bool pre_forward(const float *xyz, const float *cov, const float *sh,
                                            int deg, const float *col, const gsevt_view &V, Pre &o)
{
    const float *R = V.R, *t = V.t, *P = V.P, *cp = V.campos;
    float px = xyz[0], py = xyz[1], pz = xyz[2];
    float vx = ((R[0] * px + R[1] * py) + R[2] * pz) + t[0];
    float vy = ((R[3] * px + R[4] * py) + R[5] * pz) + t[1];
    float vz = ((R[6] * px + R[7] * py) + R[8] * pz) + t[2];
    o.pc[0] = vx; o.pc[1] = vy; o.pc[2] = vz;
    if (!(vz > 0.2f)) return false;
#pragma unroll
    for (int i = 0; i < 4; ++i)
        o.hom[i] = ((P[4 * i + 0] * vx + P[4 * i + 1] * vy) + P[4 * i + 2] * vz) + P[4 * i + 3];
    float pw = 1.0f / (o.hom[3] + 0.0000001f);
    o.pw = pw;
    float nx = o.hom[0] * pw, ny = o.hom[1] * pw;
    float limx = 1.3f * V.tanfovx, limy = 1.3f * V.tanfovy;
    float txtz = vx / vz, tytz = vy / vz;
    o.clampx = (txtz < -limx) || (txtz > limx);
    o.clampy = (tytz < -limy) || (tytz > limy);
    float tx = fminf(limx, fmaxf(-limx, txtz)) * vz;
    float ty = fminf(limy, fmaxf(-limy, tytz)) * vz;
    float fx = (float)V.width / (2.0f * V.tanfovx);
    float fy = (float)V.height / (2.0f * V.tanfovy);
    float vz2 = vz * vz;
    float J00 = fx / vz, J02 = -(fx * tx) / vz2, J11 = fy / vz, J12 = -(fy * ty) / vz2;
    o.J[0] = J00; o.J[1] = J02; o.J[2] = J11; o.J[3] = J12;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        o.T0[j] = J00 * R[j] + J02 * R[6 + j];
        o.T1[j] = J11 * R[3 + j] + J12 * R[6 + j];
    }
    float S[9] = {cov[0], cov[1], cov[2], cov[1], cov[3], cov[4], cov[2], cov[4], cov[5]};
    float U0[3], U1[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        U0[j] = (o.T0[0] * S[j] + o.T0[1] * S[3 + j]) + o.T0[2] * S[6 + j];
        U1[j] = (o.T1[0] * S[j] + o.T1[1] * S[3 + j]) + o.T1[2] * S[6 + j];
    }
    float a = (U0[0] * o.T0[0] + U0[1] * o.T0[1]) + U0[2] * o.T0[2];
    float b = (U0[0] * o.T1[0] + U0[1] * o.T1[1]) + U0[2] * o.T1[2];
    float c = (U1[0] * o.T1[0] + U1[1] * o.T1[1]) + U1[2] * o.T1[2];
    a = a + 0.3f;
    c = c + 0.3f;
    o.cov2[0] = a; o.cov2[1] = b; o.cov2[2] = c;
    float det = a * c - b * b;
    o.det = det;
    if (det == 0.0f) return false;
    float det_inv = 1.0f / det;
    o.conic[0] = c * det_inv;
    o.conic[1] = -b * det_inv;
    o.conic[2] = a * det_inv;
    float mid = 0.5f * (a + c);
    float sq = sqrtf(fmaxf(0.1f, mid * mid - det));
    float l1 = mid + sq, l2 = mid - sq;
    float rad = ceilf(3.0f * sqrtf(fmaxf(l1, l2)));
    o.radius = rad;
    float mx = ((nx + 1.0f) * (float)V.width - 1.0f) * 0.5f;
    float my = ((ny + 1.0f) * (float)V.height - 1.0f) * 0.5f;
    o.mean[0] = mx; o.mean[1] = my;
    float gx = (float)V.tiles_x, gy = (float)V.tiles_y;
    o.rect[0] = (int)fminf(gx, fmaxf(0.0f, (mx - rad) / 16.0f));
    o.rect[1] = (int)fminf(gy, fmaxf(0.0f, (my - rad) / 16.0f));
    o.rect[2] = (int)fminf(gx, fmaxf(0.0f, ((mx + rad) + 15.0f) / 16.0f));
    o.rect[3] = (int)fminf(gy, fmaxf(0.0f, ((my + rad) + 15.0f) / 16.0f));
    if (!(rad > 0.0f)) return false;
    if ((o.rect[2] - o.rect[0]) * (o.rect[3] - o.rect[1]) == 0) return false;
    if (col) {
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) { o.rgb_raw[ch] = col[ch]; o.rgb[ch] = col[ch]; }
        o.dir[0] = o.dir[1] = o.dir[2] = 0.0f;
        o.dirlen = 1.0f;
    } else {
        float dx = px - cp[0], dy = py - cp[1], dz = pz - cp[2];
        float len = sqrtf((dx * dx + dy * dy) + dz * dz);
        o.dirlen = len;
        dx = dx / len; dy = dy / len; dz = dz / len;
        o.dir[0] = dx; o.dir[1] = dy; o.dir[2] = dz;
        sh_rgb(deg, sh, dx, dy, dz, o.rgb_raw);
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) o.rgb[ch] = fmaxf(o.rgb_raw[ch], 0.0f);
    }
    return true;
}

__device__ __forceinline__ float grey_of(const float *rgb)
{
    return (0.2989f * rgb[0] + 0.587f * rgb[1]) + 0.114f * rgb[2];
}

// Attributes of one Gaussian, loaded from the packed planes or the raw drop-in tensors.
struct Attr {
    float xyz[3], opac, cov[6], sh[48], col[3];
    bool has_col;
};

__device__ __forceinline__ void load_attr(const gsevt_map &M, int g, Attr &a)
{
    int deg = M.sh_degree;
    int ncoef = (deg + 1) * (deg + 1);
    a.has_col = false;
    if (M.packed) {
        const float4 *pl = (const float4 *)M.packed;
        size_t n = (size_t)M.n;
        float4 p0 = __ldg(pl + g), p1 = __ldg(pl + n + g), p2 = __ldg(pl + 2 * n + g);
        a.xyz[0] = p0.x; a.xyz[1] = p0.y; a.xyz[2] = p0.z; a.opac = p0.w;
        a.cov[0] = p1.x; a.cov[1] = p1.y; a.cov[2] = p1.z; a.cov[3] = p1.w;
        a.cov[4] = p2.x; a.cov[5] = p2.y;
#pragma unroll
        for (int j = 0; j < 12; ++j) {
            float4 s = (j * 4 < ncoef * 3) ? __ldg(pl + (3 + j) * n + g) : make_float4(0, 0, 0, 0);
            a.sh[4 * j] = s.x; a.sh[4 * j + 1] = s.y; a.sh[4 * j + 2] = s.z; a.sh[4 * j + 3] = s.w;
        }
        return;
    }
    a.xyz[0] = __ldg(M.xyz + 3 * g); a.xyz[1] = __ldg(M.xyz + 3 * g + 1); a.xyz[2] = __ldg(M.xyz + 3 * g + 2);
    a.opac = __ldg(M.opacity + g);
    if (M.cov3d) {
#pragma unroll
        for (int k = 0; k < 6; ++k) a.cov[k] = __ldg(M.cov3d + 6 * g + k);
    } else {
        float s[3] = {__ldg(M.scales + 3 * g), __ldg(M.scales + 3 * g + 1), __ldg(M.scales + 3 * g + 2)};
        float q[4] = {__ldg(M.rotations + 4 * g), __ldg(M.rotations + 4 * g + 1),
                      __ldg(M.rotations + 4 * g + 2), __ldg(M.rotations + 4 * g + 3)};
        cov3d_from_sr(s, q, M.scale_modifier, a.cov);
    }
    if (M.colors) {
        a.has_col = true;
#pragma unroll
        for (int k = 0; k < 3; ++k) a.col[k] = __ldg(M.colors + 3 * g + k);
#pragma unroll
        for (int k = 0; k < 48; ++k) a.sh[k] = 0.0f;
    } else {
        const float *s = M.shs + (size_t)g * M.sh_coeffs * 3;
#pragma unroll
        for (int k = 0; k < 48; ++k) a.sh[k] = (k < ncoef * 3) ? __ldg(s + k) : 0.0f;
    }
}

__device__ __forceinline__ void sh_dir_grad(int deg, const float *w, float x, float y, float z, float *g);

// Forward intermediates of one visible slot that the twist-only adjoint needs, so that it
// reads 96 bytes per slot instead of the map attributes and the recomputed forward:
//   c0 {cov2 a, b, c, det}, c1 {T0 S (3), T1 S x}, c2 {T1 S y, z, J00, J02},
//   c3 {J11, J12, pc x, pc y}, c4 {pc z, pw, hom x, hom y}, c5 {U (3), clamp flags},
// with S the world covariance, T0, T1 the rows of J W, and U the direction term of the
// grey colour: for a grey gradient g, the SH view-direction gradient of the slot is
// g U, U = (D - d (d.D)) / |x - campos|, D = sum_k g_k dY_k/dd,
// g_k = sum over unclamped channels c of w_c sh_kc (the grey weights w): the grey colour
// is linear in the SH coefficients while no channel clamps, so the map's SH are folded
// into U once in the forward.
__device__ __forceinline__ void write_fcache(float4 *dst, const Pre &o, const float *cov, const float *sh,
                                             int sh_degree, bool has_col)
{
    // gradient-only quantities: fused multiply-adds (see sh_dir_grad)
    float T0S[3], T1S[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const float Sj[3] = {cov[j == 0 ? 0 : (j == 1 ? 1 : 2)], cov[j == 0 ? 1 : (j == 1 ? 3 : 4)],
                             cov[j == 0 ? 2 : (j == 1 ? 4 : 5)]};
        T0S[j] = fmaf(o.T0[2], Sj[2], fmaf(o.T0[1], Sj[1], o.T0[0] * Sj[0]));
        T1S[j] = fmaf(o.T1[2], Sj[2], fmaf(o.T1[1], Sj[1], o.T1[0] * Sj[0]));
    }
    float U[3] = {0.0f, 0.0f, 0.0f};
    if (!has_col) {
        const float wc[3] = {o.rgb_raw[0] < 0.0f ? 0.0f : 0.2989f, o.rgb_raw[1] < 0.0f ? 0.0f : 0.587f,
                             o.rgb_raw[2] < 0.0f ? 0.0f : 0.114f};
        float gk[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) gk[k] = fmaf(wc[2], sh[3 * k + 2], fmaf(wc[1], sh[3 * k + 1], wc[0] * sh[3 * k]));
        float D[3];
        sh_dir_grad(sh_degree, gk, o.dir[0], o.dir[1], o.dir[2], D);
        const float dd = fmaf(o.dir[2], D[2], fmaf(o.dir[1], D[1], o.dir[0] * D[0]));
        const float il = 1.0f / o.dirlen;
#pragma unroll
        for (int j = 0; j < 3; ++j) U[j] = fmaf(-o.dir[j], dd, D[j]) * il;
    }
    dst[0] = make_float4(o.cov2[0], o.cov2[1], o.cov2[2], o.det);
    dst[1] = make_float4(T0S[0], T0S[1], T0S[2], T1S[0]);
    dst[2] = make_float4(T1S[1], T1S[2], o.J[0], o.J[1]);
    dst[3] = make_float4(o.J[2], o.J[3], o.pc[0], o.pc[1]);
    dst[4] = make_float4(o.pc[2], o.pw, o.hom[0], o.hom[1]);
    dst[5] = make_float4(U[0], U[1], U[2], __int_as_float((o.clampx ? 1 : 0) | (o.clampy ? 2 : 0)));
}

// Batched-tracker frames (those with the adjoint cache) bin a Gaussian only into the
// tiles that its alpha support can reach: the reference's 3-sigma tile rectangle is
// intersected with the tiles holding pixels of a conservative box of the support.  A
// pixel blends the Gaussian only if alpha = min(0.99, o exp(power)) >= 1/255, i.e.
// -power <= tau = ln(255 o); in exact arithmetic -power = d^T M d / 2 for the conic M, and
// the FP32 evaluation deviates by less than 1e-6 tr(M) |d|^2, so every such pixel lies in
// the box of d^T (M/2 - 1e-6 tr(M) I) d <= tau (1 + 1e-4) + 1e-3, widened by 0.1 % + 0.5
// px.  Dropped tiles hold no pixel that could blend the Gaussian, so every tile's image,
// transmittance and gradients are unchanged; only the per-tile list indices (contributor
// counts, which these frames do not output) differ from the full rectangle's.
__device__ __forceinline__ void tighten_rect(Pre &o, float opac, const gsevt_view &V)
{
    if (!(opac >= (1.0f / 255.0f) * 0.999f)) {  // no pixel can pass the alpha test
        o.rect[2] = o.rect[0];
        return;
    }
    const float tau = logf(255.0f * opac) * 1.0001f + 1e-3f;
    const float Bx = o.conic[0], By = o.conic[1], Bz = o.conic[2];
    const float g = 1e-6f * (fabsf(Bx) + fabsf(Bz));
    const float a = 0.5f * Bx - g, b = 0.5f * By, c = 0.5f * Bz - g;
    const float det = a * c - b * b;
    if (!(a > 0.0f && c > 0.0f && det > 0.0f && tau > -1e29f && tau < 1e29f)) return;  // keep the rectangle
    const float hx = sqrtf(fmaxf(tau, 0.0f) * c / det) * 1.001f + 0.5f;
    const float hy = sqrtf(fmaxf(tau, 0.0f) * a / det) * 1.001f + 0.5f;
    const float gx = (float)V.tiles_x, gy = (float)V.tiles_y;
    const int bx0 = (int)fminf(gx, fmaxf(0.0f, floorf((o.mean[0] - hx) * (1.0f / 16.0f))));
    const int bx1 = (int)fminf(gx, fmaxf(0.0f, floorf((o.mean[0] + hx) * (1.0f / 16.0f)) + 1.0f));
    const int by0 = (int)fminf(gy, fmaxf(0.0f, floorf((o.mean[1] - hy) * (1.0f / 16.0f))));
    const int by1 = (int)fminf(gy, fmaxf(0.0f, floorf((o.mean[1] + hy) * (1.0f / 16.0f)) + 1.0f));
    o.rect[0] = max(o.rect[0], bx0);
    o.rect[1] = max(o.rect[1], by0);
    o.rect[2] = min(o.rect[2], bx1);
    o.rect[3] = min(o.rect[3], by1);
}

struct FwdParams {
    const gsevt_view *views;
    const gsevt_map *maps;
    int num_maps;
    int rgb;
    Workspace ws;
    int32_t *radii;
};

__global__ void __launch_bounds__(GS_BLOCK, 2) k_preprocess_fwd(FwdParams p)
{
    __shared__ gsevt_map M;
    __shared__ gsevt_view V;
    __shared__ uint32_t wsum[GS_BLOCK / 32];
    int b = blockIdx.x;
    if (threadIdx.x == 0) M = p.maps[gs_find_map(p.maps, p.num_maps, b)];
    __syncthreads();
    int gb = b - M.block_offset;
    int g = gb * GS_BLOCK + threadIdx.x;
    bool valid = g < M.n;
    Attr a;
    if (valid) load_attr(M, g, a);
    for (int vl = 0; vl < M.num_views; ++vl) {
        __syncthreads();
        if (threadIdx.x < sizeof(gsevt_view) / 4)
            ((uint32_t *)&V)[threadIdx.x] = ((const uint32_t *)(p.views + M.first_view + vl))[threadIdx.x];
        __syncthreads();
        uint32_t touched = 0;
        if (valid) {
            Pre o;
            // a skipped view (a finished tracking problem) culls every Gaussian
            bool vis = !V.skip && pre_forward(a.xyz, a.cov, a.sh, M.sh_degree, a.has_col ? a.col : nullptr, V, o);
            size_t vg = (size_t)V.vg_offset + g;
            if (vis && p.ws.fcache) tighten_rect(o, a.opac, V);
            vis = vis && o.rect[2] > o.rect[0] && o.rect[3] > o.rect[1];
            if (vis) {
                touched = (uint32_t)((o.rect[2] - o.rect[0]) * (o.rect[3] - o.rect[1]));
                float grey = grey_of(o.rgb);
                p.ws.bin[vg] = make_int4((int)touched, o.rect[0] | (o.rect[1] << 16),
                                         o.rect[2] | (o.rect[3] << 16), __float_as_int(o.pc[2]));
                p.ws.rec[2 * vg] = make_float4(o.mean[0], o.mean[1], o.pc[2], grey);
                p.ws.rec[2 * vg + 1] = make_float4(o.conic[0], o.conic[1], o.conic[2], a.opac);
                if (p.rgb) p.ws.recC[vg] = make_float4(o.rgb[0], o.rgb[1], o.rgb[2], 0.0f);
                if (p.ws.fcache) write_fcache(p.ws.fcache + vg * GS_FCACHE, o, a.cov, a.sh, M.sh_degree, a.has_col);
            } else {
                p.ws.bin[vg] = make_int4(0, 0, 0, 0);
            }
            if (p.radii) p.radii[vg] = vis ? (int)fminf(o.radius, 1073741824.0f) : 0;
        }
        // per (view, block) count of visible slots for the compaction scan
        uint32_t s = touched > 0 ? 1u : 0u;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t tot = 0;
            for (int w = 0; w < GS_BLOCK / 32; ++w) tot += wsum[w];
            p.ws.vis_sums[V.sb_offset + gb] = tot;
        }
    }
}

__global__ void k_pack_map(int n, const float *xyz, const float *opacity, const float *scales,
                           const float *rotations, const float *cov3d, const float *shs,
                           int sh_coeffs, float mod, float4 *out)
{
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    size_t N = (size_t)n;
    out[g] = make_float4(xyz[3 * g], xyz[3 * g + 1], xyz[3 * g + 2], opacity[g]);
    float cov[6];
    if (cov3d) {
        for (int k = 0; k < 6; ++k) cov[k] = cov3d[6 * g + k];
    } else {
        float s[3] = {scales[3 * g], scales[3 * g + 1], scales[3 * g + 2]};
        float q[4] = {rotations[4 * g], rotations[4 * g + 1], rotations[4 * g + 2], rotations[4 * g + 3]};
        cov3d_from_sr(s, q, mod, cov);
    }
    out[N + g] = make_float4(cov[0], cov[1], cov[2], cov[3]);
    out[2 * N + g] = make_float4(cov[4], cov[5], 0.0f, 0.0f);
    const float *s = shs + (size_t)g * sh_coeffs * 3;
    int have = sh_coeffs * 3;
    for (int j = 0; j < 12; ++j) {
        float v[4];
        for (int k = 0; k < 4; ++k) {
            int i = 4 * j + k;
            v[k] = (i < have && i < 48) ? s[i] : 0.0f;
        }
        out[(3 + j) * N + g] = make_float4(v[0], v[1], v[2], v[3]);
    }
}

// ----------------------------------------------------------------- adjoint -------
struct BwdParams {
    const gsevt_view *views;
    const gsevt_map *maps;
    int num_maps;
    int num_views;
    int rgb;
    Workspace ws;
    const gsevt_map_grads *grads;  // device array [num_maps] or nullptr
};

// SH basis times weights: returns sum_k w[k] * dY_k/d(x,y,z) (x,y,z treated as free).
// Gradient arithmetic only, so the terms are accumulated with explicit fused multiply-adds
// (this file is otherwise compiled without contraction, for the forward's bit parity).
__device__ __forceinline__ void sh_dir_grad(int deg, const float *w, float x, float y, float z, float *g)
{
    const float C1 = 0.4886025119029199f;
    g[0] = g[1] = g[2] = 0.0f;
    if (deg < 1) return;
    float g0 = -C1 * w[3], g1 = -C1 * w[1], g2 = C1 * w[2];
    if (deg >= 2) {
        const float C20 = 1.0925484305920792f, C21 = -1.0925484305920792f, C22 = 0.31539156525252005f,
                    C23 = -1.0925484305920792f, C24 = 0.5462742152960396f;
        g0 = fmaf(C20 * y, w[4], g0);
        g0 = fmaf((-2.0f * C22) * x, w[6], g0);
        g0 = fmaf(C23 * z, w[7], g0);
        g0 = fmaf((2.0f * C24) * x, w[8], g0);
        g1 = fmaf(C20 * x, w[4], g1);
        g1 = fmaf(C21 * z, w[5], g1);
        g1 = fmaf((-2.0f * C22) * y, w[6], g1);
        g1 = fmaf((-2.0f * C24) * y, w[8], g1);
        g2 = fmaf(C21 * y, w[5], g2);
        g2 = fmaf((4.0f * C22) * z, w[6], g2);
        g2 = fmaf(C23 * x, w[7], g2);
        if (deg >= 3) {
            const float C30 = -0.5900435899266435f, C31 = 2.890611442640554f, C32 = -0.4570457994644658f,
                        C33 = 0.3731763325901154f, C34 = -0.4570457994644658f, C35 = 1.445305721320277f,
                        C36 = -0.5900435899266435f;
            const float xx = x * x, yy = y * y, zz = z * z;
            const float xy = x * y, xz = x * z, yz = y * z;
            const float d3 = 3.0f * (xx - yy);
            g0 = fmaf((6.0f * C30) * xy, w[9], g0);
            g0 = fmaf(C31 * yz, w[10], g0);
            g0 = fmaf((-2.0f * C32) * xy, w[11], g0);
            g0 = fmaf((-6.0f * C33) * xz, w[12], g0);
            g0 = fmaf(C34 * fmaf(4.0f, zz, fmaf(-3.0f, xx, -yy)), w[13], g0);
            g0 = fmaf((2.0f * C35) * xz, w[14], g0);
            g0 = fmaf(C36 * d3, w[15], g0);
            g1 = fmaf(C30 * d3, w[9], g1);
            g1 = fmaf(C31 * xz, w[10], g1);
            g1 = fmaf(C32 * fmaf(4.0f, zz, fmaf(-3.0f, yy, -xx)), w[11], g1);
            g1 = fmaf((-6.0f * C33) * yz, w[12], g1);
            g1 = fmaf((-2.0f * C34) * xy, w[13], g1);
            g1 = fmaf((-2.0f * C35) * yz, w[14], g1);
            g1 = fmaf((-6.0f * C36) * xy, w[15], g1);
            g2 = fmaf(C31 * xy, w[10], g2);
            g2 = fmaf((8.0f * C32) * yz, w[11], g2);
            g2 = fmaf(C33 * fmaf(6.0f, zz, -3.0f * (xx + yy)), w[12], g2);
            g2 = fmaf((8.0f * C34) * xz, w[13], g2);
            g2 = fmaf(C35 * (xx - yy), w[14], g2);
        }
    }
    g[0] = g0;
    g[1] = g1;
    g[2] = g2;
}

__device__ __forceinline__ void sh_basis(int deg, float x, float y, float z, float *Y)
{
    const float C0 = 0.28209479177387814f, C1 = 0.4886025119029199f;
#pragma unroll
    for (int k = 0; k < 16; ++k) Y[k] = 0.0f;
    Y[0] = C0;
    if (deg < 1) return;
    Y[1] = -C1 * y; Y[2] = C1 * z; Y[3] = -C1 * x;
    if (deg < 2) return;
    float xx = x * x, yy = y * y, zz = z * z;
    Y[4] = 1.0925484305920792f * x * y;
    Y[5] = -1.0925484305920792f * y * z;
    Y[6] = 0.31539156525252005f * (2.0f * zz - xx - yy);
    Y[7] = -1.0925484305920792f * x * z;
    Y[8] = 0.5462742152960396f * (xx - yy);
    if (deg < 3) return;
    Y[9] = -0.5900435899266435f * y * (3.0f * xx - yy);
    Y[10] = 2.890611442640554f * x * y * z;
    Y[11] = -0.4570457994644658f * y * (4.0f * zz - xx - yy);
    Y[12] = 0.3731763325901154f * z * (2.0f * zz - 3.0f * xx - 3.0f * yy);
    Y[13] = -0.4570457994644658f * x * (4.0f * zz - xx - yy);
    Y[14] = 1.445305721320277f * z * (xx - yy);
    Y[15] = -0.5900435899266435f * x * (xx - 3.0f * yy);
}

template <bool MAPGRAD>
__global__ void __launch_bounds__(GS_BLOCK, MAPGRAD ? 1 : 2) k_preprocess_bwd(BwdParams p)
{
    __shared__ gsevt_map M;
    __shared__ gsevt_view V;
    __shared__ float wpart[GS_BLOCK / 32][6];
    int b = blockIdx.x;
    if (gs_sort_timed_out(p.ws.status)) return;  // no blend adjoint ran (uniform)
    if (threadIdx.x == 0) M = p.maps[gs_find_map(p.maps, p.num_maps, b)];
    __syncthreads();
    int m = gs_find_map(p.maps, p.num_maps, b);
    int gb = b - M.block_offset;
    int g = gb * GS_BLOCK + threadIdx.x;
    bool valid = g < M.n;
    Attr a;
    if (valid) load_attr(M, g, a);
    // map gradient accumulators (summed over the views of this map)
    float gm3[3] = {0, 0, 0}, gm2[2] = {0, 0}, gop = 0.0f, gcov[6] = {0, 0, 0, 0, 0, 0};
    float gsh[48];
    float gcol[3] = {0, 0, 0};
    if (MAPGRAD) {
#pragma unroll
        for (int k = 0; k < 48; ++k) gsh[k] = 0.0f;
    }
    for (int vl = 0; vl < M.num_views; ++vl) {
        __syncthreads();
        if (threadIdx.x < sizeof(gsevt_view) / 4)
            ((uint32_t *)&V)[threadIdx.x] = ((const uint32_t *)(p.views + M.first_view + vl))[threadIdx.x];
        __syncthreads();
        float xi[6] = {0, 0, 0, 0, 0, 0};
        size_t vg = (size_t)V.vg_offset + g;
        if (valid && p.ws.bin[vg].x > 0) {
            Pre o;
            pre_forward(a.xyz, a.cov, a.sh, M.sh_degree, a.has_col ? a.col : nullptr, V, o);
            float4 GA = p.ws.gradA[vg], GB = p.ws.gradB[vg];
            float4 GC = p.rgb ? p.ws.gradC[vg] : make_float4(0, 0, 0, 0);
            float q_mean[2] = {GA.x, GA.y};
            float gCa = GA.z, gCb = GA.w, gCc = GB.x;
            float a2 = o.cov2[0], b2 = o.cov2[1], c2 = o.cov2[2], det = o.det;
            float d2 = det * det;
            float ga = (gCa * (-c2 * c2) + gCb * (b2 * c2) + gCc * (-b2 * b2)) / d2;
            float gb_ = (gCa * (2.0f * b2 * c2) + gCb * (-(a2 * c2 + b2 * b2)) + gCc * (2.0f * a2 * b2)) / d2;
            float gc = (gCa * (-b2 * b2) + gCb * (a2 * b2) + gCc * (-a2 * a2)) / d2;
            float Gs00 = ga, Gs01 = 0.5f * gb_, Gs11 = gc;
            float S[3][3] = {{a.cov[0], a.cov[1], a.cov[2]}, {a.cov[1], a.cov[3], a.cov[4]}, {a.cov[2], a.cov[4], a.cov[5]}};
            float GT0[3], GT1[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                GT0[j] = Gs00 * o.T0[j] + Gs01 * o.T1[j];
                GT1[j] = Gs01 * o.T0[j] + Gs11 * o.T1[j];
            }
            float gT0[3], gT1[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                gT0[j] = 2.0f * (GT0[0] * S[0][j] + GT0[1] * S[1][j] + GT0[2] * S[2][j]);
                gT1[j] = 2.0f * (GT1[0] * S[0][j] + GT1[1] * S[1][j] + GT1[2] * S[2][j]);
            }
            const float *R = V.R;
            float J00 = o.J[0], J02 = o.J[1], J11 = o.J[2], J12 = o.J[3];
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
            float fx = (float)V.width / (2.0f * V.tanfovx), fy = (float)V.height / (2.0f * V.tanfovy);
            float vx = o.pc[0], vy = o.pc[1], vz = o.pc[2];
            float ivz = 1.0f / vz, ivz2 = ivz * ivz, ivz3 = ivz2 * ivz;
            float gpc[3] = {0, 0, 0};
            gpc[2] += gJ00 * (-fx * ivz2) + gJ11 * (-fy * ivz2);
            if (!o.clampx) { gpc[0] += gJ02 * (-fx * ivz2); gpc[2] += gJ02 * (2.0f * fx * vx * ivz3); }
            else { gpc[2] += gJ02 * (-J02 * ivz); }
            if (!o.clampy) { gpc[1] += gJ12 * (-fy * ivz2); gpc[2] += gJ12 * (2.0f * fy * vy * ivz3); }
            else { gpc[2] += gJ12 * (-J12 * ivz); }
            float gnx = q_mean[0] * 0.5f * (float)V.width, gny = q_mean[1] * 0.5f * (float)V.height;
            float pw = o.pw;
            float gh0 = gnx * pw, gh1 = gny * pw, gh3 = -(gnx * o.hom[0] + gny * o.hom[1]) * pw * pw;
#pragma unroll
            for (int j = 0; j < 3; ++j)
                gpc[j] += V.P[j] * gh0 + V.P[4 + j] * gh1 + V.P[12 + j] * gh3;
            gpc[2] += GB.w;
            // colour -> SH coefficients and view direction
            float grgb[3];
            if (p.rgb) { grgb[0] = GB.z; grgb[1] = GC.x; grgb[2] = GC.y; }
            else { grgb[0] = 0.2989f * GB.z; grgb[1] = 0.587f * GB.z; grgb[2] = 0.114f * GB.z; }
            float gu[3] = {0, 0, 0};
            if (a.has_col) {
                if (MAPGRAD) { gcol[0] += grgb[0]; gcol[1] += grgb[1]; gcol[2] += grgb[2]; }
            } else {
                float gr[3];
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) gr[ch] = (o.rgb_raw[ch] < 0.0f) ? 0.0f : grgb[ch];
                float wk[16];
#pragma unroll
                for (int k = 0; k < 16; ++k)
                    wk[k] = gr[0] * a.sh[3 * k] + gr[1] * a.sh[3 * k + 1] + gr[2] * a.sh[3 * k + 2];
                float gdir[3];
                sh_dir_grad(M.sh_degree, wk, o.dir[0], o.dir[1], o.dir[2], gdir);
                float dd = o.dir[0] * gdir[0] + o.dir[1] * gdir[1] + o.dir[2] * gdir[2];
                float il = 1.0f / o.dirlen;
#pragma unroll
                for (int j = 0; j < 3; ++j) gu[j] = (gdir[j] - o.dir[j] * dd) * il;
                if (MAPGRAD) {
                    float Y[16];
                    sh_basis(M.sh_degree, o.dir[0], o.dir[1], o.dir[2], Y);
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        gsh[3 * k] += gr[0] * Y[k];
                        gsh[3 * k + 1] += gr[1] * Y[k];
                        gsh[3 * k + 2] += gr[2] * Y[k];
                    }
                }
            }
            // left twist of the view: rho then theta
            float Rgu0 = R[0] * gu[0] + R[1] * gu[1] + R[2] * gu[2];
            float Rgu1 = R[3] * gu[0] + R[4] * gu[1] + R[5] * gu[2];
            float Rgu2 = R[6] * gu[0] + R[7] * gu[1] + R[8] * gu[2];
            xi[0] = gpc[0] + Rgu0;
            xi[1] = gpc[1] + Rgu1;
            xi[2] = gpc[2] + Rgu2;
            float M12 = R[3] * gW[2][0] + R[4] * gW[2][1] + R[5] * gW[2][2];
            float M21 = R[6] * gW[1][0] + R[7] * gW[1][1] + R[8] * gW[1][2];
            float M20 = R[6] * gW[0][0] + R[7] * gW[0][1] + R[8] * gW[0][2];
            float M02 = R[0] * gW[2][0] + R[1] * gW[2][1] + R[2] * gW[2][2];
            float M01 = R[0] * gW[1][0] + R[1] * gW[1][1] + R[2] * gW[1][2];
            float M10 = R[3] * gW[0][0] + R[4] * gW[0][1] + R[5] * gW[0][2];
            xi[3] = (vy * gpc[2] - vz * gpc[1]) + (M12 - M21);
            xi[4] = (vz * gpc[0] - vx * gpc[2]) + (M20 - M02);
            xi[5] = (vx * gpc[1] - vy * gpc[0]) + (M01 - M10);
            if (MAPGRAD) {
                gm2[0] += gnx; gm2[1] += gny;
                gop += GB.y;
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    gm3[j] += (R[j] * gpc[0] + R[3 + j] * gpc[1] + R[6 + j] * gpc[2]) + gu[j];
                // dL/dSigma = T^T Gs T (symmetric); 6-vector with doubled off-diagonals
                float gS00 = o.T0[0] * GT0[0] + o.T1[0] * GT1[0];
                float gS01 = o.T0[0] * GT0[1] + o.T1[0] * GT1[1];
                float gS02 = o.T0[0] * GT0[2] + o.T1[0] * GT1[2];
                float gS11 = o.T0[1] * GT0[1] + o.T1[1] * GT1[1];
                float gS12 = o.T0[1] * GT0[2] + o.T1[1] * GT1[2];
                float gS22 = o.T0[2] * GT0[2] + o.T1[2] * GT1[2];
                gcov[0] += gS00; gcov[1] += 2.0f * gS01; gcov[2] += 2.0f * gS02;
                gcov[3] += gS11; gcov[4] += 2.0f * gS12; gcov[5] += gS22;
            }
        }
        // reduce the view's twist gradient: FP32 within the warp, the warp sums added as a
        // float pair (error-free FP32 additions), stored unevaluated as (hi, lo)
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const float sm = warp_sum(xi[k]);
            if ((threadIdx.x & 31) == 0) wpart[threadIdx.x >> 5][k] = sm;
        }
        __syncthreads();
        if (threadIdx.x < 6) {
            FP2 sm;
            for (int w = 0; w < GS_BLOCK / 32; ++w) sm.add(wpart[w][threadIdx.x], 0.0f);
            ((float2 *)p.ws.xi_part)[(size_t)(V.sb_offset + gb) * 6 + threadIdx.x] = make_float2(sm.hi, sm.lo);
        }
    }
    if (MAPGRAD && valid && p.grads) {
        gsevt_map_grads G = p.grads[m];
        if (G.means3d) { G.means3d[3 * g] = gm3[0]; G.means3d[3 * g + 1] = gm3[1]; G.means3d[3 * g + 2] = gm3[2]; }
        if (G.means2d) { G.means2d[3 * g] = gm2[0]; G.means2d[3 * g + 1] = gm2[1]; G.means2d[3 * g + 2] = 0.0f; }
        if (G.opacity) G.opacity[g] = gop;
        if (G.cov3d)
            for (int k = 0; k < 6; ++k) G.cov3d[6 * g + k] = gcov[k];
        if (G.colors) { G.colors[3 * g] = gcol[0]; G.colors[3 * g + 1] = gcol[1]; G.colors[3 * g + 2] = gcol[2]; }
        if (G.shs) {
            float *o = G.shs + (size_t)g * M.sh_coeffs * 3;
            for (int k = 0; k < M.sh_coeffs * 3; ++k) o[k] = k < 48 ? gsh[k] : 0.0f;
        }
        if ((G.scales || G.rotations) && M.scales && M.rotations) {
            // Sigma = L L^T, L = Rq diag(s * mod)
            float gS[3][3] = {{gcov[0], 0.5f * gcov[1], 0.5f * gcov[2]},
                              {0.5f * gcov[1], gcov[3], 0.5f * gcov[4]},
                              {0.5f * gcov[2], 0.5f * gcov[4], gcov[5]}};
            float r = M.rotations[4 * g], x = M.rotations[4 * g + 1], y = M.rotations[4 * g + 2], z = M.rotations[4 * g + 3];
            float Rq[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)},
                              {2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)},
                              {2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)}};
            float mod = M.scale_modifier;
            float s[3] = {mod * M.scales[3 * g], mod * M.scales[3 * g + 1], mod * M.scales[3 * g + 2]};
            float gL[3][3];
            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < 3; ++k) {
                    float acc = 0;
                    for (int j = 0; j < 3; ++j) acc += 2.0f * gS[i][j] * Rq[j][k] * s[k];
                    gL[i][k] = acc;
                }
            if (G.scales)
                for (int k = 0; k < 3; ++k) {
                    float acc = 0;
                    for (int i = 0; i < 3; ++i) acc += gL[i][k] * Rq[i][k];
                    G.scales[3 * g + k] = acc * mod;
                }
            if (G.rotations) {
                float gR[3][3];
                for (int i = 0; i < 3; ++i)
                    for (int k = 0; k < 3; ++k) gR[i][k] = gL[i][k] * s[k];
                G.rotations[4 * g] = 2 * z * (gR[1][0] - gR[0][1]) + 2 * y * (gR[0][2] - gR[2][0]) + 2 * x * (gR[2][1] - gR[1][2]);
                G.rotations[4 * g + 1] = 2 * y * (gR[0][1] + gR[1][0]) + 2 * z * (gR[0][2] + gR[2][0]) + 2 * r * (gR[2][1] - gR[1][2]) - 4 * x * (gR[1][1] + gR[2][2]);
                G.rotations[4 * g + 2] = 2 * x * (gR[0][1] + gR[1][0]) + 2 * r * (gR[0][2] - gR[2][0]) + 2 * z * (gR[1][2] + gR[2][1]) - 4 * y * (gR[0][0] + gR[2][2]);
                G.rotations[4 * g + 3] = 2 * r * (gR[1][0] - gR[0][1]) + 2 * x * (gR[0][2] + gR[2][0]) + 2 * y * (gR[1][2] + gR[2][1]) - 4 * z * (gR[0][0] + gR[1][1]);
            }
        }
    }
}


// per view: xi[v] = sum over the view's scan blocks of xi_part, in a fixed order (FP64)
__global__ void k_xi_reduce(const gsevt_view *views, const gsevt_map *maps, Workspace ws, int num_views,
                            double *xi_out)
{
    int v = blockIdx.x;
    if (v >= num_views) return;
    gsevt_view V = views[v];
    int nb = (maps[V.map].n + GS_BLOCK - 1) / GS_BLOCK;
    __shared__ double part[GS_BLOCK / 32][6];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
        for (int k = 0; k < 6; ++k) {
            const float2 e = ((const float2 *)ws.xi_part)[(size_t)(V.sb_offset + i) * 6 + k];
            acc[k] += (double)e.x + (double)e.y;
        }
    for (int k = 0; k < 6; ++k) {
        double s = warp_sum_d(acc[k]);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5][k] = s;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) s += part[w][threadIdx.x];
        ws.xi[v * 6 + threadIdx.x] = s;
        if (xi_out) xi_out[v * 6 + threadIdx.x] = s;
    }
}

}  // namespace

// ------------------------------------------------------------------ launchers ----
int gs_launch_preprocess_fwd(const gsevt_frame *f, const Workspace &ws, cudaStream_t s)
{
    FwdParams p;
    p.views = f->views;
    p.maps = f->maps;
    p.num_maps = f->L.num_maps;
    p.rgb = f->L.channels == 3;
    p.ws = ws;
    p.radii = f->radii;
    if (f->L.preprocess_blocks <= 0) return GSEVT_OK;
    k_preprocess_fwd<<<f->L.preprocess_blocks, GS_BLOCK, 0, s>>>(p);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}


// reduce = false leaves the per-view sums to the caller (the batched tracker's finalize
// kernel reduces the partials itself)
int gs_launch_preprocess_bwd(const gsevt_frame *f, const Workspace &ws, const gsevt_map_grads *grads_dev,
                             double *xi_out, cudaStream_t s, bool reduce)
{
    BwdParams p;
    p.views = f->views;
    p.maps = f->maps;
    p.num_maps = f->L.num_maps;
    p.num_views = f->L.num_views;
    p.rgb = f->L.channels == 3;
    p.ws = ws;
    p.grads = grads_dev;
    if (f->L.preprocess_blocks > 0) {
        if (grads_dev) k_preprocess_bwd<true><<<f->L.preprocess_blocks, GS_BLOCK, 0, s>>>(p);
        else k_preprocess_bwd<false><<<f->L.preprocess_blocks, GS_BLOCK, 0, s>>>(p);
        GS_CUDA_CHECK();
    }
    if (reduce) k_xi_reduce<<<f->L.num_views, GS_BLOCK, 0, s>>>(f->views, f->maps, ws, f->L.num_views, xi_out);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

extern "C" int gsevt_pack_map(int32_t n, const float *xyz, const float *opacity, const float *scales,
                              const float *rotations, const float *cov3d, const float *shs,
                              int32_t sh_coeffs, float scale_modifier, void *packed, gsevt_stream_t stream)
{
    GS_ENTRY();
    if (n < 0 || !xyz || !opacity || !shs || !packed || sh_coeffs <= 0) return GSEVT_ERR_ARG;
    if (!cov3d && (!scales || !rotations)) return GSEVT_ERR_ARG;
    if (((uintptr_t)packed & 15) != 0) return GSEVT_ERR_ARG;
    if (n == 0) return GSEVT_OK;
    k_pack_map<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(n, xyz, opacity, scales, rotations, cov3d, shs,
                                                                  sh_coeffs, scale_modifier, (float4 *)packed);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}
