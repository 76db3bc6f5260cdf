/*
 * gsevt CPU oracle — TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm may
 * load this library; the product path never does.
 *
 * What it restates, and how far parity is pinned:
 *   - The rasterizer's native source (submodule diff-gaussian-rasterization-vwRT,
 *     .gitmodules:1-3, pinned version unknown) is ABSENT from the reference tree.
 *     Its contract is known only from the call sites
 *     gaussian_splatting/gaussian_renderer/__init__.py:313-383.  Projection, EWA
 *     covariance, tile binning, front-to-back blending and the adjoint restate the
 *     published 3D Gaussian Splatting method (Kerbl et al., SIGGRAPH 2023; EWA
 *     splatting, Zwicker et al. 2001).  PARITY UNPINNED for those stages: there is
 *     no reference output to compare against.  Sub-steps that live in the reference's
 *     own Python (SH polynomials, cov3D, camera matrices, grey, loss) are pinned by
 *     the golden fixtures under tests/golden/, generated from the reference Python.
 *   - The FP32 functions (or_preprocess, or_duplicate, or_sort_pairs, or_ranges,
 *     or_blend_fwd) fix the operation order bit for bit; the CUDA kernels follow it,
 *     so keys, sort order, tile ranges, radii and images compare bit-exactly.
 *   - The FP64 functions evaluate the same formulas in double along the contributor
 *     lists recorded by the FP32 forward ("frozen decisions"), so that central
 *     finite differences of the loss are well defined and the analytic FP64 gradient
 *     can be checked against them.
 *   - Pose algebra lives in oracle/pose.py (restating utils/pose.py and
 *     utils/render_camera/camera.py); events in or_event_frame below (restating
 *     utils/event_camera/event.py:116-128).
 *
 * Build: oracle/build_oracle.py (gcc -O2 -ffp-contract=off -fopenmp -shared).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define TILE 16

/* ---------------------------------------------------------------- exp -------- */
/* The blend's weight in base 2 (the CUDA blends' gs_log2_conic / gs_power2 / gs_exp2f):
 * the conic (cx, cy, cz) scaled to K = (-log2(e)/2 cx, -log2(e) cy, -log2(e)/2 cz), the
 * exponent y = Kx dx^2 + Ky dx dy + Kz dy^2 (log2(e) times the published power) and the
 * weight 2^y.  Deterministic 2^y for y <= 0: k = rint(y), r = y - k exact, 2^r = 1 + r c(r)
 * with c of degree 5 (Lawson's reweighted least squares, oracle/fit_exp.py fit_exp2)
 * evaluated with fused multiply-adds, and an exact power-of-two scale.  Max error below one
 * ulp (checked against numpy in tests/test_oracle.py).  y below -126 and NaN are raised to
 * -126 (2^-126 fails the alpha test as 0 would).  The kernels' gs_exp2f forms rint(y) and
 * the scale without conversion instructions; tests/test_oracle.py checks that it returns
 * this function's value for every float in [-126, 0]. */
#define OR_KHALF (-0x1.715476p-1f)
#define OR_KFULL (-0x1.715476p+0f)
static float or_exp2f(float y)
{
    y = fmaxf(y, -126.0f);
    float k = rintf(y);
    float r = y - k;
    float p = 0x1.41fbb8p-13f;
    p = fmaf(p, r, 0x1.5f3e56p-10f);
    p = fmaf(p, r, 0x1.3b2d4ep-7f);
    p = fmaf(p, r, 0x1.c6aee8p-5f);
    p = fmaf(p, r, 0x1.ebfbdcp-3f);
    p = fmaf(p, r, 0x1.62e43p-1f);
    p = fmaf(p, r, 1.0f);
    int ki = (int)k;
    uint32_t bits = (uint32_t)(ki + 127) << 23;
    float sc;
    memcpy(&sc, &bits, 4);
    return p * sc;
}

float or_exp2f_export(float y) { return or_exp2f(y); }

/* ------------------------------------------------------- FP32 / FP64 instances */
#define REAL float
#define FN(n) n##_f
#define RC(x) x##f
#define FMIN fminf
#define FMAX fmaxf
#define SQRT sqrtf
#define CEIL ceilf
#include "or_math.inc"
#undef REAL
#undef FN
#undef RC
#undef FMIN
#undef FMAX
#undef SQRT
#undef CEIL

#define REAL double
#define FN(n) n##_d
#define RC(x) x
#define FMIN fmin
#define FMAX fmax
#define SQRT sqrt
#define CEIL ceil
#include "or_math.inc"
#undef REAL
#undef FN
#undef RC
#undef FMIN
#undef FMAX
#undef SQRT
#undef CEIL

/* SH colour (value + 0.5, before the clamp) for n directions, FP64 instance.
 * sh: [n][16][3], dirs: [n][3] unit vectors, out: [n][3]. */
void or_sh_eval_f64(int n, int deg, const float *sh, const double *dirs, double *out)
{
    for (int i = 0; i < n; ++i)
        sh_rgb_d(deg, sh + 48 * i, dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2], out + 3 * i);
}

/* ------------------------------------------------------------ cov3D -------- */
void or_cov3d(int n, const float *scale, const float *rot, float mod, float *cov6)
{
    for (int i = 0; i < n; ++i) cov3d_f(scale + 3 * i, rot + 4 * i, mod, cov6 + 6 * i);
}

/* -------------------------------------------------------- preprocess (FP32) -- */
/* view: 33 floats = R[9] t[3] Praw[16] campos[3] tanfx tanfy.
 * colors_pre (nullable) replaces SH evaluation, as colors_precomp in the drop-in API.
 * Outputs are written for every Gaussian (zeros when culled). */
void or_preprocess(int n, const float *xyz, const float *cov6, const float *sh, int sh_deg,
                   const float *colors_pre, const float *view, int W, int H,
                   int *radii, int *touched, float *mean2d, float *depth, float *conic,
                   float *rgb, float *grey, int *rect)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        pre_t_f o;
        float cov[6];
        for (int k = 0; k < 6; ++k) cov[k] = cov6[6 * i + k];
        int vis = preprocess_one_f(xyz + 3 * i, cov, sh ? sh + 48 * i : NULL, sh_deg,
                                   colors_pre ? colors_pre + 3 * i : NULL, view, W, H, &o);
        radii[i] = vis ? (int)o.radius : 0;
        touched[i] = vis ? (o.rect[2] - o.rect[0]) * (o.rect[3] - o.rect[1]) : 0;
        mean2d[2 * i] = vis ? o.mean[0] : 0.0f;
        mean2d[2 * i + 1] = vis ? o.mean[1] : 0.0f;
        depth[i] = vis ? o.pc[2] : 0.0f;
        for (int k = 0; k < 3; ++k) conic[3 * i + k] = vis ? o.conic[k] : 0.0f;
        for (int k = 0; k < 3; ++k) rgb[3 * i + k] = vis ? o.rgb[k] : 0.0f;
        grey[i] = vis ? grey_f(o.rgb) : 0.0f;
        if (rect)
            for (int k = 0; k < 4; ++k) rect[4 * i + k] = vis ? o.rect[k] : 0;
    }
}

/* ----------------------------------------------------- duplicate / sort / ranges */
/* Emits, in Gaussian order, one (key, value) per touched tile in row-major rect order:
 * key = ((tile_offset + ty*tiles_x + tx) << 32) | float_bits(depth), value = val_offset + i. */
int64_t or_duplicate(int n, const int *touched, const float *mean2d, const int *radii,
                     const float *depth, int W, int H, uint32_t tile_offset, uint32_t val_offset,
                     uint64_t *keys, uint32_t *vals)
{
    int tiles_x = (W + 15) / 16, tiles_y = (H + 15) / 16;
    float gx = (float)tiles_x, gy = (float)tiles_y;
    int64_t k = 0;
    for (int i = 0; i < n; ++i) {
        if (touched[i] == 0) continue;
        float r = (float)radii[i];
        float mx = mean2d[2 * i], my = mean2d[2 * i + 1];
        int x0 = (int)fminf(gx, fmaxf(0.0f, (mx - r) / 16.0f));
        int y0 = (int)fminf(gy, fmaxf(0.0f, (my - r) / 16.0f));
        int x1 = (int)fminf(gx, fmaxf(0.0f, ((mx + r) + 15.0f) / 16.0f));
        int y1 = (int)fminf(gy, fmaxf(0.0f, ((my + r) + 15.0f) / 16.0f));
        uint32_t db;
        memcpy(&db, &depth[i], 4);
        for (int y = y0; y < y1; ++y)
            for (int x = x0; x < x1; ++x) {
                uint64_t tile = (uint64_t)(tile_offset + (uint32_t)(y * tiles_x + x));
                keys[k] = (tile << 32) | (uint64_t)db;
                vals[k] = val_offset + (uint32_t)i;
                ++k;
            }
    }
    return k;
}

/* stable ascending sort of (key, value) by key: LSD radix sort, 8-bit digits */
void or_sort_pairs(int64_t k, uint64_t *keys, uint32_t *vals, int bits)
{
    if (k <= 1) return;
    uint64_t *k2 = (uint64_t *)malloc(sizeof(uint64_t) * k);
    uint32_t *v2 = (uint32_t *)malloc(sizeof(uint32_t) * k);
    uint64_t *ka = keys, *kb = k2;
    uint32_t *va = vals, *vb = v2;
    int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        int64_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        int sh = 8 * p;
        for (int64_t i = 0; i < k; ++i) cnt[((ka[i] >> sh) & 255) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (int64_t i = 0; i < k; ++i) {
            int d = (int)((ka[i] >> sh) & 255);
            int64_t pos = cnt[d]++;
            kb[pos] = ka[i];
            vb[pos] = va[i];
        }
        uint64_t *tk = ka; ka = kb; kb = tk;
        uint32_t *tv = va; va = vb; vb = tv;
    }
    if (ka != keys) {
        memcpy(keys, ka, sizeof(uint64_t) * k);
        memcpy(vals, va, sizeof(uint32_t) * k);
    }
    free(k2);
    free(v2);
}

/* ranges[t] = [start, end) of tile t in the sorted key list (zeros if empty) */
void or_ranges(int64_t k, const uint64_t *keys, int ntiles, uint32_t *ranges)
{
    memset(ranges, 0, sizeof(uint32_t) * 2 * (size_t)ntiles);
    for (int64_t i = 0; i < k; ++i) {
        uint32_t t = (uint32_t)(keys[i] >> 32);
        if (i == 0 || (uint32_t)(keys[i - 1] >> 32) != t) ranges[2 * t] = (uint32_t)i;
        if (i == k - 1 || (uint32_t)(keys[i + 1] >> 32) != t) ranges[2 * t + 1] = (uint32_t)(i + 1);
    }
}

/* ------------------------------------------------------------ blend (FP32) -- */
/* Front-to-back alpha blending of one view.  ranges/vals index the per-view arrays
 * (value v refers to Gaussian v).  colors: [n][nch].  Outputs are [nch][H][W] etc.
 * Optional outputs may be NULL.  If rec_count is non-NULL, per-pixel contributor
 * counts are written; if additionally rec_ids is non-NULL (with rec_start[P+1]
 * prefix offsets), contributor ids and clamp flags are recorded for the FP64 path. */
void or_blend_fwd(int W, int H, int nch, const uint32_t *ranges, const uint32_t *vals,
                  const float *mean2d, const float *conic, const float *opac,
                  const float *colors, const float *depth, const float *bg,
                  float *out_color, float *out_T, float *out_depth, float *out_alpha,
                  int *n_contrib, int *n_touched,
                  int *rec_count, const int64_t *rec_start, uint32_t *rec_ids, uint8_t *rec_clamp)
{
    int tiles_x = (W + 15) / 16, tiles_y = (H + 15) / 16;
    int ntiles = tiles_x * tiles_y;
#pragma omp parallel for schedule(dynamic, 4)
    for (int t = 0; t < ntiles; ++t) {
        int tx = t % tiles_x, ty = t / tiles_x;
        uint32_t s = ranges[2 * t], e = ranges[2 * t + 1];
        for (int ly = 0; ly < TILE; ++ly)
            for (int lx = 0; lx < TILE; ++lx) {
                int px = tx * TILE + lx, py = ty * TILE + ly;
                if (px >= W || py >= H) continue;
                int pix = py * W + px;
                float pxf = (float)px, pyf = (float)py;
                float T = 1.0f, C[3] = {0.0f, 0.0f, 0.0f}, D = 0.0f, A = 0.0f;
                int last = 0, cnt = 0;
                int64_t rp = rec_ids ? rec_start[pix] : 0;
                for (uint32_t j = s; j < e; ++j) {
                    uint32_t g = vals[j];
                    float dx = mean2d[2 * g] - pxf, dy = mean2d[2 * g + 1] - pyf;
                    /* base-2 exponent: K from the conic, then dx (Kx dx + Ky dy) + Kz dy^2
                     * with two fused multiply-adds (the CUDA blends' gs_log2_conic and
                     * gs_power2 use the same order) */
                    float kx = OR_KHALF * conic[3 * g], ky = OR_KFULL * conic[3 * g + 1];
                    float kz = OR_KHALF * conic[3 * g + 2];
                    float y2 = fmaf(fmaf(ky, dy, kx * dx), dx, (kz * dy) * dy);
                    if (y2 > 0.0f) continue;
                    float G = or_exp2f(y2);
                    float araw = opac[g] * G;
                    float alpha = fminf(0.99f, araw);
                    if (alpha < 1.0f / 255.0f) continue;
                    float test_T = fmaf(-T, alpha, T); /* T (1 - alpha), one rounding */
                    if (test_T < 0.0001f) break;
                    for (int ch = 0; ch < nch; ++ch)
                        C[ch] = fmaf(colors[nch * g + ch] * alpha, T, C[ch]);
                    if (depth) D = fmaf(depth[g] * alpha, T, D);
                    A = fmaf(alpha, T, A);
                    if (n_touched && test_T > 0.5f) {
#pragma omp atomic
                        n_touched[g] += 1;
                    }
                    if (rec_ids) {
                        rec_ids[rp] = g;
                        rec_clamp[rp] = (uint8_t)(araw > 0.99f);
                        ++rp;
                    }
                    T = test_T;
                    last = (int)(j - s) + 1;
                    ++cnt;
                }
                for (int ch = 0; ch < nch; ++ch)
                    out_color[(size_t)ch * W * H + pix] = C[ch] + T * bg[ch];
                if (out_T) out_T[pix] = T;
                if (out_depth) out_depth[pix] = D;
                if (out_alpha) out_alpha[pix] = A;
                if (n_contrib) n_contrib[pix] = last;
                if (rec_count) rec_count[pix] = cnt;
            }
    }
}

/* --------------------------------------------------------- FP64 frozen path -- */
/* view_d: 33 doubles, same layout as the FP32 view.  Preprocess every Gaussian in FP64. */
typedef struct {
    pre_t_d *pre;
    int *vis;
} or_pre64;

static void pre64_all(int n, const float *xyz, const double *cov6d, const float *sh, int deg,
                      const float *colors_pre, const double *view, int W, int H, pre_t_d *pre,
                      int *vis)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i)
        vis[i] = preprocess_one_d(xyz + 3 * i, cov6d + 6 * i, sh ? sh + 48 * i : NULL, deg,
                                  colors_pre ? colors_pre + 3 * i : NULL, view, W, H, &pre[i]);
}

static void cov6d_all(int n, const float *scale, const float *rot, const float *cov_pre,
                      double mod, double *cov6d)
{
    for (int i = 0; i < n; ++i) {
        if (cov_pre) {
            for (int k = 0; k < 6; ++k) cov6d[6 * i + k] = (double)cov_pre[6 * i + k];
        } else {
            cov3d_d(scale + 3 * i, rot + 4 * i, mod, cov6d + 6 * i);
        }
    }
}

/* Frozen FP64 render: nch colour channels (3 = RGB, 1 = grey of RGB).  out: [nch][H][W]
 * plus optional depth/alpha. */
static void frozen_fwd(int n, const pre_t_d *pre, const float *opac, int W, int H, int nch,
                       const double *bg, const int64_t *rec_start, const uint32_t *rec_ids,
                       const uint8_t *rec_clamp, double *out, double *out_depth, double *out_alpha)
{
    int P = W * H;
#pragma omp parallel for schedule(static)
    for (int pix = 0; pix < P; ++pix) {
        double pxf = (double)(pix % W), pyf = (double)(pix / W);
        double T = 1.0, C[3] = {0, 0, 0}, D = 0.0, A = 0.0;
        for (int64_t r = rec_start[pix]; r < rec_start[pix + 1]; ++r) {
            const pre_t_d *o = &pre[rec_ids[r]];
            double dx = o->mean[0] - pxf, dy = o->mean[1] - pyf;
            double power = -0.5 * (o->conic[0] * dx * dx + o->conic[2] * dy * dy) - o->conic[1] * dx * dy;
            double alpha = rec_clamp[r] ? 0.99 : (double)opac[rec_ids[r]] * exp(power);
            double col[3];
            if (nch == 1) col[0] = grey_d(o->rgb);
            else for (int c = 0; c < 3; ++c) col[c] = o->rgb[c];
            for (int c = 0; c < nch; ++c) C[c] += col[c] * alpha * T;
            D += o->pc[2] * alpha * T;
            A += alpha * T;
            T *= (1.0 - alpha);
        }
        for (int c = 0; c < nch; ++c) out[(size_t)c * P + pix] = C[c] + T * bg[c];
        if (out_depth) out_depth[pix] = D;
        if (out_alpha) out_alpha[pix] = A;
    }
}

int or_frozen_render_f64(int n, const float *xyz, const float *scale, const float *rot,
                         const float *cov_pre, double mod, const float *opac, const float *sh,
                         int deg, const float *colors_pre, const double *view, int W, int H,
                         int nch, const double *bg, const int64_t *rec_start,
                         const uint32_t *rec_ids, const uint8_t *rec_clamp, double *out,
                         double *out_depth, double *out_alpha)
{
    if (!cov_pre && (!scale || !rot)) return -1;
    if (!sh && !colors_pre) return -1;
    double *cov6d = (double *)malloc(sizeof(double) * 6 * (size_t)(n > 0 ? n : 1));
    pre_t_d *pre = (pre_t_d *)malloc(sizeof(pre_t_d) * (size_t)(n > 0 ? n : 1));
    int *vis = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    cov6d_all(n, scale, rot, cov_pre, mod, cov6d);
    pre64_all(n, xyz, cov6d, sh, deg, colors_pre, view, W, H, pre, vis);
    frozen_fwd(n, pre, opac, W, H, nch, bg, rec_start, rec_ids, rec_clamp, out, out_depth, out_alpha);
    free(cov6d);
    free(pre);
    free(vis);
    return 0;
}

/* SH basis values Y_k(dir) and their gradients d/d(x,y,z) (treating x,y,z as free) */
static void sh_basis_d(int deg, double x, double y, double z, double *Y, double (*dY)[3])
{
    const double C0 = 0.28209479177387814, C1 = 0.4886025119029199;
    const double C2[5] = {1.0925484305920792, -1.0925484305920792, 0.31539156525252005,
                          -1.0925484305920792, 0.5462742152960396};
    const double C3[7] = {-0.5900435899266435, 2.890611442640554, -0.4570457994644658,
                          0.3731763325901154, -0.4570457994644658, 1.445305721320277,
                          -0.5900435899266435};
    for (int k = 0; k < 16; ++k) { Y[k] = 0; dY[k][0] = dY[k][1] = dY[k][2] = 0; }
    Y[0] = C0;
    if (deg < 1) return;
    Y[1] = -C1 * y; dY[1][1] = -C1;
    Y[2] = C1 * z;  dY[2][2] = C1;
    Y[3] = -C1 * x; dY[3][0] = -C1;
    if (deg < 2) return;
    double xx = x * x, yy = y * y, zz = z * z;
    Y[4] = C2[0] * x * y; dY[4][0] = C2[0] * y; dY[4][1] = C2[0] * x;
    Y[5] = C2[1] * y * z; dY[5][1] = C2[1] * z; dY[5][2] = C2[1] * y;
    Y[6] = C2[2] * (2 * zz - xx - yy); dY[6][0] = -2 * C2[2] * x; dY[6][1] = -2 * C2[2] * y; dY[6][2] = 4 * C2[2] * z;
    Y[7] = C2[3] * x * z; dY[7][0] = C2[3] * z; dY[7][2] = C2[3] * x;
    Y[8] = C2[4] * (xx - yy); dY[8][0] = 2 * C2[4] * x; dY[8][1] = -2 * C2[4] * y;
    if (deg < 3) return;
    Y[9] = C3[0] * y * (3 * xx - yy);
    dY[9][0] = C3[0] * 6 * x * y; dY[9][1] = C3[0] * (3 * xx - 3 * yy);
    Y[10] = C3[1] * x * y * z;
    dY[10][0] = C3[1] * y * z; dY[10][1] = C3[1] * x * z; dY[10][2] = C3[1] * x * y;
    Y[11] = C3[2] * y * (4 * zz - xx - yy);
    dY[11][0] = C3[2] * (-2 * x * y); dY[11][1] = C3[2] * (4 * zz - xx - 3 * yy); dY[11][2] = C3[2] * 8 * y * z;
    Y[12] = C3[3] * z * (2 * zz - 3 * xx - 3 * yy);
    dY[12][0] = C3[3] * (-6 * x * z); dY[12][1] = C3[3] * (-6 * y * z); dY[12][2] = C3[3] * (6 * zz - 3 * xx - 3 * yy);
    Y[13] = C3[4] * x * (4 * zz - xx - yy);
    dY[13][0] = C3[4] * (4 * zz - 3 * xx - yy); dY[13][1] = C3[4] * (-2 * x * y); dY[13][2] = C3[4] * 8 * x * z;
    Y[14] = C3[5] * z * (xx - yy);
    dY[14][0] = C3[5] * 2 * x * z; dY[14][1] = C3[5] * (-2 * y * z); dY[14][2] = C3[5] * (xx - yy);
    Y[15] = C3[6] * x * (xx - 3 * yy);
    dY[15][0] = C3[6] * (3 * xx - 3 * yy); dY[15][1] = C3[6] * (-6 * x * y);
}

/* Analytic FP64 gradient along the frozen contributor lists.
 * dL_dout: [nch][H][W]; dL_ddepth / dL_dalpha nullable ([H][W]).
 * Outputs (all nullable except g_xi):
 *   g_xi[6]         : dL/d(left twist of this view) = (rho, theta)
 *   g_mean2d[n][2]  : dL/d(NDC mean) (the drop-in means2D gradient convention)
 *   g_means3d[n][3], g_sh[n][48], g_opac[n], g_scale[n][3], g_rot[n][4], g_cov[n][6],
 *   g_colors[n][3] (when colors_pre is given).
 * Map gradients through scale/rot use the rotation as given (no re-normalisation). */
void or_frozen_backward_f64(int n, const float *xyz, const float *scale, const float *rot,
                            const float *cov_pre, double mod, const float *opac, const float *sh,
                            int deg, const float *colors_pre, const double *view, int W, int H,
                            int nch, const double *bg, const int64_t *rec_start,
                            const uint32_t *rec_ids, const uint8_t *rec_clamp,
                            const double *dL_dout, const double *dL_ddepth, const double *dL_dalpha,
                            double *g_xi, double *g_mean2d, double *g_means3d, double *g_sh,
                            double *g_opac, double *g_scale, double *g_rot, double *g_cov,
                            double *g_colors)
{
    if ((!cov_pre && (!scale || !rot)) || (!sh && !colors_pre)) {
        for (int k = 0; k < 6; ++k) g_xi[k] = NAN;
        return;
    }
    int P = W * H;
    size_t nn = (size_t)(n > 0 ? n : 1);
    double *cov6d = (double *)malloc(sizeof(double) * 6 * nn);
    pre_t_d *pre = (pre_t_d *)malloc(sizeof(pre_t_d) * nn);
    int *vis = (int *)malloc(sizeof(int) * nn);
    cov6d_all(n, scale, rot, cov_pre, mod, cov6d);
    pre64_all(n, xyz, cov6d, sh, deg, colors_pre, view, W, H, pre, vis);

    /* per-Gaussian 2D gradients: mean (pixel units) 2, conic 3, opacity 1, colour 3, depth 1 */
    double *g2 = (double *)calloc(nn * 10, sizeof(double));
    for (int pix = 0; pix < P; ++pix) {
        double pxf = (double)(pix % W), pyf = (double)(pix / W);
        int64_t r0 = rec_start[pix], r1 = rec_start[pix + 1];
        /* forward totals */
        double T = 1.0, C[3] = {0, 0, 0}, D = 0, A = 0;
        for (int64_t r = r0; r < r1; ++r) {
            const pre_t_d *o = &pre[rec_ids[r]];
            double dx = o->mean[0] - pxf, dy = o->mean[1] - pyf;
            double power = -0.5 * (o->conic[0] * dx * dx + o->conic[2] * dy * dy) - o->conic[1] * dx * dy;
            double alpha = rec_clamp[r] ? 0.99 : (double)opac[rec_ids[r]] * exp(power);
            double col[3];
            if (nch == 1) col[0] = grey_d(o->rgb);
            else for (int c = 0; c < 3; ++c) col[c] = o->rgb[c];
            for (int c = 0; c < nch; ++c) C[c] += col[c] * alpha * T;
            D += o->pc[2] * alpha * T;
            A += alpha * T;
            T *= (1.0 - alpha);
        }
        double Tf = T;
        double gC[3] = {0, 0, 0};
        for (int c = 0; c < nch; ++c) gC[c] = dL_dout[(size_t)c * P + pix];
        double gD = dL_ddepth ? dL_ddepth[pix] : 0.0, gA = dL_dalpha ? dL_dalpha[pix] : 0.0;
        /* second sweep: prefix sums and gradients */
        T = 1.0;
        double Pc[3] = {0, 0, 0}, PD = 0, PA = 0;
        for (int64_t r = r0; r < r1; ++r) {
            uint32_t g = rec_ids[r];
            const pre_t_d *o = &pre[g];
            double dx = o->mean[0] - pxf, dy = o->mean[1] - pyf;
            double power = -0.5 * (o->conic[0] * dx * dx + o->conic[2] * dy * dy) - o->conic[1] * dx * dy;
            double G = exp(power);
            double alpha = rec_clamp[r] ? 0.99 : (double)opac[g] * G;
            double col[3];
            if (nch == 1) col[0] = grey_d(o->rgb);
            else for (int c = 0; c < 3; ++c) col[c] = o->rgb[c];
            double w = alpha * T;
            double dalpha = 0.0;
            for (int c = 0; c < nch; ++c) {
                Pc[c] += col[c] * w;
                double suffix = (C[c] - Pc[c]) + Tf * bg[c];
                dalpha += gC[c] * (T * col[c] - suffix / (1.0 - alpha));
                g2[10 * g + 6 + c] += gC[c] * w;
            }
            PD += o->pc[2] * w;
            PA += w;
            dalpha += gD * (T * o->pc[2] - (D - PD) / (1.0 - alpha));
            dalpha += gA * (T - (A - PA) / (1.0 - alpha));
            g2[10 * g + 9] += gD * w;
            if (!rec_clamp[r]) {
                g2[10 * g + 5] += dalpha * G;
                double dpower = dalpha * (double)opac[g] * G;
                /* power = -0.5(cx dx^2 + cz dy^2) - cy dx dy, d = mean - pix */
                g2[10 * g + 2] += dpower * (-0.5 * dx * dx);
                g2[10 * g + 3] += dpower * (-dx * dy);
                g2[10 * g + 4] += dpower * (-0.5 * dy * dy);
                g2[10 * g + 0] += dpower * (-o->conic[0] * dx - o->conic[1] * dy);
                g2[10 * g + 1] += dpower * (-o->conic[2] * dy - o->conic[1] * dx);
            }
            T *= (1.0 - alpha);
        }
    }

    const double *R = view, *P4 = view + 12;
    double fx = (double)W / (2.0 * view[31]), fy = (double)H / (2.0 * view[32]);
    double xi[6] = {0, 0, 0, 0, 0, 0};
    for (int g = 0; g < n; ++g) {
        if (!vis[g]) continue;
        const double *q = g2 + 10 * g;
        int any = 0;
        for (int k = 0; k < 10; ++k) any |= (q[k] != 0.0);
        if (!any) continue;
        const pre_t_d *o = &pre[g];
        double a = o->cov2[0], b = o->cov2[1], c = o->cov2[2], det = o->det;
        double d2 = det * det;
        double gCa = q[2], gCb = q[3], gCc = q[4];
        double ga = gCa * (-c * c / d2) + gCb * (b * c / d2) + gCc * (-b * b / d2);
        double gb = gCa * (2 * b * c / d2) + gCb * (-(a * c + b * b) / d2) + gCc * (2 * a * b / d2);
        double gc = gCa * (-b * b / d2) + gCb * (a * b / d2) + gCc * (-a * a / d2);
        double Gs[2][2] = {{ga, 0.5 * gb}, {0.5 * gb, gc}};
        const double *cv = cov6d + 6 * g;
        double S[3][3] = {{cv[0], cv[1], cv[2]}, {cv[1], cv[3], cv[4]}, {cv[2], cv[4], cv[5]}};
        double Tm[2][3] = {{o->T[0], o->T[1], o->T[2]}, {o->T[3], o->T[4], o->T[5]}};
        /* dL/dSigma = T^T Gs T ; dL/dT = 2 Gs T Sigma */
        double gS[3][3], GT[2][3], gT[2][3];
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 3; ++j) GT[i][j] = Gs[i][0] * Tm[0][j] + Gs[i][1] * Tm[1][j];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) gS[i][j] = Tm[0][i] * GT[0][j] + Tm[1][i] * GT[1][j];
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int k = 0; k < 3; ++k) s += GT[i][k] * S[k][j];
                gT[i][j] = 2.0 * s;
            }
        double J00 = o->J[0], J02 = o->J[1], J11 = o->J[2], J12 = o->J[3];
        double gJ00 = 0, gJ02 = 0, gJ11 = 0, gJ12 = 0;
        double gW[3][3];
        for (int j = 0; j < 3; ++j) {
            gJ00 += gT[0][j] * R[j];
            gJ02 += gT[0][j] * R[6 + j];
            gJ11 += gT[1][j] * R[3 + j];
            gJ12 += gT[1][j] * R[6 + j];
            gW[0][j] = gT[0][j] * J00;
            gW[1][j] = gT[1][j] * J11;
            gW[2][j] = gT[0][j] * J02 + gT[1][j] * J12;
        }
        double vx = o->pc[0], vy = o->pc[1], vz = o->pc[2];
        double vz2 = vz * vz, vz3 = vz2 * vz;
        double gpc[3] = {0, 0, 0};
        gpc[2] += gJ00 * (-fx / vz2) + gJ11 * (-fy / vz2);
        if (!o->clampx) { gpc[0] += gJ02 * (-fx / vz2); gpc[2] += gJ02 * (2.0 * fx * vx / vz3); }
        else { gpc[2] += gJ02 * (-J02 / vz); }
        if (!o->clampy) { gpc[1] += gJ12 * (-fy / vz2); gpc[2] += gJ12 * (2.0 * fy * vy / vz3); }
        else { gpc[2] += gJ12 * (-J12 / vz); }
        /* mean (pixel) -> clip */
        double gnx = q[0] * 0.5 * W, gny = q[1] * 0.5 * H;
        double pw = o->pw;
        double gh[4] = {gnx * pw, gny * pw, 0.0, -(gnx * o->hom[0] + gny * o->hom[1]) * pw * pw};
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 4; ++i) gpc[j] += P4[4 * i + j] * gh[i];
        gpc[2] += q[9];
        /* colour -> SH and direction */
        double gu[3] = {0, 0, 0};
        double grgb[3] = {0, 0, 0};
        if (nch == 1) { grgb[0] = 0.2989 * q[6]; grgb[1] = 0.587 * q[6]; grgb[2] = 0.114 * q[6]; }
        else { grgb[0] = q[6]; grgb[1] = q[7]; grgb[2] = q[8]; }
        if (colors_pre) {
            if (g_colors) for (int ch = 0; ch < 3; ++ch) g_colors[3 * g + ch] += grgb[ch];
        } else {
            double Y[16], dY[16][3];
            sh_basis_d(deg, o->dir[0], o->dir[1], o->dir[2], Y, dY);
            double gdir[3] = {0, 0, 0};
            for (int ch = 0; ch < 3; ++ch) {
                double gr = (o->rgb_raw[ch] < 0.0) ? 0.0 : grgb[ch];
                if (gr == 0.0) continue;
                for (int k = 0; k < 16; ++k) {
                    if (g_sh) g_sh[48 * g + 3 * k + ch] += gr * Y[k];
                    const float *s = sh + 48 * g + 3 * k + ch;
                    gdir[0] += gr * (double)(*s) * dY[k][0];
                    gdir[1] += gr * (double)(*s) * dY[k][1];
                    gdir[2] += gr * (double)(*s) * dY[k][2];
                }
            }
            double dd = o->dir[0] * gdir[0] + o->dir[1] * gdir[1] + o->dir[2] * gdir[2];
            for (int j = 0; j < 3; ++j) gu[j] = (gdir[j] - o->dir[j] * dd) / o->dirlen;
        }
        /* pose twist (rho, theta): p_c' = p_c + rho + theta x p_c ; W' = (I + [theta]x) W ;
         * campos' = campos - R^T rho */
        double Rgu[3];
        for (int i = 0; i < 3; ++i) Rgu[i] = R[3 * i] * gu[0] + R[3 * i + 1] * gu[1] + R[3 * i + 2] * gu[2];
        xi[0] += gpc[0] + Rgu[0];
        xi[1] += gpc[1] + Rgu[1];
        xi[2] += gpc[2] + Rgu[2];
        double cx = vy * gpc[2] - vz * gpc[1];
        double cy = vz * gpc[0] - vx * gpc[2];
        double cz = vx * gpc[1] - vy * gpc[0];
        double M[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) M[i][j] = R[3 * i] * gW[j][0] + R[3 * i + 1] * gW[j][1] + R[3 * i + 2] * gW[j][2];
        xi[3] += cx + (M[1][2] - M[2][1]);
        xi[4] += cy + (M[2][0] - M[0][2]);
        xi[5] += cz + (M[0][1] - M[1][0]);
        /* map gradients */
        if (g_mean2d) { g_mean2d[2 * g] += gnx; g_mean2d[2 * g + 1] += gny; }
        if (g_opac) g_opac[g] += q[5];
        if (g_means3d)
            for (int j = 0; j < 3; ++j)
                g_means3d[3 * g + j] += (R[j] * gpc[0] + R[3 + j] * gpc[1] + R[6 + j] * gpc[2]) + gu[j];
        if (g_cov) {
            g_cov[6 * g + 0] += gS[0][0];
            g_cov[6 * g + 1] += gS[0][1] + gS[1][0];
            g_cov[6 * g + 2] += gS[0][2] + gS[2][0];
            g_cov[6 * g + 3] += gS[1][1];
            g_cov[6 * g + 4] += gS[1][2] + gS[2][1];
            g_cov[6 * g + 5] += gS[2][2];
        }
        if (!cov_pre && (g_scale || g_rot)) {
            double r = rot[4 * g], x = rot[4 * g + 1], y = rot[4 * g + 2], z = rot[4 * g + 3];
            double Rq[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)},
                               {2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)},
                               {2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)}};
            double s[3] = {mod * scale[3 * g], mod * scale[3 * g + 1], mod * scale[3 * g + 2]};
            double L[3][3], gL[3][3];
            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < 3; ++k) L[i][k] = Rq[i][k] * s[k];
            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < 3; ++k) {
                    double acc = 0;
                    for (int j = 0; j < 3; ++j) acc += (gS[i][j] + gS[j][i]) * L[j][k];
                    gL[i][k] = acc;
                }
            if (g_scale)
                for (int k = 0; k < 3; ++k) {
                    double acc = 0;
                    for (int i = 0; i < 3; ++i) acc += gL[i][k] * Rq[i][k];
                    g_scale[3 * g + k] += acc * mod;
                }
            if (g_rot) {
                double gR[3][3];
                for (int i = 0; i < 3; ++i)
                    for (int k = 0; k < 3; ++k) gR[i][k] = gL[i][k] * s[k];
                double gr_ = 2 * z * (gR[1][0] - gR[0][1]) + 2 * y * (gR[0][2] - gR[2][0]) + 2 * x * (gR[2][1] - gR[1][2]);
                double gx_ = 2 * y * (gR[0][1] + gR[1][0]) + 2 * z * (gR[0][2] + gR[2][0]) + 2 * r * (gR[2][1] - gR[1][2]) - 4 * x * (gR[1][1] + gR[2][2]);
                double gy_ = 2 * x * (gR[0][1] + gR[1][0]) + 2 * r * (gR[0][2] - gR[2][0]) + 2 * z * (gR[1][2] + gR[2][1]) - 4 * y * (gR[0][0] + gR[2][2]);
                double gz_ = 2 * r * (gR[1][0] - gR[0][1]) + 2 * x * (gR[0][2] + gR[2][0]) + 2 * y * (gR[1][2] + gR[2][1]) - 4 * z * (gR[0][0] + gR[1][1]);
                g_rot[4 * g] += gr_; g_rot[4 * g + 1] += gx_; g_rot[4 * g + 2] += gy_; g_rot[4 * g + 3] += gz_;
            }
        }
    }
    for (int k = 0; k < 6; ++k) g_xi[k] = xi[k];
    free(g2);
    free(cov6d);
    free(pre);
    free(vis);
}

/* ------------------------------------------------------------------ loss -- */
/* Normalised intensity-change loss (utils/render_camera/frame.py:86-94 and
 * utils/tracker.py:93-103): dI = I_next - I_last; n = dI/||dI||;
 * signed: L = ||n - E||; unsigned: L = || |n| - |E| ||.  FP64 throughout.
 * Gradients dL/dI_next = -dL/dI_last written when non-NULL. */
/* Pair loss of utils/tracker.py:93-103 over dI of utils/render_camera/frame.py:86-92,
 * in FP64.  log_eps > 0 selects the log-intensity change dI = ln(I_next + eps) -
 * ln(I_last + eps) (the image gradients then carry the factor 1 / (I + eps)); log_eps <= 0
 * the reference's linear dI = I_next - I_last. */
static double dI_at(const float *I_last, const float *I_next, int64_t i, double log_eps)
{
    if (log_eps > 0) return log((double)I_next[i] + log_eps) - log((double)I_last[i] + log_eps);
    return (double)I_next[i] - (double)I_last[i];
}

double or_loss(int64_t npix, const float *I_last, const float *I_next, const float *E,
               int unsigned_mode, double log_eps, double *dL_dnext, double *dL_dlast)
{
    double s2 = 0, cross = 0, e2 = 0;
    for (int64_t i = 0; i < npix; ++i) {
        double d = dI_at(I_last, I_next, i, log_eps);
        double e = E[i];
        s2 += d * d;
        e2 += e * e;
        cross += unsigned_mode ? fabs(d) * fabs(e) : d * e;
    }
    double s = sqrt(s2);
    double L2 = 1.0 - 2.0 * cross / s + e2;
    double L = sqrt(L2 > 0 ? L2 : 0);
    if (dL_dnext || dL_dlast) {
        double ng = (1.0 - cross / s) / L;
        for (int64_t i = 0; i < npix; ++i) {
            double d = dI_at(I_last, I_next, i, log_eps);
            double n = d / s, e = E[i], g;
            if (unsigned_mode) {
                double sg = (d > 0) - (d < 0);
                g = sg * (fabs(n) - fabs(e)) / L;
            } else {
                g = (n - e) / L;
            }
            double dd = (g - n * ng) / s;
            if (dL_dnext) dL_dnext[i] = log_eps > 0 ? dd / ((double)I_next[i] + log_eps) : dd;
            if (dL_dlast) dL_dlast[i] = log_eps > 0 ? -dd / ((double)I_last[i] + log_eps) : -dd;
        }
    }
    return L;
}

/* --------------------------------------------------------------- events -- */
/* Undistortion of a float image (cv2.undistort with the camera matrix reused as the new
 * camera matrix, as utils/event_camera/event.py:121 calls it).  OpenCV's documented
 * model: for destination pixel (u, v), x = (u - cx)/fx, y = (v - cy)/fy, r2 = x^2 + y^2,
 * kr = 1 + ((k3 r2 + k2) r2 + k1) r2, xd = x kr + 2 p1 x y + p2 (r2 + 2 x^2),
 * yd = y kr + p1 (r2 + 2 y^2) + 2 p2 x y, source = (fx xd + cx, fy yd + cy); the source
 * position is rounded to 1/32 pixel (INTER_TAB_SIZE = 32) and sampled bilinearly with a
 * zero border.  cam = {fx, fy, cx, cy, k1, k2, p1, p2, k3}. */
void or_undistort(const float *src, int W, int H, const double *cam, float *dst)
{
    double fx = cam[0], fy = cam[1], cx = cam[2], cy = cam[3];
    double k1 = cam[4], k2 = cam[5], p1 = cam[6], p2 = cam[7], k3 = cam[8];
    for (int v = 0; v < H; ++v)
        for (int u = 0; u < W; ++u) {
            double x = (u - cx) / fx, y = (v - cy) / fy;
            double x2 = x * x, y2 = y * y, r2 = x2 + y2, xy2 = 2.0 * x * y;
            double kr = 1.0 + ((k3 * r2 + k2) * r2 + k1) * r2;
            double xd = x * kr + p1 * xy2 + p2 * (r2 + 2.0 * x2);
            double yd = y * kr + p1 * (r2 + 2.0 * y2) + p2 * xy2;
            double mx = fx * xd + cx, my = fy * yd + cy;
            long iu = lrint(mx * 32.0), iv = lrint(my * 32.0);
            long ix = iu >> 5, iy = iv >> 5;
            float ax = (float)(iu & 31) / 32.0f, ay = (float)(iv & 31) / 32.0f;
            float acc = 0.0f;
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    long sx = ix + dx, sy = iy + dy;
                    if (sx < 0 || sy < 0 || sx >= W || sy >= H) continue;
                    float w = (dx ? ax : 1.0f - ax) * (dy ? ay : 1.0f - ay);
                    acc += w * src[(size_t)sy * W + sx];
                }
            dst[(size_t)v * W + u] = acc;
        }
}

/* Event frame (utils/event_camera/event.py:116-128): count[y][x] += +1/-1 per event
 * (EVENT_BRIGHTNESS = 1, event.py:8), undistortion when cam is given (or_undistort),
 * separable Gaussian blur with the OpenCV kernel of size ksize and
 * sigma = 0.3*((ksize-1)*0.5 - 1) + 0.8 with BORDER_REPLICATE, then division by the
 * L2 norm (cv2.normalize defaults: NORM_L2, alpha 1; zero frame stays zero).
 * Blur arithmetic in double, results rounded to float. */
void or_event_frame(int W, int H, int64_t n, const uint16_t *ex, const uint16_t *ey,
                    const uint8_t *ep, int ksize, const double *cam, float *out_signed,
                    float *out_unsigned, int32_t *out_count)
{
    int32_t *cnt = (int32_t *)calloc((size_t)W * H, sizeof(int32_t));
    for (int64_t i = 0; i < n; ++i) {
        if (ex[i] >= W || ey[i] >= H) continue;
        cnt[(size_t)ey[i] * W + ex[i]] += ep[i] ? 1 : -1;
    }
    if (out_count) memcpy(out_count, cnt, sizeof(int32_t) * (size_t)W * H);
    float *img = (float *)malloc(sizeof(float) * (size_t)W * H);
    for (size_t i = 0; i < (size_t)W * H; ++i) img[i] = (float)cnt[i];
    if (cam) {
        float *und = (float *)malloc(sizeof(float) * (size_t)W * H);
        or_undistort(img, W, H, cam, und);
        free(img);
        img = und;
    }
    double sigma = 0.3 * ((ksize - 1) * 0.5 - 1.0) + 0.8;
    double kw[64], ksum = 0;
    int r = ksize / 2;
    for (int i = 0; i < ksize; ++i) {
        double x = i - r;
        kw[i] = exp(-(x * x) / (2.0 * sigma * sigma));
        ksum += kw[i];
    }
    for (int i = 0; i < ksize; ++i) kw[i] /= ksum;
    double *tmp = (double *)malloc(sizeof(double) * (size_t)W * H);
    double *blur = (double *)malloc(sizeof(double) * (size_t)W * H);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            double s = 0;
            for (int k = -r; k <= r; ++k) {
                int xx = x + k;
                xx = xx < 0 ? 0 : (xx >= W ? W - 1 : xx);
                s += kw[k + r] * (double)img[(size_t)y * W + xx];
            }
            tmp[(size_t)y * W + x] = s;
        }
    double n2 = 0;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            double s = 0;
            for (int k = -r; k <= r; ++k) {
                int yy = y + k;
                yy = yy < 0 ? 0 : (yy >= H ? H - 1 : yy);
                s += kw[k + r] * tmp[(size_t)yy * W + x];
            }
            blur[(size_t)y * W + x] = s;
            n2 += s * s;
        }
    double nrm = sqrt(n2);
    double sc = nrm > 2.220446049250313e-16 ? 1.0 / nrm : 0.0;
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        float v = (float)(blur[i] * sc);
        out_signed[i] = v;
        if (out_unsigned) out_unsigned[i] = fabsf(v);
    }
    free(cnt);
    free(img);
    free(tmp);
    free(blur);
}

/* Nearest-neighbour resize (cv2.resize INTER_NEAREST, utils/tracker.py:78-91):
 * src x = min(floor(dx * (sw / dw)), sw - 1). */
void or_resize_nearest(const float *src, int sw, int sh, float *dst, int dw, int dh)
{
    double ifx = (double)sw / dw, ify = (double)sh / dh;
    for (int y = 0; y < dh; ++y) {
        int sy = (int)floor(y * ify);
        if (sy > sh - 1) sy = sh - 1;
        for (int x = 0; x < dw; ++x) {
            int sx = (int)floor(x * ifx);
            if (sx > sw - 1) sx = sw - 1;
            dst[(size_t)y * dw + x] = src[(size_t)sy * sw + sx];
        }
    }
}
