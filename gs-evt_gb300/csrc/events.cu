// Event frame on the device (utils/event_camera/event.py:116-128 and the pyramid of
// utils/tracker.py:78-91), replacing a Python loop over events, cv2 and two
// host<->device copies per frame.
//   1. count[y][x] += +1 / -1 per event (EVENT_BRIGHTNESS = 1, event.py:8) with int32
//      atomics: integer sums, so the result does not depend on event order.
//   2. separable ksize Gaussian blur (OpenCV kernel, sigma = 0.3((ksize-1)/2 - 1) + 0.8
//      when sigma = 0), BORDER_REPLICATE, FP32 with FP64 weights rounded once.
//   3. L2 norm (FP64 block partials, fixed-order final sum), E = blur / ||blur||
//      (cv2.normalize defaults; a zero frame stays zero), |E|.
//   4. pyramid level l = nearest resize of level 0 to int(W 0.5^l) x int(H 0.5^l):
//      source index min(floor(x * W / w_l), W - 1) (cv2.resize INTER_NEAREST).
//   1b. when a camera is given, undistortion (cv2.undistort with the camera matrix as the
//      new camera matrix, event.py:121): OpenCV's documented distortion model maps each
//      destination pixel to its source position (computed in FP64, the same operation
//      order as the oracle), which is rounded to 1/32 pixel (INTER_TAB_SIZE = 32) and
//      sampled bilinearly with a zero border.
#include "common.cuh"

#include <cuda.h>

#include <mutex>

#define EV_MAX_K 31

namespace {

struct EvScratch {
    int32_t *count;
    float *tmp;
    float *blur;
    double *part;   // [EV_PART_BLOCKS]
    float *img;     // undistorted count image
};

#define EV_PART_BLOCKS 256

EvScratch ev_carve(void *base, int W, int H)
{
    EvScratch s;
    size_t P = (size_t)W * H;
    char *p = (char *)base;
    size_t off = 0;
    s.count = (int32_t *)(p + off); off += gs_align(P * 4);
    s.tmp = (float *)(p + off); off += gs_align(P * 4);
    s.blur = (float *)(p + off); off += gs_align(P * 4);
    s.part = (double *)(p + off); off += gs_align(EV_PART_BLOCKS * 8);
    s.img = (float *)(p + off); off += gs_align(P * 4);
    return s;
}

struct Cam { double fx, fy, cx, cy, k1, k2, p1, p2, k3; };

__global__ void k_ev_undistort(const int32_t *count, int W, int H, Cam c, float *dst)
{
    const int u = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y;
    if (u >= W) return;
    const double x = (u - c.cx) / c.fx, y = (v - c.cy) / c.fy;
    const double x2 = x * x, y2 = y * y, r2 = x2 + y2, xy2 = 2.0 * x * y;
    const double kr = 1.0 + ((c.k3 * r2 + c.k2) * r2 + c.k1) * r2;
    const double xd = x * kr + c.p1 * xy2 + c.p2 * (r2 + 2.0 * x2);
    const double yd = y * kr + c.p1 * (r2 + 2.0 * y2) + c.p2 * xy2;
    const double mx = c.fx * xd + c.cx, my = c.fy * yd + c.cy;
    const long long iu = llrint(mx * 32.0), iv = llrint(my * 32.0);
    const long long ix = iu >> 5, iy = iv >> 5;
    const float ax = (float)(iu & 31) / 32.0f, ay = (float)(iv & 31) / 32.0f;
    float acc = 0.0f;
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            const long long sx = ix + dx, sy = iy + dy;
            if (sx < 0 || sy < 0 || sx >= W || sy >= H) continue;
            const float w = (dx ? ax : 1.0f - ax) * (dy ? ay : 1.0f - ay);
            acc += w * (float)count[(size_t)sy * W + sx];
        }
    dst[(size_t)v * W + u] = acc;
}

__global__ void k_ev_to_float(const int32_t *count, size_t n, float *dst)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (float)count[i];
}

struct Kern { float w[EV_MAX_K]; int r; };

__global__ void k_ev_count(int64_t n, const uint16_t *x, const uint16_t *y, const uint8_t *pol, int W, int H,
                           int32_t *count)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int xx = x[i], yy = y[i];
        if (xx < W && yy < H) atomicAdd(count + (size_t)yy * W + xx, pol[i] ? 1 : -1);
    }
}

__global__ void k_ev_blur_h(const float *img, int W, int H, Kern k, float *tmp)
{
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    float s = 0.0f;
    for (int j = -k.r; j <= k.r; ++j) {
        int xx = min(W - 1, max(0, x + j));
        s = fmaf(k.w[j + k.r], img[(size_t)y * W + xx], s);
    }
    tmp[(size_t)y * W + x] = s;
}

__global__ void k_ev_blur_v(const float *tmp, int W, int H, Kern k, float *blur, double *part)
{
    __shared__ double red[32];
    double acc = 0.0;
    size_t P = (size_t)W * H;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < P; i += (size_t)gridDim.x * blockDim.x) {
        int x = (int)(i % W), y = (int)(i / W);
        float s = 0.0f;
        for (int j = -k.r; j <= k.r; ++j) {
            int yy = min(H - 1, max(0, y + j));
            s = fmaf(k.w[j + k.r], tmp[(size_t)yy * W + x], s);
        }
        blur[i] = s;
        acc += (double)s * (double)s;
    }
    acc = warp_sum_d(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += red[w];
        part[blockIdx.x] = t;
    }
}

// Grid-wide: every block forms the same scale from the partial sums (same order, same
// bits) and writes a grid-stride share of every pyramid level.
__global__ void k_ev_normalize(const float *blur, const double *part, int nparts, int W, int H, int levels,
                               float *out_s, float *out_u)
{
    __shared__ float scale;
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < nparts; ++i) t += part[i];
        double nrm = sqrt(t);
        scale = nrm > 2.220446049250313e-16 ? (float)(1.0 / nrm) : 0.0f;
    }
    __syncthreads();
    size_t off = 0;
    for (int l = 0; l < levels; ++l) {
        double f = 1.0;
        for (int i = 0; i < l; ++i) f *= 0.5;
        int w = (int)(W * f), h = (int)(H * f);
        double ifx = (double)W / w, ify = (double)H / h;
        size_t P = (size_t)w * h;
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < P; i += (size_t)gridDim.x * blockDim.x) {
            int x = (int)(i % w), y = (int)(i / w);
            int sx = min(W - 1, (int)floor(x * ifx)), sy = min(H - 1, (int)floor(y * ify));
            float v = blur[(size_t)sy * W + sx] * scale;
            out_s[off + i] = v;
            if (out_u) out_u[off + i] = fabsf(v);
        }
        off += P;
    }
}

// blocks of the normalisation: one thread per level-0 pixel, at most 8 blocks per SM
inline int ev_norm_blocks(int W, int H)
{
    const size_t P = (size_t)W * H;
    return (int)std::min<size_t>((P + 255) / 256, 152 * 8);
}

// Argument checks shared by both entry points; nothing is enqueued before they pass.
int ev_check(int64_t n, const uint16_t *x, const uint16_t *y, const uint8_t *polarity, int32_t width, int32_t height,
             const double *camera, int32_t ksize, int32_t levels, const float *out_signed)
{
    if (width <= 0 || height <= 0 || ksize < 1 || (ksize & 1) == 0 || ksize > EV_MAX_K || levels < 1 ||
        !out_signed || n < 0 || (n > 0 && (!x || !y || !polarity)))
        return GSEVT_ERR_ARG;
    for (int l = 1; l < levels; ++l)
        if ((int)(width * (1.0 / (1 << l))) < 1 || (int)(height * (1.0 / (1 << l))) < 1) return GSEVT_ERR_ARG;
    if (camera && !(camera[0] != 0.0 && camera[1] != 0.0)) return GSEVT_ERR_ARG;
    return GSEVT_OK;
}

// The launch sequence of the event frame over a scratch area at `base` (carved by
// ev_carve), for arguments that passed ev_check: clear the count image, count, undistort
// or convert, blur, normalise and write the pyramid.
int ev_enqueue(void *base, int64_t n, const uint16_t *x, const uint16_t *y, const uint8_t *polarity, int32_t width,
               int32_t height, const double *camera, int32_t ksize, int32_t levels, float *out_signed,
               float *out_unsigned, cudaStream_t s)
{
    EvScratch sc = ev_carve(base, width, height);
    Kern k;
    k.r = ksize / 2;
    double sigma = 0.3 * ((ksize - 1) * 0.5 - 1.0) + 0.8, ws[EV_MAX_K], sum = 0.0;
    for (int i = 0; i < ksize; ++i) {
        double xx = i - k.r;
        ws[i] = exp(-(xx * xx) / (2.0 * sigma * sigma));
        sum += ws[i];
    }
    for (int i = 0; i < EV_MAX_K; ++i) k.w[i] = i < ksize ? (float)(ws[i] / sum) : 0.0f;
    const size_t P = (size_t)width * height;
    // the count image accumulates with atomics and must start at zero on every call
    if (cudaMemsetAsync(sc.count, 0, P * 4, s) != cudaSuccess) return GSEVT_ERR_CUDA;
    if (n > 0) {
        int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)152 * 8);
        k_ev_count<<<blocks, 256, 0, s>>>(n, x, y, polarity, width, height, sc.count);
        GS_CUDA_CHECK();
    }
    dim3 gh((width + 127) / 128, height);
    if (camera) {
        Cam c = {camera[0], camera[1], camera[2], camera[3], camera[4], camera[5], camera[6], camera[7], camera[8]};
        k_ev_undistort<<<gh, 128, 0, s>>>(sc.count, width, height, c, sc.img);
    } else {
        k_ev_to_float<<<(int)std::min<size_t>((P + 255) / 256, 152 * 8), 256, 0, s>>>(sc.count, P, sc.img);
    }
    GS_CUDA_CHECK();
    k_ev_blur_h<<<gh, 128, 0, s>>>(sc.img, width, height, k, sc.tmp);
    GS_CUDA_CHECK();
    k_ev_blur_v<<<EV_PART_BLOCKS, 256, 0, s>>>(sc.tmp, width, height, k, sc.blur, sc.part);
    GS_CUDA_CHECK();
    k_ev_normalize<<<ev_norm_blocks(width, height), 256, 0, s>>>(sc.blur, sc.part, EV_PART_BLOCKS, width, height,
                                                                 levels, out_signed, out_unsigned);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

}  // namespace

extern "C" size_t gsevt_event_scratch_bytes(int32_t width, int32_t height)
{
    size_t P = (size_t)(width > 0 ? width : 1) * (size_t)(height > 0 ? height : 1);
    return 4 * gs_align(P * 4) + gs_align(EV_PART_BLOCKS * 8);
}

extern "C" int gsevt_events_accumulate(int64_t n, const uint16_t *x, const uint16_t *y, const uint8_t *polarity,
                                       int32_t width, int32_t height, const double *camera, int32_t ksize,
                                       int32_t levels, void *scratch, float *out_signed, float *out_unsigned,
                                       gsevt_stream_t stream)
{
    GS_ENTRY();
    int rc = ev_check(n, x, y, polarity, width, height, camera, ksize, levels, out_signed);
    if (rc != GSEVT_OK) return rc;
    if (!scratch) return GSEVT_ERR_ARG;
    return ev_enqueue(scratch, n, x, y, polarity, width, height, camera, ksize, levels, out_signed, out_unsigned,
                      (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------------
// gsevt_events_accumulate_noalloc: the launch sequence above over a fixed library-owned
// device buffer instead of caller scratch, for callers that cannot allocate (see the
// declaration in gsevt.h).  A __device__ variable exists once in every CUDA context the
// module is loaded into, so its address is a property of the context: it is resolved
// with cudaGetSymbolAddress the first time a call runs in a context and cached under that
// context's unique id (cuCtxGetId; ids are never reused within a process, so a context
// created after cudaDeviceReset, or one a driver-API caller made current, resolves its
// own address).  Calls that overlap on the GPU share the buffer and race.

#define EV_NOALLOC_CONTEXTS 64
#define EV_NOALLOC_BYTES (4 * ((((size_t)GSEVT_EVENTS_NOALLOC_MAX_PIXELS * 4) + 255) & ~(size_t)255) + \
                          (((size_t)EV_PART_BLOCKS * 8 + 255) & ~(size_t)255))

static __device__ __align__(256) unsigned char g_ev_noalloc_scratch[EV_NOALLOC_BYTES];

namespace {

// driver entry points, resolved through the runtime (the library links only cudart)
typedef CUresult (*CtxGetCurrentFn)(CUcontext *ctx);
typedef CUresult (*CtxGetIdFn)(CUcontext ctx, unsigned long long *id);

struct NoallocCache {
    std::mutex mu;
    CtxGetCurrentFn get_current = nullptr;
    CtxGetIdFn get_id = nullptr;
    bool resolved = false;
    int used = 0, next = 0;
    unsigned long long ids[EV_NOALLOC_CONTEXTS];
    void *addr[EV_NOALLOC_CONTEXTS];
};
NoallocCache g_noalloc;

// Address of the fixed buffer in the calling thread's current context (the current
// device's primary context when none is current yet).
int ev_noalloc_scratch(void **out)
{
    std::lock_guard<std::mutex> lock(g_noalloc.mu);
    if (!g_noalloc.resolved) {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
            qa != cudaDriverEntryPointSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
            qb != cudaDriverEntryPointSuccess || !a || !b)
            return GSEVT_ERR_CUDA;
        g_noalloc.get_current = (CtxGetCurrentFn)a;
        g_noalloc.get_id = (CtxGetIdFn)b;
        g_noalloc.resolved = true;
    }
    CUcontext ctx = nullptr;
    if (g_noalloc.get_current(&ctx) != CUDA_SUCCESS) return GSEVT_ERR_CUDA;
    if (!ctx) {
        // no context on this thread yet: bind the current device's primary context
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) return GSEVT_ERR_CUDA;
        if (g_noalloc.get_current(&ctx) != CUDA_SUCCESS || !ctx) return GSEVT_ERR_CUDA;
    }
    unsigned long long id = 0;
    if (g_noalloc.get_id(ctx, &id) != CUDA_SUCCESS) return GSEVT_ERR_CUDA;
    for (int i = 0; i < g_noalloc.used; ++i)
        if (g_noalloc.ids[i] == id) {
            *out = g_noalloc.addr[i];
            return GSEVT_OK;
        }
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_ev_noalloc_scratch) != cudaSuccess || !p) return GSEVT_ERR_CUDA;
    // a full table overwrites its entries in turn, oldest first
    const int slot = g_noalloc.next;
    g_noalloc.next = (g_noalloc.next + 1) % EV_NOALLOC_CONTEXTS;
    if (g_noalloc.used < EV_NOALLOC_CONTEXTS) ++g_noalloc.used;
    g_noalloc.ids[slot] = id;
    g_noalloc.addr[slot] = p;
    *out = p;
    return GSEVT_OK;
}

}  // namespace

extern "C" int gsevt_events_accumulate_noalloc(int64_t n, const uint16_t *x, const uint16_t *y,
                                               const uint8_t *polarity, int32_t width, int32_t height,
                                               const double *camera, int32_t ksize, int32_t levels,
                                               float *out_signed, float *out_unsigned, gsevt_stream_t stream)
{
    int rc = ev_check(n, x, y, polarity, width, height, camera, ksize, levels, out_signed);
    if (rc != GSEVT_OK) return rc;
    if ((int64_t)width * height > (int64_t)GSEVT_EVENTS_NOALLOC_MAX_PIXELS) return GSEVT_ERR_TOO_LARGE;
    GS_ENTRY();
    void *base = nullptr;
    rc = ev_noalloc_scratch(&base);
    if (rc != GSEVT_OK) return rc;
    return ev_enqueue(base, n, x, y, polarity, width, height, camera, ksize, levels, out_signed, out_unsigned,
                      (cudaStream_t)stream);
}
