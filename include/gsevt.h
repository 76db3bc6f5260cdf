/*
 * gsevt — C ABI of the GB300-native tracking hot path of GS-EVT (libgsevt.so).
 *
 * The reference binds its rasterizer as a Python extension of the absent submodule
 * diff-gaussian-rasterization-vwRT (.gitmodules:1-3); its interface is known from the
 * call sites gaussian_splatting/gaussian_renderer/__init__.py:313-383
 * (GaussianRasterizationSettings fields :318-337, GaussianRasterizer forward
 * arguments :362-375, 5-tuple return :362).  Each entry point below names the part of
 * that interface, or of the tracker around it, that it replaces.
 *
 * Conventions
 *   - All buffers are device memory owned by the caller, except the gsevt_frame /
 *     gsevt_layout structs themselves, which are host memory read at call time.
 *   - Work is enqueued on the stream passed in; calls return before the GPU finishes.
 *   - Every call returns an int status (GSEVT_OK = 0 or a negative code).  Nothing
 *     throws across the ABI.  Device-side failures (key-buffer overflow, a bounded
 *     wait that ran out) are recorded in the frame's status words and read back with
 *     gsevt_read_status.
 *   - No entry point allocates device memory: scratch lives in the caller-provided
 *     workspace sized by gsevt_workspace_bytes (gsevt_events_accumulate_noalloc uses a
 *     fixed library-owned buffer instead; see its declaration).
 *   - Re-entrant per stream.  Process-wide state: the cooperative sort's grid per device
 *     (set once by gsevt_workspace_init), and the no-allocation event frame's fixed
 *     buffer with its per-context address cache.
 *   - Every entry point that enqueues work first clears a non-sticky CUDA error that an
 *     earlier, unrelated call left pending, so that GSEVT_ERR_CUDA always refers to the
 *     call's own launches and copies.
 */
#ifndef GSEVT_H
#define GSEVT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *gsevt_stream_t; /* = cudaStream_t */

enum {
    GSEVT_OK = 0,
    GSEVT_ERR_ARG = -1,          /* bad shape, size or pointer */
    GSEVT_ERR_KEY_OVERFLOW = -2, /* more (tile, Gaussian) pairs than the key capacity */
    GSEVT_ERR_NONFINITE = -3,    /* non-finite loss or gradient */
    GSEVT_ERR_TIMEOUT = -4,      /* a bounded device-side wait ran out */
    GSEVT_ERR_CUDA = -5,         /* a CUDA launch or copy failed */
    GSEVT_ERR_WORKSPACE = -6     /* workspace smaller than gsevt_workspace_bytes */
};

/* status word bits, in gsevt_read_status()[0] */
#define GSEVT_STATUS_KEY_OVERFLOW 1u
#define GSEVT_STATUS_SORT_TIMEOUT 2u
#define GSEVT_STATUS_NONFINITE 4u
#define GSEVT_STATUS_LAYOUT 8u /* the views need more super-tiles than layout.super_tiles */
#define GSEVT_STATUS_STAGE_TIMEOUT 16u /* a blend's wait for its staged batch ran out */

#define GSEVT_TILE 16
#define GSEVT_LOSS_PIXELS_PER_BLOCK 2048 /* pixels reduced by one loss block */
#define GSEVT_MAP_PLANES 15 /* packed map: 15 float4 planes of n entries */

/* One rendered view (device-resident table entry, 192 bytes).  Replaces the per-call
 * GaussianRasterizationSettings record (gaussian_renderer/__init__.py:318-337):
 * viewmatrix -> R, t; projmatrix_raw -> P; campos; tanfovx/y; bg; image size. */
typedef struct gsevt_view {
    float R[9];       /* world -> camera rotation, row-major */
    float t[3];       /* world -> camera translation */
    float P[16];      /* camera -> clip projection, row-major (projmatrix_raw^T) */
    float campos[3];  /* camera centre in world coordinates */
    float tanfovx, tanfovy;
    float bg[3];      /* background colour (grey uses 0.2989/0.5870/0.1140 weights) */
    int32_t width, height;
    int32_t tiles_x, tiles_y;
    int32_t tile_offset;  /* first global tile id of this view */
    int32_t pix_offset;   /* first pixel of this view in per-pixel buffers */
    int32_t map;          /* index into the map table */
    int32_t vg_offset;    /* first (view, Gaussian) slot of this view */
    int32_t sb_offset;    /* first scan block of this view */
    int32_t pair;         /* render pair this view belongs to, or -1 */
    int32_t pair_role;    /* 0: t (last), 1: t + dtau (next) */
    int32_t skip;         /* 1: render nothing for this view (every Gaussian is culled); the
                           * batched step sets it for the views of a problem whose pyramid
                           * level has finished, gsevt_track_init_views clears it */
} gsevt_view;

/* One Gaussian map (device-resident table entry).  Exactly one colour source
 * (shs or colors) and one covariance source (scales+rotations or cov3d) or the packed
 * planes, mirroring the rasterizer's "exactly one of" rules
 * (gaussian_renderer/__init__.py:80-113). */
typedef struct gsevt_map {
    const float *xyz;        /* [n][3] means3D */
    const float *opacity;    /* [n] activated opacity */
    const float *scales;     /* [n][3] activated scales, or NULL */
    const float *rotations;  /* [n][4] (w,x,y,z) normalised, or NULL */
    const float *cov3d;      /* [n][6] cov3D_precomp, or NULL */
    const float *shs;        /* [n][sh_coeffs][3], or NULL */
    const float *colors;     /* [n][3] colors_precomp, or NULL */
    const void *packed;      /* [15][n] float4 planes from gsevt_pack_map, or NULL */
    int32_t n;
    int32_t sh_degree;       /* active SH degree 0..3 */
    int32_t sh_coeffs;       /* coefficients per channel in shs (>= (deg+1)^2) */
    float scale_modifier;
    int32_t first_view;      /* views of this map are contiguous in the view table */
    int32_t num_views;
    int32_t block_offset;    /* first preprocess block of this map */
    int32_t pad;
} gsevt_map;

/* Per-map gradient outputs of gsevt_preprocess_bwd (all nullable; device pointers).
 * Gradients are written (not accumulated) for every Gaussian of the map. */
typedef struct gsevt_map_grads {
    float *means3d;    /* [n][3] */
    float *means2d;    /* [n][3] dL/d(NDC x, y), z = 0 (the means2D convention) */
    float *opacity;    /* [n] */
    float *scales;     /* [n][3] */
    float *rotations;  /* [n][4] */
    float *cov3d;      /* [n][6] */
    float *shs;        /* [n][sh_coeffs][3] */
    float *colors;     /* [n][3] */
} gsevt_map_grads;

/* A (t, t + dtau) render pair and its event frame (utils/render_camera/frame.py:86-94,
 * utils/tracker.py:93-103).  The intensity change is dI = I_next - I_last of the grey
 * renders (the reference's linear grey, frame.py:39-43,86-92), or with log_grey set the
 * log-intensity change of the paper, dI = ln(I_next + log_eps) - ln(I_last + log_eps),
 * applied per pixel after blending. */
typedef struct gsevt_pair {
    int32_t last_view, next_view;
    const float *event;      /* [H][W] signed event frame E */
    const float *event_abs;  /* [H][W] |E| (unsigned mode); NULL: use |event| */
    int32_t unsigned_mode;   /* 0: L = ||n - E||, 1: L = || |n| - |E| || */
    int32_t pose;            /* pose state this pair belongs to (batched tracker) */
    int32_t block_offset;    /* first loss-reduction block of this pair */
    int32_t num_blocks;
    int32_t log_grey;        /* 0: linear grey (default), 1: log grey */
    float log_eps;           /* offset inside the logarithm (log_grey only), > 0 */
} gsevt_pair;

/* Launch choices of a frame; all zeros select the library's defaults.  The autotuner
 * (gsevt.tuner) times the alternatives per workload shape and keeps the fastest. */
typedef struct gsevt_tuning {
    int32_t blend_staging;   /* how a blend block stages its batch of 256 records in shared
                              * memory: 0 or 1, one 16-byte cp.async per record half and thread;
                              * 2, TMA tile::gather4 tensor copies issued by one warp; 3, the
                              * same issued by every warp for its 32 candidates (the grey
                              * tracker blends; the RGB drop-in blends always use cp.async) */
    int32_t depth_sort_kpt;  /* keys per thread of the onesweep depth sort: 0 (= 12), 4, 8, 12 */
    int32_t pair_sort_kpt;   /* keys per thread of the onesweep pair sorts: 0 (= 12), 4, 8, 12 */
    int32_t coop_sort;       /* 0: sorts that fit run as one cooperative launch, 1: never */
    int32_t blend_schedule;  /* batched step's grey blends: 0, one block per tile in tile
                              * order; 1, longest tile lists first: the one-pixel blends run
                              * as resident blocks taking tiles from one work queue holding
                              * every view's tiles, the two-pixel blends launch one block per
                              * tile in that order */
    int32_t adjoint_pixels;  /* pixels per lane of the tracker adjoint blend: 0 or 2, two
                              * (128 threads per tile, 8x8-pixel warps, batches of 128
                              * records, cp.async staging whatever blend_staging says); 1, one
                              * (256 threads per tile, 8x4-pixel warps, the staging above) */
    int32_t forward_pixels;  /* pixels per lane of the grey forward blend without extras (the
                              * batched step): 0 or 2, two (128 threads per tile, 8x8-pixel
                              * warps, batches of 128 records, cp.async staging); 1, one (256
                              * threads per tile, the staging above); the images are the same
                              * bits either way */
    int32_t reserved[1];
} gsevt_tuning;

/* Sizes of one rendering frame (host struct). */
typedef struct gsevt_layout {
    int32_t num_views, num_maps, num_pairs;
    int32_t num_vg;             /* sum over views of the view's map size */
    int32_t num_scan_blocks;    /* sum over views of ceil(n / 256) */
    int32_t preprocess_blocks;  /* sum over maps of ceil(n / 256) */
    int32_t total_tiles, total_pixels;
    int32_t channels;           /* 3 = RGB (drop-in), 1 = grey (tracker) */
    int32_t sort_bits;          /* 32 + bits of (total_tiles - 1) */
    uint32_t key_capacity;      /* max (tile, Gaussian) pairs */
    int32_t loss_blocks;        /* sum over pairs of loss-reduction blocks */
    int32_t super_tiles;        /* sum over views of ceil(tiles_x / 4) * ceil(tiles_y / 4)
                                 * (the batched step's 4x4-tile super-tiles); 0: use the
                                 * bound total_tiles / 4 + num_views + 1, which can cost the
                                 * super-tile sort a second pass */
    uint32_t spin_limit;        /* polls a bounded device wait (sort look-back, cooperative
                                 * grid barrier) makes before it gives up and records
                                 * GSEVT_STATUS_SORT_TIMEOUT; 0: the default, 2^22.  After a
                                 * timeout the stages that follow the sort do nothing (no
                                 * image, loss or pose update) until the status is cleared,
                                 * which every gsevt_preprocess_fwd and
                                 * gsevt_track_step_batched call does first. */
    gsevt_tuning tuning;        /* launch choices (zeros: defaults) */
} gsevt_layout;

/* One rendering frame: layout, device tables, workspace and caller-owned outputs. */
typedef struct gsevt_frame {
    gsevt_layout L;
    const gsevt_view *views;   /* device [num_views] */
    const gsevt_map *maps;     /* device [num_maps] */
    const gsevt_pair *pairs;   /* device [num_pairs] or NULL */
    void *workspace;           /* device, gsevt_workspace_bytes(&L) */
    size_t workspace_bytes;
    float *image;              /* [channels][total_pixels] */
    float *final_T;            /* [total_pixels] */
    float *depth;              /* [total_pixels] or NULL */
    float *alpha;              /* [total_pixels] or NULL */
    int32_t *n_contrib;        /* [total_pixels] or NULL */
    int32_t *radii;            /* [num_vg] or NULL */
    int32_t *n_touched;        /* [num_vg] or NULL */
} gsevt_frame;

/* ---- sizing ---- */
size_t gsevt_workspace_bytes(const gsevt_layout *L);
/* Zero the parts of a fresh workspace that must start at zero (status words, sort
 * look-back table, loss tickets, tile ranges) and set up the single-launch cooperative
 * sort on the current device.  Call once after allocating it, outside stream capture. */
int gsevt_workspace_init(const gsevt_frame *f, gsevt_stream_t stream);
/* sizeof of the ABI structs, for binding checks: view, map, map_grads, pair, layout,
 * frame, pose_state (7 entries).  Touches no GPU state. */
void gsevt_abi_sizes(int32_t *out7);
/* Byte offsets of the workspace regions for a layout (introspection for tests and
 * tools), in this order: status, bin, recA, recB (the two float4 halves of one 32-byte
 * record per slot, so both have a 32-byte stride), recC, gradA, gradB, gradC, vis_sums,
 * vis_offs, dkeys0, dkeys1, dvals0, dvals1, tsums, toffs, keys0, keys1, vals0, vals1,
 * sort_hist, sort_counter, sort_lookback, ranges, loss_part, loss_scal, loss_done,
 * xi_part, xi, csums, coffs, soffs, sranges, fcache (34 entries; absent regions are
 * reported as UINT64_MAX).  keys are 32-bit global tile ids, vals 32-bit (view, Gaussian)
 * slots.  Touches no GPU state. */
void gsevt_workspace_offsets(const gsevt_layout *L, uint64_t *out34);

/* ---- map packing ----
 * Replaces the per-call activation + torch.cat of get_features
 * (gaussian_renderer/__init__.py:277-297, gaussian_model.py:75-95): packs a map once
 * into 15 float4 planes {x,y,z,opacity}, {cov xx,xy,xz,yy}, {yz,zz,0,0}, 12 x SH. */
int gsevt_pack_map(int32_t n, const float *xyz, const float *opacity, const float *scales,
                   const float *rotations, const float *cov3d, const float *shs,
                   int32_t sh_coeffs, float scale_modifier, void *packed, gsevt_stream_t stream);

/* ---- forward stages (GaussianRasterizer.forward, gaussian_renderer/__init__.py:362-375) ----
 * preprocess: per (view, Gaussian) projection, EWA conic, radius, tile rect, SH colour.
 * Also writes radii (the forward's 2nd return value) when frame->radii is set. */
int gsevt_preprocess_fwd(const gsevt_frame *f, gsevt_stream_t stream);
/* key duplication in depth order, onesweep radix sort by (view|tile), tile ranges: the
 * order of a stable sort of (view|tile|depth) keys.
 * max_keys bounds the sort grid: the host-known key count (after gsevt_read_status),
 * or 0 to size it from the key capacity (no host sync; CUDA-graph friendly). */
int gsevt_bin_and_sort(const gsevt_frame *f, uint32_t max_keys, gsevt_stream_t stream);
/* per-tile front-to-back blend: image, final T, depth, opacity, n_touched */
int gsevt_blend_fwd(const gsevt_frame *f, gsevt_stream_t stream);

/* ---- loss (utils/render_camera/frame.py:86-94 + utils/tracker.py:93-103) ----
 * Per pair reductions in FP64; loss_out[p] = L of pair p (device doubles). */
int gsevt_loss_fwd(const gsevt_frame *f, double *loss_out, gsevt_stream_t stream);

/* ---- backward (GaussianRasterizer backward, implicit in loss.backward(),
 *      utils/tracker.py:212) ----
 * blend adjoint: per-Gaussian 2D gradients.  dL_dimage ([channels][total_pixels]) etc.
 * come from the caller (drop-in); when dL_dimage is NULL the per-pixel gradient is
 * formed from the pair losses computed by gsevt_loss_fwd (tracker). */
int gsevt_blend_bwd(const gsevt_frame *f, const float *dL_dimage, const float *dL_ddepth,
                    const float *dL_dalpha, gsevt_stream_t stream);
/* preprocess adjoint: per-view left-twist gradient xi_out[v][6] = dL/d(rho, theta) of
 * view v (FP32 per Gaussian, warp-reduced, FP64 across blocks), plus map gradients
 * for map m into grads[m] (host array of num_maps structs, nullable). */
int gsevt_preprocess_bwd(const gsevt_frame *f, double *xi_out, const gsevt_map_grads *grads,
                         gsevt_stream_t stream);

/* Chain one view's twist gradient to the 12 optimised deltas of the drop-in call
 * (theta, rho, w, v: gaussian_renderer/__init__.py:301-304) using the settings'
 * vel_transofrm (4x4, transposed as passed, :266-269), delta_time (:270-271) and the
 * current velocities (:331-332).  Exact SE(3) adjoint and left Jacobian, FP64.
 * out12 = [theta(3), rho(3), w(3), v(3)] as float, written (not accumulated). */
int gsevt_chain_view_grad(const double *xi, const float *vel_transform_t, float delta_time,
                          const float *linear_vel, const float *angular_vel, float *out12,
                          gsevt_stream_t stream);

/* Build a view entry on the device from the drop-in settings tensors without a host
 * sync: viewmatrix (4x4, transposed world_view_transform), projmatrix_raw (4x4,
 * transposed), campos[3], bg[3]. */
int gsevt_view_from_settings(const float *viewmatrix_t, const float *projmatrix_raw_t,
                             const float *campos, const float *bg, float tanfovx, float tanfovy,
                             int32_t width, int32_t height, int32_t tile_offset,
                             int32_t pix_offset, int32_t map, int32_t vg_offset,
                             int32_t sb_offset, gsevt_view *view_out, gsevt_stream_t stream);

/* Copy the frame's status words to host (synchronises the stream):
 * out[0] = status bits, out[1] = number of keys (tile, Gaussian pairs). */
int gsevt_read_status(const gsevt_frame *f, uint32_t *out2, gsevt_stream_t stream);
/* Clear the status words (enqueued on the stream). */
int gsevt_clear_status(const gsevt_frame *f, gsevt_stream_t stream);

/* ---- event frame (utils/event_camera/event.py:116-128, tracker.py:78-91) ----
 * count += +1/-1 per event (int32 atomics); when camera (host array {fx, fy, cx, cy,
 * k1, k2, p1, p2, k3}) is non-NULL, undistortion as cv2.undistort with the camera matrix
 * reused (source position rounded to 1/32 pixel, bilinear, zero border); separable ksize
 * Gaussian blur (sigma = 0.3((ksize-1)/2 - 1) + 0.8, replicate border), L2
 * normalisation, |E|, and nearest-neighbour pyramid levels.  out_signed / out_unsigned
 * hold the levels back to back: level l is int(W*0.5^l) x int(H*0.5^l).  scratch must
 * hold gsevt_event_scratch_bytes(W, H). */
size_t gsevt_event_scratch_bytes(int32_t width, int32_t height);
int gsevt_events_accumulate(int64_t n, const uint16_t *x, const uint16_t *y,
                            const uint8_t *polarity, int32_t width, int32_t height,
                            const double *camera, int32_t ksize, int32_t levels, void *scratch,
                            float *out_signed, float *out_unsigned, gsevt_stream_t stream);

/* gsevt_events_accumulate without the scratch argument; it allocates nothing.  This entry
 * point has no counterpart in the reference (which builds its event frame on the host).
 * It is for callers that cannot allocate device memory: a C sensor-driver callback that
 * turns each event packet into a frame and holds no device allocator, a host whose device
 * memory is all handed to its own pool, or a per-packet path that must not pay
 * cudaMalloc's implicit device synchronisation.
 *   - Scratch is one fixed library-owned buffer per CUDA context, sized for frames of up
 *     to GSEVT_EVENTS_NOALLOC_MAX_PIXELS pixels (1280 x 720; 14,747,648 bytes of device
 *     memory, reserved when the library's event module is loaded into a context, which
 *     under CUDA's default lazy module loading is its first use there, and held until
 *     the context ends).  width * height above that returns GSEVT_ERR_TOO_LARGE before
 *     anything is enqueued.
 *   - Set-up: the first call in each context (a device's primary context, or a context
 *     the caller created and made current) resolves the buffer's address there with
 *     cudaGetSymbolAddress and caches it under the context's unique id, so a context
 *     created later (after cudaDeviceReset, say) resolves its own; make that first call
 *     outside any stream capture.
 *   - The count image that must start at zero is cleared on the stream by every call;
 *     the other scratch regions are fully overwritten.
 *   - Calls that overlap on one device (two streams, or two host threads, without an
 *     ordering between them) share the buffer and race: order them on one stream or
 *     wait for the previous call to finish.
 * Outputs and every other argument are as for gsevt_events_accumulate. */
#define GSEVT_EVENTS_NOALLOC_MAX_PIXELS (1280 * 720)
enum { GSEVT_ERR_TOO_LARGE = -7 };  /* input larger than a fixed-size scratch buffer, or an
                                     * output capacity, holds */
int gsevt_events_accumulate_noalloc(int64_t n, const uint16_t *x, const uint16_t *y,
                                    const uint8_t *polarity, int32_t width, int32_t height,
                                    const double *camera, int32_t ksize, int32_t levels,
                                    float *out_signed, float *out_unsigned, gsevt_stream_t stream);

/* Event-file ingestion (replaces load_events_from_txt's line loop,
 * utils/event_camera/event.py:11-39): parses a buffer holding the file's text, one event
 * per line as "ts x y polarity" decimal integers separated by spaces or tabs, into host
 * arrays ts[i] (the timestamp as written, microseconds), x[i], y[i] (0..65535) and
 * polarity[i] = (p != 0).  Blank lines are skipped.  Host memory only: it launches
 * nothing and needs no GPU.  capacity: entries of each output array, at least the number
 * of lines in the buffer (GSEVT_ERR_TOO_LARGE otherwise, nothing parsed); threads: host
 * threads to use (0: the hardware's count; buffers under 1 MB use one).  A line that is
 * not four integers ends the parse with GSEVT_ERR_ARG and *count = the events before it. */
int gsevt_parse_events_txt(const char *text, size_t len, int64_t *ts, uint16_t *x, uint16_t *y,
                           uint8_t *polarity, size_t capacity, size_t *count, int32_t threads);

/* ---- batched tracker iteration (utils/tracker.py:176-240) ----
 * Per pose state (one tracking hypothesis / sequence): FP64 pose, velocity, Adam
 * moments.  One call = render all pairs, loss, adjoint, exact chain to
 * (theta, rho, w, v), Adam step with the reference's four parameter groups, pose and
 * velocity update, and rewrite of the pose's two view-table entries. */
typedef struct gsevt_pose_state {
    double R[9], t[3];           /* current world -> camera pose */
    double lin_vel[3], ang_vel[3];
    double delta_tau;
    double m[12], v[12];         /* Adam moments: theta, rho, w, v */
    double lr[4];                /* base learning rates theta, rho, w, v */
    double lr_scale[4];          /* current multipliers (velocity ramp) */
    int32_t step[4];             /* Adam step per group */
    int32_t opt_vel;             /* 0: coarse stage (theta, rho), 1: fine stage (all 12) */
    int32_t last_view, next_view;
    int32_t iter;
    int32_t pad;
    float fx, fy;                /* focal lengths of the rendered views */
    double loss;                 /* last loss */
    double grad[12];             /* last gradient (theta, rho, w, v) */
    /* per-level stage control (utils/tracker.py:149-240), used when control != 0:
     * coarse stage (opt_vel 0, unsigned loss) until the loss slope converges, then fine
     * stage (opt_vel 1, signed loss, velocity learning-rate ramp) until it converges
     * again or max_iter more iterations pass; then the problem is frozen. */
    int32_t control;
    int32_t frozen;
    int32_t level_iter;          /* optim_iter of the current level */
    int32_t start_vel;           /* start_vel_opt_iter */
    int32_t hist_n;              /* losses recorded in this level */
    int32_t max_iter;            /* max_optim_iter */
    double conv_thr;             /* converged_threshold */
    double hist[11];             /* last 11 losses of this level (ring) */
} gsevt_pose_state;

/* poses: device array.  Pair p's loss goes to loss_out[p] (device, nullable).
 * The frame must be grey (channels == 1) with render pairs; its workspace then carries
 * the forward cache the twist-only adjoint reads.  Binning goes through 4x4-tile
 * super-tiles and yields the same per-tile lists as gsevt_bin_and_sort (depth order,
 * ties in slot order); the key capacity bounds the (tile, Gaussian) pairs as there, and
 * an overflow is flagged in the status words with every tile range left inside the
 * buffers.  Call gsevt_track_init_views once before the first step. */
int gsevt_track_step_batched(const gsevt_frame *f, gsevt_pose_state *poses, int32_t num_poses,
                             double *loss_out, gsevt_stream_t stream);
/* Write the two view entries (pose R, t, campos) of every pose from its state; the
 * other view fields (size, projection, offsets, pair) are set by the caller. */
int gsevt_track_init_views(gsevt_view *views, const gsevt_pose_state *poses, int32_t num_poses,
                           gsevt_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* GSEVT_H */
