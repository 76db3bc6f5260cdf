// extern "C" entry points of libgsevt.so (declared in include/gsevt.h): argument
// validation, workspace carving and the stage sequencing of one rendering frame.
#include <cstring>

#include "common.cuh"

int gs_launch_preprocess_fwd(const gsevt_frame *f, const Workspace &ws, cudaStream_t s);
int gs_launch_preprocess_bwd_cached(const gsevt_frame *f, const Workspace &ws, cudaStream_t s);
int gs_launch_preprocess_bwd(const gsevt_frame *f, const Workspace &ws, const gsevt_map_grads *grads_dev,
                             double *xi_out, cudaStream_t s,
                             bool reduce);
int gs_launch_depth_order(const gsevt_frame *f, const Workspace &ws, cudaStream_t s, bool coarse,
                          bool *binned = nullptr);
int gs_launch_bin_coarse(const gsevt_frame *f, const Workspace &ws, uint32_t max_keys, uint32_t **fine_vals,
                         cudaStream_t s, bool binned);
int gs_launch_bin(const gsevt_frame *f, const Workspace &ws, uint32_t max_keys, cudaStream_t s);
int gs_launch_blend_fwd(const gsevt_frame *f, const Workspace &ws, const uint32_t *vals, cudaStream_t s,
                        bool persist = false);
int gs_launch_blend_bwd(const gsevt_frame *f, const Workspace &ws, const uint32_t *vals, const float *dL_dimage,
                        const float *dL_ddepth, const float *dL_dalpha, cudaStream_t s, bool persist = false);
bool gs_blend_persistent(const gsevt_frame *f);
int gs_launch_tile_order(const gsevt_frame *f, const Workspace &ws, cudaStream_t s);
int gs_launch_loss(const gsevt_frame *f, const Workspace &ws, double *loss_out, cudaStream_t s);
int gs_launch_track_finalize(const gsevt_frame *f, const Workspace &ws, gsevt_pose_state *poses, int num_poses,
                             const double *loss, cudaStream_t s);

namespace {

// extra workspace tail: the device copy of the per-map gradient table
size_t grads_tab_bytes(const gsevt_layout &L) { return gs_align((size_t)(L.num_maps > 0 ? L.num_maps : 1) * sizeof(gsevt_map_grads)); }

int check_frame(const gsevt_frame *f, Workspace *ws)
{
    if (!f) return GSEVT_ERR_ARG;
    const gsevt_layout &L = f->L;
    if (L.num_views <= 0 || L.num_maps <= 0 || L.num_vg < 0 || L.num_scan_blocks < 0 || L.total_tiles <= 0 ||
        L.total_pixels <= 0 || (L.channels != 1 && L.channels != 3) || L.sort_bits < 33 || L.sort_bits > 64 ||
        L.key_capacity >= (1u << 30))
        return GSEVT_ERR_ARG;
    if (!f->views || !f->maps || !f->workspace || !f->image || !f->final_T) return GSEVT_ERR_ARG;
    Workspace w = gs_carve(L, f->workspace);
    if (f->workspace_bytes < w.bytes + grads_tab_bytes(L)) return GSEVT_ERR_WORKSPACE;
    *ws = w;
    return GSEVT_OK;
}

int sorted_buffer(const gsevt_frame *f) { return gs_tile_sort_buffer(f->L); }

}  // namespace

extern "C" size_t gsevt_workspace_bytes(const gsevt_layout *L)
{
    if (!L) return 0;
    return gs_carve(*L, nullptr).bytes + grads_tab_bytes(*L);
}

extern "C" int gsevt_workspace_init(const gsevt_frame *f, gsevt_stream_t stream)
{
    GS_ENTRY();
    Workspace ws;
    int st = check_frame(f, &ws);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    gs_sort_prepare();
    cudaMemsetAsync(ws.status, 0, 64, s);
    cudaMemsetAsync(ws.sort_lookback, 0, (size_t)gs_lookback_tiles(f->L) * 256 * 8, s);
    if (f->L.num_pairs > 0) cudaMemsetAsync(ws.loss_done, 0, (size_t)f->L.num_pairs * 4, s);
    // tile and super-tile ranges always point inside the value buffers, even where a step
    // whose layout check failed (GSEVT_STATUS_LAYOUT) or whose sort gave up
    // (GSEVT_STATUS_SORT_TIMEOUT) leaves them unwritten
    cudaMemsetAsync(ws.ranges, 0, (size_t)f->L.total_tiles * sizeof(uint2), s);
    cudaMemsetAsync(ws.sranges, 0, (size_t)gs_super_bound(f->L) * sizeof(uint2), s);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

extern "C" void gsevt_abi_sizes(int32_t *out7)
{
    if (!out7) return;
    out7[0] = (int32_t)sizeof(gsevt_view);
    out7[1] = (int32_t)sizeof(gsevt_map);
    out7[2] = (int32_t)sizeof(gsevt_map_grads);
    out7[3] = (int32_t)sizeof(gsevt_pair);
    out7[4] = (int32_t)sizeof(gsevt_layout);
    out7[5] = (int32_t)sizeof(gsevt_frame);
    out7[6] = (int32_t)sizeof(gsevt_pose_state);
}

extern "C" void gsevt_workspace_offsets(const gsevt_layout *L, uint64_t *out)
{
    if (!L || !out) return;
    // carve against a fake non-null base so absent regions stay null
    char *base = (char *)(uintptr_t)4096;
    Workspace w = gs_carve(*L, base);
    // recA / recB: the two halves of the interleaved 32-byte blend records
    const void *ptrs[GS_WS_REGIONS] = {w.status, w.bin, w.rec, w.rec + 1, w.recC, w.gradA, w.gradB, w.gradC,
                                       w.vis_sums, w.vis_offs, w.dkeys[0], w.dkeys[1], w.dvals[0], w.dvals[1],
                                       w.tsums, w.toffs, w.keys[0], w.keys[1], w.vals[0], w.vals[1], w.sort_hist,
                                       w.sort_counter, w.sort_lookback, w.ranges, w.loss_part, w.loss_scal,
                                       w.loss_done, w.xi_part, w.xi, w.csums, w.coffs, w.soffs,
                                       w.sranges, w.fcache};
    for (int i = 0; i < GS_WS_REGIONS; ++i)
        out[i] = ptrs[i] ? (uint64_t)((const char *)ptrs[i] - base) : UINT64_MAX;
}

extern "C" int gsevt_clear_status(const gsevt_frame *f, gsevt_stream_t stream)
{
    GS_ENTRY();
    Workspace ws;
    int st = check_frame(f, &ws);
    if (st) return st;
    cudaMemsetAsync(ws.status, 0, 8, (cudaStream_t)stream);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

extern "C" int gsevt_read_status(const gsevt_frame *f, uint32_t *out2, gsevt_stream_t stream)
{
    GS_ENTRY();
    Workspace ws;
    int st = check_frame(f, &ws);
    if (st) return st;
    if (!out2) return GSEVT_ERR_ARG;
    if (cudaMemcpyAsync(out2, ws.status, 8, cudaMemcpyDeviceToHost, (cudaStream_t)stream) != cudaSuccess)
        return GSEVT_ERR_CUDA;
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return GSEVT_ERR_CUDA;
    return GSEVT_OK;
}

extern "C" int gsevt_preprocess_fwd(const gsevt_frame *f, gsevt_stream_t stream)
{
    GS_ENTRY();
    Workspace ws;
    int st = check_frame(f, &ws);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemsetAsync(ws.status, 0, 8, s);
    GS_CUDA_CHECK();
    st = gs_launch_preprocess_fwd(f, ws, s);
    if (st) return st;
    return gs_launch_depth_order(f, ws, s, false);
}

extern "C" int gsevt_bin_and_sort(const gsevt_frame *f, uint32_t max_keys, gsevt_stream_t stream)
{
    GS_ENTRY();
    Workspace ws;
    int st = check_frame(f, &ws);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (max_keys == 0 || max_keys > f->L.key_capacity) max_keys = f->L.key_capacity;
    return gs_launch_bin(f, ws, max_keys, s);
}

extern "C" int gsevt_blend_fwd(const gsevt_frame *f, gsevt_stream_t stream)
{
    GS_ENTRY();
    Workspace ws;
    int st = check_frame(f, &ws);
    if (st) return st;
    return gs_launch_blend_fwd(f, ws, ws.vals[sorted_buffer(f)], (cudaStream_t)stream);
}

extern "C" int gsevt_loss_fwd(const gsevt_frame *f, double *loss_out, gsevt_stream_t stream)
{
    GS_ENTRY();
    Workspace ws;
    int st = check_frame(f, &ws);
    if (st) return st;
    if (f->L.channels != 1) return GSEVT_ERR_ARG;
    return gs_launch_loss(f, ws, loss_out, (cudaStream_t)stream);
}

extern "C" int gsevt_blend_bwd(const gsevt_frame *f, const float *dL_dimage, const float *dL_ddepth,
                               const float *dL_dalpha, gsevt_stream_t stream)
{
    GS_ENTRY();
    Workspace ws;
    int st = check_frame(f, &ws);
    if (st) return st;
    if (!dL_dimage && (!f->pairs || f->L.channels != 1)) return GSEVT_ERR_ARG;
    if (dL_ddepth && !f->depth) return GSEVT_ERR_ARG;
    if (dL_dalpha && !f->alpha) return GSEVT_ERR_ARG;
    return gs_launch_blend_bwd(f, ws, ws.vals[sorted_buffer(f)], dL_dimage, dL_ddepth, dL_dalpha,
                               (cudaStream_t)stream);
}

extern "C" int gsevt_preprocess_bwd(const gsevt_frame *f, double *xi_out, const gsevt_map_grads *grads,
                                    gsevt_stream_t stream)
{
    GS_ENTRY();
    Workspace ws;
    int st = check_frame(f, &ws);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    gsevt_map_grads *dev_tab = nullptr;
    if (grads) {
        dev_tab = (gsevt_map_grads *)((char *)f->workspace + ws.bytes);
        if (cudaMemcpyAsync(dev_tab, grads, sizeof(gsevt_map_grads) * f->L.num_maps, cudaMemcpyHostToDevice, s) !=
            cudaSuccess)
            return GSEVT_ERR_CUDA;
    }
    return gs_launch_preprocess_bwd(f, ws, dev_tab, xi_out, s, true);
}

extern "C" int gsevt_track_step_batched(const gsevt_frame *f, gsevt_pose_state *poses, int32_t num_poses,
                                        double *loss_out, gsevt_stream_t stream)
{
    GS_ENTRY();
    Workspace ws;
    int st = check_frame(f, &ws);
    if (st) return st;
    if (!poses || num_poses <= 0 || !f->pairs || f->L.num_pairs <= 0 || f->L.channels != 1) return GSEVT_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    // binning through super-tiles: the same per-tile lists as gsevt_bin_and_sort
    cudaMemsetAsync(ws.status, 0, 8, s);
    GS_CUDA_CHECK();
    if ((st = gs_launch_preprocess_fwd(f, ws, s))) return st;
    bool binned = false;
    if ((st = gs_launch_depth_order(f, ws, s, true, &binned))) return st;
    uint32_t *fine = nullptr;
    if ((st = gs_launch_bin_coarse(f, ws, f->L.key_capacity, &fine, s, binned))) return st;
    const bool persist = gs_blend_persistent(f);
    if (persist && (st = gs_launch_tile_order(f, ws, s))) return st;
    if ((st = gs_launch_blend_fwd(f, ws, fine, s, persist))) return st;
    if ((st = gs_launch_loss(f, ws, loss_out, s))) return st;
    if ((st = gs_launch_blend_bwd(f, ws, fine, nullptr, nullptr, nullptr, s, persist))) return st;
    if ((st = gs_launch_preprocess_bwd_cached(f, ws, s))) return st;
    return gs_launch_track_finalize(f, ws, poses, num_poses, loss_out, s);
}
