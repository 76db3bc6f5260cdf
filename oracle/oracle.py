"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm use
this module.  It wraps oracle/gsevt_oracle.c (see the header there for what is
restated from which reference file and what is "parity unpinned") and composes the
per-view functions into the full FP32 rasterization of one view and the FP64
frozen-decision forward/backward used for finite differences.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def _opt(t):
    """ndpointer that also accepts None."""
    class _P(t):
        @classmethod
        def from_param(cls, obj):
            if obj is None:
                return None
            return t.from_param(obj)
    return _P


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        L.or_exp2f_export.restype = C.c_float
        L.or_exp2f_export.argtypes = [C.c_float]
        L.or_cov3d.argtypes = [C.c_int, f32p, f32p, C.c_float, f32p]
        L.or_sh_eval_f64.argtypes = [C.c_int, C.c_int, f32p, f64p, f64p]
        L.or_preprocess.argtypes = [C.c_int, f32p, f32p, _opt(f32p), C.c_int, _opt(f32p), f32p,
                                    C.c_int, C.c_int, i32p, i32p, f32p, f32p, f32p, f32p, f32p,
                                    _opt(i32p)]
        L.or_duplicate.restype = C.c_int64
        L.or_duplicate.argtypes = [C.c_int, i32p, f32p, i32p, f32p, C.c_int, C.c_int, C.c_uint32,
                                   C.c_uint32, u64p, u32p]
        L.or_sort_pairs.argtypes = [C.c_int64, u64p, u32p, C.c_int]
        L.or_ranges.argtypes = [C.c_int64, u64p, C.c_int, u32p]
        L.or_blend_fwd.argtypes = [C.c_int, C.c_int, C.c_int, u32p, u32p, f32p, f32p, f32p, f32p,
                                   _opt(f32p), f32p, f32p, _opt(f32p), _opt(f32p), _opt(f32p),
                                   _opt(i32p), _opt(i32p), _opt(i32p), _opt(i64p), _opt(u32p),
                                   _opt(u8p)]
        L.or_frozen_render_f64.restype = C.c_int
        L.or_frozen_render_f64.argtypes = [C.c_int, f32p, _opt(f32p), _opt(f32p), _opt(f32p),
                                           C.c_double, f32p, _opt(f32p), C.c_int, _opt(f32p), f64p,
                                           C.c_int, C.c_int, C.c_int, f64p, i64p, u32p, u8p, f64p,
                                           _opt(f64p), _opt(f64p)]
        L.or_frozen_backward_f64.argtypes = [C.c_int, f32p, _opt(f32p), _opt(f32p), _opt(f32p),
                                             C.c_double, f32p, _opt(f32p), C.c_int, _opt(f32p), f64p,
                                             C.c_int, C.c_int, C.c_int, f64p, i64p, u32p, u8p, f64p,
                                             _opt(f64p), _opt(f64p), f64p, _opt(f64p), _opt(f64p),
                                             _opt(f64p), _opt(f64p), _opt(f64p), _opt(f64p),
                                             _opt(f64p), _opt(f64p)]
        L.or_loss.restype = C.c_double
        L.or_loss.argtypes = [C.c_int64, f32p, f32p, f32p, C.c_int, C.c_double, _opt(f64p), _opt(f64p)]
        L.or_event_frame.argtypes = [C.c_int, C.c_int, C.c_int64, u16p, u16p, u8p, C.c_int, _opt(f64p),
                                     f32p, _opt(f32p), _opt(i32p)]
        L.or_undistort.argtypes = [f32p, C.c_int, C.c_int, f64p, f32p]
        L.or_resize_nearest.argtypes = [f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int]
        _lib = L
    return _lib


def _c(a, dt):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


def exp2f(y):
    return np.float32(lib().or_exp2f_export(float(y)))


def cov3d(scale, rot, mod=1.0):
    scale, rot = _c(scale, np.float32), _c(rot, np.float32)
    n = scale.shape[0]
    out = np.zeros((n, 6), np.float32)
    lib().or_cov3d(n, scale, rot, mod, out)
    return out


def sh_eval(sh, dirs, deg=3):
    """SH value + 0.5 (no clamp) in FP64; sh [n, 16, 3], dirs [n, 3]."""
    sh, dirs = _c(sh, np.float32), _c(dirs, np.float64)
    n = sh.shape[0]
    out = np.zeros((n, 3), np.float64)
    lib().or_sh_eval_f64(n, deg, sh.reshape(n, 48), dirs.reshape(n, 3), out)
    return out


def tiles(W, H):
    return (W + 15) // 16, (H + 15) // 16


def preprocess(xyz, cov6, sh, view, W, H, sh_deg=3, colors_pre=None):
    xyz, cov6, view = _c(xyz, np.float32), _c(cov6, np.float32), _c(view, np.float32)
    sh, colors_pre = _c(sh, np.float32), _c(colors_pre, np.float32)
    n = xyz.shape[0]
    o = dict(radii=np.zeros(n, np.int32), touched=np.zeros(n, np.int32),
             mean2d=np.zeros((n, 2), np.float32), depth=np.zeros(n, np.float32),
             conic=np.zeros((n, 3), np.float32), rgb=np.zeros((n, 3), np.float32),
             grey=np.zeros(n, np.float32), rect=np.zeros((n, 4), np.int32))
    lib().or_preprocess(n, xyz, cov6, sh, sh_deg, colors_pre, view, W, H, o["radii"], o["touched"],
                        o["mean2d"], o["depth"], o["conic"], o["rgb"], o["grey"], o["rect"])
    return o


def duplicate(pre, W, H, tile_offset=0, val_offset=0):
    K = int(pre["touched"].astype(np.int64).sum())
    keys = np.zeros(max(K, 1), np.uint64)
    vals = np.zeros(max(K, 1), np.uint32)
    n = pre["touched"].shape[0]
    k = lib().or_duplicate(n, pre["touched"], pre["mean2d"], pre["radii"], pre["depth"], W, H,
                           tile_offset, val_offset, keys, vals)
    assert k == K
    return keys[:K].copy(), vals[:K].copy()


def sort_pairs(keys, vals, bits=64):
    keys, vals = keys.copy(), vals.copy()
    if keys.shape[0]:
        lib().or_sort_pairs(keys.shape[0], keys, vals, bits)
    return keys, vals


def ranges(keys, ntiles):
    r = np.zeros((ntiles, 2), np.uint32)
    k = _c(keys, np.uint64) if keys.shape[0] else np.zeros(1, np.uint64)
    lib().or_ranges(keys.shape[0], k, ntiles, r)
    return r


def blend(W, H, rng, vals, pre, opac, colors, bg, record=False, want_extra=True):
    """FP32 front-to-back blend of one view.  colors: [n, nch]."""
    colors = _c(colors, np.float32)
    nch = colors.shape[1]
    P = W * H
    out = np.zeros((nch, H, W), np.float32)
    T = np.zeros((H, W), np.float32)
    D = np.zeros((H, W), np.float32) if want_extra else None
    A = np.zeros((H, W), np.float32) if want_extra else None
    nc = np.zeros((H, W), np.int32)
    nt = np.zeros(colors.shape[0], np.int32) if want_extra else None
    cnt = np.zeros(P, np.int32)
    vals = vals if vals.shape[0] else np.zeros(1, np.uint32)
    L = lib()
    args = (W, H, nch, _c(rng, np.uint32), _c(vals, np.uint32), pre["mean2d"], pre["conic"],
            _c(opac, np.float32), colors, pre["depth"], _c(bg, np.float32), out, T, D, A, nc, nt)
    L.or_blend_fwd(*args, cnt, None, None, None)
    res = dict(image=out, final_T=T, depth=D, alpha=A, n_contrib=nc, n_touched=nt, count=cnt)
    if record:
        start = np.zeros(P + 1, np.int64)
        start[1:] = np.cumsum(cnt)
        tot = int(start[-1])
        ids = np.zeros(max(tot, 1), np.uint32)
        clamp = np.zeros(max(tot, 1), np.uint8)
        # second pass only records contributors: do not count n_touched twice
        args2 = args[:-1] + (None,)
        L.or_blend_fwd(*args2, cnt, start, ids, clamp)
        res.update(rec_start=start, rec_ids=ids, rec_clamp=clamp)
    return res


def rasterize_view(xyz, cov6, sh, opac, view, W, H, bg, nch=3, sh_deg=3, colors_pre=None,
                   record=False):
    """Full FP32 pipeline for one view: preprocess, duplicate, sort, ranges, blend."""
    pre = preprocess(xyz, cov6, sh, view, W, H, sh_deg, colors_pre)
    keys, vals = duplicate(pre, W, H)
    tx, ty = tiles(W, H)
    ntiles = tx * ty
    tile_bits = max(1, int(ntiles - 1).bit_length())
    keys, vals = sort_pairs(keys, vals, 32 + tile_bits)
    rng = ranges(keys, ntiles)
    colors = pre["rgb"] if nch == 3 else pre["grey"][:, None]
    out = blend(W, H, rng, vals, pre, opac, colors, bg, record=record)
    out.update(pre=pre, keys=keys, vals=vals, ranges=rng)
    return out


def frozen_render(rec, xyz, opac, view64, W, H, bg, nch, sh=None, scale=None, rot=None,
                  cov_pre=None, sh_deg=3, colors_pre=None, mod=1.0):
    n = xyz.shape[0]
    out = np.zeros((nch, H, W), np.float64)
    D = np.zeros((H, W), np.float64)
    A = np.zeros((H, W), np.float64)
    bgv = np.zeros(3, np.float64)
    bgv[:len(bg)] = bg
    if cov_pre is None and (scale is None or rot is None):
        raise ValueError("frozen_render needs cov_pre or scale + rot")
    lib().or_frozen_render_f64(n, _c(xyz, np.float32), _c(scale, np.float32), _c(rot, np.float32),
                               _c(cov_pre, np.float32), mod, _c(opac, np.float32), _c(sh, np.float32),
                               sh_deg, _c(colors_pre, np.float32), _c(view64, np.float64), W, H, nch,
                               bgv, rec["rec_start"], rec["rec_ids"], rec["rec_clamp"], out, D, A)
    return out, D, A


def frozen_backward(rec, xyz, opac, view64, W, H, bg, nch, dL_dout, sh=None, scale=None,
                    rot=None, cov_pre=None, sh_deg=3, colors_pre=None, mod=1.0, dL_ddepth=None,
                    dL_dalpha=None, map_grads=False):
    n = xyz.shape[0]
    g_xi = np.zeros(6, np.float64)
    mg = None
    if map_grads:
        mg = dict(mean2d=np.zeros((n, 2)), means3d=np.zeros((n, 3)), sh=np.zeros((n, 48)),
                  opac=np.zeros(n), scale=np.zeros((n, 3)), rot=np.zeros((n, 4)),
                  cov=np.zeros((n, 6)), colors=np.zeros((n, 3)))
    g = (lambda k: mg[k]) if map_grads else (lambda k: None)
    bgv = np.zeros(3, np.float64)
    bgv[:len(bg)] = bg
    lib().or_frozen_backward_f64(n, _c(xyz, np.float32), _c(scale, np.float32), _c(rot, np.float32),
                                 _c(cov_pre, np.float32), mod, _c(opac, np.float32),
                                 _c(sh, np.float32), sh_deg, _c(colors_pre, np.float32),
                                 _c(view64, np.float64), W, H, nch, bgv, rec["rec_start"],
                                 rec["rec_ids"], rec["rec_clamp"], _c(dL_dout, np.float64),
                                 _c(dL_ddepth, np.float64), _c(dL_dalpha, np.float64), g_xi,
                                 g("mean2d"), g("means3d"), g("sh"), g("opac"), g("scale"),
                                 g("rot"), g("cov"), g("colors"))
    return g_xi, mg


def loss(I_last, I_next, E, unsigned=False, grads=False, log_eps=None):
    """Pair loss (FP64) of two grey renders against the event frame; log_eps selects the
    log-intensity change ln(I + eps) instead of the linear one."""
    I_last, I_next, E = _c(I_last, np.float32), _c(I_next, np.float32), _c(E, np.float32)
    n = I_last.size
    gn = np.zeros(n, np.float64) if grads else None
    gl = np.zeros(n, np.float64) if grads else None
    L = lib().or_loss(n, I_last.reshape(-1), I_next.reshape(-1), E.reshape(-1), int(unsigned),
                      float(log_eps) if log_eps else -1.0, gn, gl)
    return (L, gn, gl) if grads else L


def loss_f64(I_last, I_next, E, unsigned=False, log_eps=None):
    """Same loss evaluated from FP64 images (numpy), for finite differences."""
    if log_eps:
        d = np.log(np.asarray(I_next, np.float64) + log_eps) - np.log(np.asarray(I_last, np.float64) + log_eps)
    else:
        d = np.asarray(I_next, np.float64) - np.asarray(I_last, np.float64)
    n = d / np.sqrt(np.sum(d * d))
    E = np.asarray(E, np.float64)
    r = (np.abs(n) - np.abs(E)) if unsigned else (n - E)
    return float(np.sqrt(np.sum(r * r)))


def event_frame(W, H, x, y, p, ksize=9, camera=None):
    """camera: None (no undistortion) or (fx, fy, cx, cy, k1, k2, p1, p2, k3)."""
    x, y, p = _c(x, np.uint16), _c(y, np.uint16), _c(p, np.uint8)
    s = np.zeros((H, W), np.float32)
    u = np.zeros((H, W), np.float32)
    c = np.zeros((H, W), np.int32)
    n = x.shape[0]
    if n == 0:
        x = np.zeros(1, np.uint16); y = np.zeros(1, np.uint16); p = np.zeros(1, np.uint8)
    cam = None if camera is None else np.ascontiguousarray(camera, np.float64)
    lib().or_event_frame(W, H, n, x, y, p, ksize, cam, s, u, c)
    return s, u, c


def undistort(img, camera):
    img = _c(img, np.float32)
    H, W = img.shape
    out = np.zeros((H, W), np.float32)
    lib().or_undistort(img, W, H, np.ascontiguousarray(camera, np.float64), out)
    return out


def resize_nearest(img, dw, dh):
    img = _c(img, np.float32)
    sh_, sw = img.shape
    out = np.zeros((dh, dw), np.float32)
    lib().or_resize_nearest(img, sw, sh_, out, dw, dh)
    return out


def pyramid(img, levels=3):
    """utils/tracker.py:78-91: level l is the full image resized to int(size * 0.5**l)."""
    H, W = img.shape
    return [resize_nearest(img, int(W * 0.5 ** l), int(H * 0.5 ** l)) for l in range(levels)]
