"""ctypes binding of libgsevt.so (the C ABI declared in include/gsevt.h).

The structs below mirror the C structs field by field; `check_abi()` compares their
sizes with the library's own sizeof values.  There is no CPU fallback: if the library
has not been built, importing the engine raises with the build command to run.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libgsevt.so")

GSEVT_OK = 0
GSEVT_ERR_ARG = -1
GSEVT_ERR_TOO_LARGE = -7
ERRORS = {
    -1: "bad argument (shape, size or pointer)",
    -2: "key capacity overflow",
    -3: "non-finite loss or gradient",
    -4: "bounded device wait ran out",
    -5: "CUDA launch or copy failed",
    -6: "workspace smaller than gsevt_workspace_bytes",
    -7: "input larger than the fixed scratch buffer or the given capacity holds",
}
STATUS_KEY_OVERFLOW = 1
STATUS_SORT_TIMEOUT = 2
STATUS_NONFINITE = 4
STATUS_LAYOUT = 8
STATUS_STAGE_TIMEOUT = 16
_STATUS_NAMES = ((STATUS_KEY_OVERFLOW, "key capacity overflow"), (STATUS_SORT_TIMEOUT, "bounded device wait ran out"),
                 (STATUS_NONFINITE, "non-finite loss or gradient"),
                 (STATUS_LAYOUT, "layout provides too few super-tiles"),
                 (STATUS_STAGE_TIMEOUT, "blend staging wait ran out"))


def status_names(flags):
    """The conditions set in a device status word (gsevt_read_status word 0), as text."""
    names = [n for bit, n in _STATUS_NAMES if flags & bit]
    rest = flags & ~sum(bit for bit, _ in _STATUS_NAMES)
    if rest:
        names.append("unknown flags %#x" % rest)
    return ", ".join(names) if names else "none"
TILE = 16
MAP_PLANES = 15
LOSS_PIXELS_PER_BLOCK = 2048
SCAN_BLOCK = 256


class GsevtError(RuntimeError):
    pass


class View(C.Structure):
    _fields_ = [("R", C.c_float * 9), ("t", C.c_float * 3), ("P", C.c_float * 16),
                ("campos", C.c_float * 3), ("tanfovx", C.c_float), ("tanfovy", C.c_float),
                ("bg", C.c_float * 3), ("width", C.c_int32), ("height", C.c_int32),
                ("tiles_x", C.c_int32), ("tiles_y", C.c_int32), ("tile_offset", C.c_int32),
                ("pix_offset", C.c_int32), ("map", C.c_int32), ("vg_offset", C.c_int32),
                ("sb_offset", C.c_int32), ("pair", C.c_int32), ("pair_role", C.c_int32),
                ("skip", C.c_int32)]


class Map(C.Structure):
    _fields_ = [("xyz", C.c_void_p), ("opacity", C.c_void_p), ("scales", C.c_void_p),
                ("rotations", C.c_void_p), ("cov3d", C.c_void_p), ("shs", C.c_void_p),
                ("colors", C.c_void_p), ("packed", C.c_void_p), ("n", C.c_int32),
                ("sh_degree", C.c_int32), ("sh_coeffs", C.c_int32), ("scale_modifier", C.c_float),
                ("first_view", C.c_int32), ("num_views", C.c_int32), ("block_offset", C.c_int32),
                ("pad", C.c_int32)]


class MapGrads(C.Structure):
    _fields_ = [("means3d", C.c_void_p), ("means2d", C.c_void_p), ("opacity", C.c_void_p),
                ("scales", C.c_void_p), ("rotations", C.c_void_p), ("cov3d", C.c_void_p),
                ("shs", C.c_void_p), ("colors", C.c_void_p)]


class Pair(C.Structure):
    _fields_ = [("last_view", C.c_int32), ("next_view", C.c_int32), ("event", C.c_void_p),
                ("event_abs", C.c_void_p), ("unsigned_mode", C.c_int32), ("pose", C.c_int32),
                ("block_offset", C.c_int32), ("num_blocks", C.c_int32), ("log_grey", C.c_int32),
                ("log_eps", C.c_float)]


class Tuning(C.Structure):
    _fields_ = [("blend_staging", C.c_int32), ("depth_sort_kpt", C.c_int32), ("pair_sort_kpt", C.c_int32),
                ("coop_sort", C.c_int32), ("blend_schedule", C.c_int32), ("adjoint_pixels", C.c_int32),
                ("forward_pixels", C.c_int32), ("reserved", C.c_int32 * 1)]


class Layout(C.Structure):
    _fields_ = [("num_views", C.c_int32), ("num_maps", C.c_int32), ("num_pairs", C.c_int32),
                ("num_vg", C.c_int32), ("num_scan_blocks", C.c_int32),
                ("preprocess_blocks", C.c_int32), ("total_tiles", C.c_int32),
                ("total_pixels", C.c_int32), ("channels", C.c_int32), ("sort_bits", C.c_int32),
                ("key_capacity", C.c_uint32), ("loss_blocks", C.c_int32), ("super_tiles", C.c_int32),
                ("spin_limit", C.c_uint32), ("tuning", Tuning)]


class Frame(C.Structure):
    _fields_ = [("L", Layout), ("views", C.c_void_p), ("maps", C.c_void_p), ("pairs", C.c_void_p),
                ("workspace", C.c_void_p), ("workspace_bytes", C.c_size_t), ("image", C.c_void_p),
                ("final_T", C.c_void_p), ("depth", C.c_void_p), ("alpha", C.c_void_p),
                ("n_contrib", C.c_void_p), ("radii", C.c_void_p), ("n_touched", C.c_void_p)]


class PoseState(C.Structure):
    _fields_ = [("R", C.c_double * 9), ("t", C.c_double * 3), ("lin_vel", C.c_double * 3),
                ("ang_vel", C.c_double * 3), ("delta_tau", C.c_double), ("m", C.c_double * 12),
                ("v", C.c_double * 12), ("lr", C.c_double * 4), ("lr_scale", C.c_double * 4),
                ("step", C.c_int32 * 4), ("opt_vel", C.c_int32), ("last_view", C.c_int32),
                ("next_view", C.c_int32), ("iter", C.c_int32), ("pad", C.c_int32),
                ("fx", C.c_float), ("fy", C.c_float), ("loss", C.c_double),
                ("grad", C.c_double * 12), ("control", C.c_int32), ("frozen", C.c_int32),
                ("level_iter", C.c_int32), ("start_vel", C.c_int32), ("hist_n", C.c_int32),
                ("max_iter", C.c_int32), ("conv_thr", C.c_double), ("hist", C.c_double * 11)]


_lib = None


def lib():
    """Load libgsevt.so once; raise loudly if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GsevtError(
            "libgsevt.so is not built (%s); run `python -c \"import __graft_entry__ as g; g.build()\"` "
            "or `python gs-evt_gb300/csrc/build.py`" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, i32, u32, f32, i64 = C.c_void_p, C.c_int32, C.c_uint32, C.c_float, C.c_int64
    fp = C.POINTER(Frame)
    sig = {
        "gsevt_workspace_bytes": (C.c_size_t, [C.POINTER(Layout)]),
        "gsevt_workspace_init": (C.c_int, [fp, vp]),
        "gsevt_abi_sizes": (None, [C.POINTER(i32)]),
        "gsevt_workspace_offsets": (None, [C.POINTER(Layout), C.POINTER(C.c_uint64)]),
        "gsevt_pack_map": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, i32, f32, vp, vp]),
        "gsevt_preprocess_fwd": (C.c_int, [fp, vp]),
        "gsevt_bin_and_sort": (C.c_int, [fp, u32, vp]),
        "gsevt_blend_fwd": (C.c_int, [fp, vp]),
        "gsevt_loss_fwd": (C.c_int, [fp, vp, vp]),
        "gsevt_blend_bwd": (C.c_int, [fp, vp, vp, vp, vp]),
        "gsevt_preprocess_bwd": (C.c_int, [fp, vp, C.POINTER(MapGrads), vp]),
        "gsevt_chain_view_grad": (C.c_int, [vp, vp, f32, vp, vp, vp, vp]),
        "gsevt_view_from_settings": (C.c_int, [vp, vp, vp, vp, f32, f32, i32, i32, i32, i32, i32, i32,
                                                i32, vp, vp]),
        "gsevt_read_status": (C.c_int, [fp, C.POINTER(u32), vp]),
        "gsevt_clear_status": (C.c_int, [fp, vp]),
        "gsevt_event_scratch_bytes": (C.c_size_t, [i32, i32]),
        "gsevt_events_accumulate": (C.c_int, [i64, vp, vp, vp, i32, i32, C.POINTER(C.c_double), i32, i32, vp,
                                              vp, vp, vp]),
        "gsevt_track_step_batched": (C.c_int, [fp, vp, i32, vp, vp]),
        "gsevt_track_init_views": (C.c_int, [vp, vp, i32, vp]),
        "gsevt_parse_events_txt": (C.c_int, [C.c_char_p, C.c_size_t, vp, vp, vp, vp, C.c_size_t,
                                             C.POINTER(C.c_size_t), i32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return _lib


EXPORTED = [
    "gsevt_workspace_bytes", "gsevt_workspace_init", "gsevt_abi_sizes", "gsevt_workspace_offsets",
    "gsevt_pack_map",
    "gsevt_preprocess_fwd", "gsevt_bin_and_sort", "gsevt_blend_fwd", "gsevt_loss_fwd",
    "gsevt_blend_bwd", "gsevt_preprocess_bwd", "gsevt_chain_view_grad", "gsevt_view_from_settings",
    "gsevt_read_status", "gsevt_clear_status", "gsevt_event_scratch_bytes",
    "gsevt_events_accumulate", "gsevt_events_accumulate_noalloc", "gsevt_track_step_batched",
    "gsevt_track_init_views", "gsevt_parse_events_txt",
]


WORKSPACE_REGIONS = ["status", "bin", "recA", "recB", "recC", "gradA", "gradB", "gradC", "vis_sums",
                     "vis_offs", "dkeys0", "dkeys1", "dvals0", "dvals1", "tsums", "toffs", "keys0", "keys1",
                     "vals0", "vals1", "sort_hist", "sort_counter", "sort_lookback", "ranges", "loss_part",
                     "loss_scal", "loss_done", "xi_part", "xi", "csums", "coffs", "soffs", "sranges",
                     "fcache"]


def workspace_offsets(layout):
    out = (C.c_uint64 * len(WORKSPACE_REGIONS))()
    lib().gsevt_workspace_offsets(C.byref(layout), out)
    return {k: (None if o == 0xFFFFFFFFFFFFFFFF else int(o)) for k, o in zip(WORKSPACE_REGIONS, out)}


def check(status, what=""):
    if status != GSEVT_OK:
        raise GsevtError("%s failed: %s (%d)" % (what, ERRORS.get(status, "unknown error"), status))


def check_abi():
    out = (C.c_int32 * 7)()
    lib().gsevt_abi_sizes(out)
    mine = [C.sizeof(View), C.sizeof(Map), C.sizeof(MapGrads), C.sizeof(Pair), C.sizeof(Layout),
            C.sizeof(Frame), C.sizeof(PoseState)]
    if list(out) != mine:
        raise GsevtError("ABI struct sizes differ: library %s, binding %s" % (list(out), mine))
    return mine
