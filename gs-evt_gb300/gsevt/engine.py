"""Rendering frame engine over the C ABI (include/gsevt.h).

A `GSFrame` holds one launch's worth of work: the device map table (one or more
Gaussian maps), the device view table (every rendered view, of any size), optional
render pairs with their event frames, the caller-owned outputs and the workspace.  Its
methods enqueue the library's stages on the current torch CUDA stream; none of them
synchronises except `status()`.

Device tensors come from PyTorch (allocator and streams only); every compute step is a
kernel of libgsevt.so.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _lib
from ._lib import check, lib

SORT_DEPTH_BITS = 32


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _struct_tensor(structs, device):
    """Copy an array of ctypes structs to a device uint8 tensor."""
    raw = b"".join(bytes(s) for s in structs)
    return torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(device)


class MapSpec:
    """One Gaussian map.  Either raw drop-in tensors (xyz, opacity, scales+rotations or
    cov3d, shs or colors) or `packed` planes from `pack_map`."""

    def __init__(self, n, xyz=None, opacity=None, scales=None, rotations=None, cov3d=None, shs=None,
                 colors=None, packed=None, sh_degree=3, sh_coeffs=16, scale_modifier=1.0):
        self.n = int(n)
        self.xyz, self.opacity, self.scales, self.rotations = xyz, opacity, scales, rotations
        self.cov3d, self.shs, self.colors, self.packed = cov3d, shs, colors, packed
        self.sh_degree, self.sh_coeffs, self.scale_modifier = int(sh_degree), int(sh_coeffs), float(scale_modifier)
        if not 0 <= self.sh_degree <= 3 or (shs is not None and (self.sh_degree + 1) ** 2 > self.sh_coeffs):
            raise ValueError("sh_degree %d needs %d coefficients per channel, got %d"
                             % (self.sh_degree, (self.sh_degree + 1) ** 2, self.sh_coeffs))


class ViewSpec:
    """One rendered view: image size, background and map index.  The pose fields are
    filled on the host (R, t, P, campos, tanfov) or on the device from the drop-in
    settings tensors (`settings=`)."""

    def __init__(self, width, height, map_index=0, bg=(0.0, 0.0, 0.0), R=None, t=None, P=None, campos=None,
                 tanfovx=None, tanfovy=None, pair=-1, pair_role=0, settings=None):
        self.width, self.height, self.map_index = int(width), int(height), int(map_index)
        self.bg = bg
        self.R, self.t, self.P, self.campos = R, t, P, campos
        self.tanfovx, self.tanfovy = tanfovx, tanfovy
        self.pair, self.pair_role = int(pair), int(pair_role)
        self.settings = settings


def pack_map(xyz, opacity, shs, scales=None, rotations=None, cov3d=None, scale_modifier=1.0):
    """Pack a map once into 15 float4 planes (position+opacity, cov3D, 48 SH floats)."""
    n = xyz.shape[0]
    dev = xyz.device
    packed = torch.empty((_lib.MAP_PLANES, max(n, 1), 4), dtype=torch.float32, device=dev)
    xyz = xyz.contiguous().float()
    opacity = opacity.reshape(-1).contiguous().float()
    shs = shs.reshape(n, -1, 3).contiguous().float()
    scales = None if scales is None else scales.contiguous().float()
    rotations = None if rotations is None else rotations.contiguous().float()
    cov3d = None if cov3d is None else cov3d.contiguous().float()
    check(lib().gsevt_pack_map(n, _ptr(xyz), _ptr(opacity), _ptr(scales), _ptr(rotations), _ptr(cov3d),
                               _ptr(shs), shs.shape[1], float(scale_modifier), _ptr(packed), _stream()),
          "gsevt_pack_map")
    return packed


class GSFrame:
    def __init__(self, maps, views, channels, pairs=None, key_capacity=None, want_depth=False,
                 want_alpha=False, want_radii=False, want_n_touched=False, want_n_contrib=False,
                 device=None):
        self.device = device or torch.device("cuda")
        self.maps, self.views, self.pairs = maps, views, pairs or []
        self.channels = int(channels)
        # views of a map must be contiguous in the table
        order = sorted(range(len(views)), key=lambda i: views[i].map_index)
        assert order == list(range(len(views))), "views must be grouped by map"
        L = _lib.Layout()
        L.num_views, L.num_maps, L.num_pairs = len(views), len(maps), len(self.pairs)
        self.vg_offset, self.sb_offset, self.tile_offset, self.pix_offset = [], [], [], []
        vg = sb = tiles = pix = supers = 0
        for v in views:
            n = maps[v.map_index].n
            tx, ty = (v.width + 15) // 16, (v.height + 15) // 16
            supers += ((tx + 3) // 4) * ((ty + 3) // 4)
            self.vg_offset.append(vg); self.sb_offset.append(sb)
            self.tile_offset.append(tiles); self.pix_offset.append(pix)
            vg += n
            sb += (n + 255) // 256
            tiles += tx * ty
            pix += v.width * v.height
        L.num_vg, L.num_scan_blocks, L.total_tiles, L.total_pixels = vg, sb, tiles, pix
        L.super_tiles = supers
        self.block_offset = []
        pb = 0
        for m in maps:
            self.block_offset.append(pb)
            pb += (m.n + 255) // 256
        L.preprocess_blocks = pb
        L.channels = self.channels
        L.sort_bits = SORT_DEPTH_BITS + max(1, int(tiles - 1).bit_length())
        if key_capacity is None:
            key_capacity = max(1 << 20, 4 * vg)
        L.key_capacity = int(min(key_capacity, (1 << 30) - 1))
        lb = 0
        self.loss_block_offset = []
        for p in self.pairs:
            v = views[p["last"]]
            nb = (v.width * v.height + _lib.LOSS_PIXELS_PER_BLOCK - 1) // _lib.LOSS_PIXELS_PER_BLOCK
            self.loss_block_offset.append((lb, nb))
            lb += nb
        L.loss_blocks = lb
        self.L = L

        # map table
        mstructs = []
        first_view = {}
        count = {}
        for i, v in enumerate(views):
            first_view.setdefault(v.map_index, i)
            count[v.map_index] = count.get(v.map_index, 0) + 1
        for mi, m in enumerate(maps):
            s = _lib.Map()
            for name in ("xyz", "opacity", "scales", "rotations", "cov3d", "shs", "colors", "packed"):
                t = getattr(m, name)
                setattr(s, name, None if t is None else t.data_ptr())
            s.n, s.sh_degree, s.sh_coeffs, s.scale_modifier = m.n, m.sh_degree, m.sh_coeffs, m.scale_modifier
            s.first_view, s.num_views = first_view.get(mi, 0), count.get(mi, 0)
            s.block_offset = self.block_offset[mi]
            mstructs.append(s)
        self.map_table = _struct_tensor(mstructs, self.device)

        # view table
        vstructs = []
        self._settings_views = []
        for i, v in enumerate(views):
            s = _lib.View()
            if v.settings is None and v.R is not None:
                for k in range(9):
                    s.R[k] = float(v.R[k // 3][k % 3])
                for k in range(3):
                    s.t[k] = float(v.t[k]); s.campos[k] = float(v.campos[k])
                for k in range(16):
                    s.P[k] = float(v.P[k // 4][k % 4])
                s.tanfovx, s.tanfovy = float(v.tanfovx), float(v.tanfovy)
            for k in range(3):
                s.bg[k] = float(v.bg[k]) if not torch.is_tensor(v.bg) else 0.0
            s.width, s.height = v.width, v.height
            s.tiles_x, s.tiles_y = (v.width + 15) // 16, (v.height + 15) // 16
            s.tile_offset, s.pix_offset = self.tile_offset[i], self.pix_offset[i]
            s.map, s.vg_offset, s.sb_offset = v.map_index, self.vg_offset[i], self.sb_offset[i]
            s.pair, s.pair_role = v.pair, v.pair_role
            vstructs.append(s)
            if v.settings is not None:
                self._settings_views.append(i)
        self.view_table = _struct_tensor(vstructs, self.device)
        for i in self._settings_views:
            self._fill_from_settings(i)

        # pairs
        if self.pairs:
            pstructs = []
            for (lb_, nb), p in zip(self.loss_block_offset, self.pairs):
                s = _lib.Pair()
                s.last_view, s.next_view = p["last"], p["next"]
                s.event = p["event"].data_ptr()
                ea = p.get("event_abs")
                s.event_abs = None if ea is None else ea.data_ptr()
                s.unsigned_mode = int(p.get("unsigned", False))
                s.pose = int(p.get("pose", 0))
                s.block_offset, s.num_blocks = lb_, nb
                eps = p.get("log_eps")
                if eps is not None:
                    if not eps > 0:
                        raise ValueError("log_eps must be positive, got %r" % (eps,))
                    s.log_grey, s.log_eps = 1, float(eps)
                pstructs.append(s)
            self.pair_table = _struct_tensor(pstructs, self.device)
        else:
            self.pair_table = None

        # outputs
        dev = self.device
        self.image = torch.empty((self.channels, pix), dtype=torch.float32, device=dev)
        self.final_T = torch.empty(pix, dtype=torch.float32, device=dev)
        self.depth = torch.empty(pix, dtype=torch.float32, device=dev) if want_depth else None
        self.alpha = torch.empty(pix, dtype=torch.float32, device=dev) if want_alpha else None
        self.n_contrib = torch.empty(pix, dtype=torch.int32, device=dev) if want_n_contrib else None
        self.radii = torch.empty(max(vg, 1), dtype=torch.int32, device=dev) if want_radii else None
        self.n_touched = torch.empty(max(vg, 1), dtype=torch.int32, device=dev) if want_n_touched else None
        self._alloc_workspace()

    # ------------------------------------------------------------------ setup --
    def _fill_from_settings(self, i):
        v = self.views[i]
        st = v.settings
        vm = st["viewmatrix"].contiguous().float()
        pr = st["projmatrix_raw"].contiguous().float()
        cp = st["campos"].contiguous().float()
        bg = st["bg"].contiguous().float()
        st["_keep"] = (vm, pr, cp, bg)
        dst = self.view_table[i * C.sizeof(_lib.View):].data_ptr()
        check(lib().gsevt_view_from_settings(_ptr(vm), _ptr(pr), _ptr(cp), _ptr(bg), float(st["tanfovx"]),
                                             float(st["tanfovy"]), v.width, v.height, self.tile_offset[i],
                                             self.pix_offset[i], v.map_index, self.vg_offset[i],
                                             self.sb_offset[i], C.c_void_p(dst), _stream()),
              "gsevt_view_from_settings")

    def _alloc_workspace(self):
        nbytes = int(lib().gsevt_workspace_bytes(C.byref(self.L)))
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self._frame = self._make_frame()
        check(lib().gsevt_workspace_init(C.byref(self._frame), _stream()), "gsevt_workspace_init")

    def _make_frame(self):
        f = _lib.Frame()
        f.L = self.L
        f.views = self.view_table.data_ptr()
        f.maps = self.map_table.data_ptr()
        f.pairs = None if self.pair_table is None else self.pair_table.data_ptr()
        f.workspace = self.workspace.data_ptr()
        f.workspace_bytes = self.workspace.numel()
        f.image = self.image.data_ptr()
        f.final_T = self.final_T.data_ptr()
        for name in ("depth", "alpha", "n_contrib", "radii", "n_touched"):
            t = getattr(self, name)
            setattr(f, name, None if t is None else t.data_ptr())
        return f

    def set_view_pose(self, i, R, t):
        """Move host-filled view i to the world -> camera pose (R, t) (enqueued copy)."""
        v = self.views[i]
        v.R, v.t = R, t
        v.campos = (-(np.asarray(R, np.float64).T @ np.asarray(t, np.float64))).tolist()
        s = _lib.View.from_buffer_copy(bytes(self.view_table[i * C.sizeof(_lib.View):(i + 1) * C.sizeof(_lib.View)]
                                             .cpu().numpy()))
        for k in range(9):
            s.R[k] = float(R[k // 3][k % 3])
        for k in range(3):
            s.t[k] = float(t[k])
            s.campos[k] = float(v.campos[k])
        raw = torch.frombuffer(bytearray(bytes(s)), dtype=torch.uint8)
        self.view_table[i * C.sizeof(_lib.View):(i + 1) * C.sizeof(_lib.View)].copy_(raw)

    def set_tuning(self, **choices):
        """Launch choices (gsevt_tuning fields: blend_staging, depth_sort_kpt, pair_sort_kpt,
        coop_sort, blend_schedule, adjoint_pixels, forward_pixels); unnamed fields keep their
        values.  A CUDA
        graph captured before keeps the launches it recorded."""
        for k, v in choices.items():
            setattr(self.L.tuning, k, int(v))
            setattr(self._frame.L.tuning, k, int(v))

    def tuning(self):
        t = self.L.tuning
        return {k: int(getattr(t, k)) for k in ("blend_staging", "depth_sort_kpt", "pair_sort_kpt", "coop_sort",
                                                "blend_schedule", "adjoint_pixels", "forward_pixels")}

    def set_spin_limit(self, limit):
        """Polls a bounded device wait makes before it gives up (0: the library default)."""
        self.L.spin_limit = int(limit)
        self._frame.L.spin_limit = int(limit)

    def grow(self, key_capacity):
        """Reallocate the workspace for a larger key capacity (contents are lost)."""
        self.L.key_capacity = int(min(key_capacity, (1 << 30) - 1))
        self._alloc_workspace()

    # ----------------------------------------------------------------- stages --
    @property
    def fref(self):
        return C.byref(self._frame)

    def preprocess(self):
        check(lib().gsevt_preprocess_fwd(self.fref, _stream()), "gsevt_preprocess_fwd")

    def status(self):
        out = (C.c_uint32 * 2)()
        check(lib().gsevt_read_status(self.fref, out, _stream()), "gsevt_read_status")
        return int(out[0]), int(out[1])

    def bin_and_sort(self, max_keys=0):
        check(lib().gsevt_bin_and_sort(self.fref, int(max_keys), _stream()), "gsevt_bin_and_sort")

    def blend(self):
        check(lib().gsevt_blend_fwd(self.fref, _stream()), "gsevt_blend_fwd")

    def loss(self, out=None):
        check(lib().gsevt_loss_fwd(self.fref, _ptr(out), _stream()), "gsevt_loss_fwd")

    def blend_backward(self, dL_dimage=None, dL_ddepth=None, dL_dalpha=None):
        check(lib().gsevt_blend_bwd(self.fref, _ptr(dL_dimage), _ptr(dL_ddepth), _ptr(dL_dalpha), _stream()),
              "gsevt_blend_bwd")

    def preprocess_backward(self, xi_out=None, map_grads=None):
        """map_grads: list (per map) of dicts name -> tensor (or None)."""
        gptr = None
        if map_grads is not None:
            arr = (_lib.MapGrads * len(self.maps))()
            for mi, g in enumerate(map_grads):
                for name in ("means3d", "means2d", "opacity", "scales", "rotations", "cov3d", "shs", "colors"):
                    t = None if g is None else g.get(name)
                    setattr(arr[mi], name, None if t is None else t.data_ptr())
            gptr = arr
        check(lib().gsevt_preprocess_bwd(self.fref, _ptr(xi_out), gptr, _stream()), "gsevt_preprocess_bwd")

    def render(self, exact_keys=True):
        """preprocess -> (host read of the key count) -> bin/sort -> blend.  With
        exact_keys the key count is read back (one sync, as the reference's rasterizer
        does) and the workspace grows if needed; otherwise the sort grid is sized from
        the capacity and overflow is reported through status()."""
        self.preprocess()
        max_keys = 0
        if exact_keys:
            st, k = self.status()
            if k > self.L.key_capacity:
                self.grow(int(k * 1.25) + 1024)
                self.preprocess()
                st, k = self.status()
            if st & _lib.STATUS_SORT_TIMEOUT:
                raise _lib.GsevtError("depth sort: %s" % _lib.status_names(st & _lib.STATUS_SORT_TIMEOUT))
            max_keys = max(k, 1)  # 0 would mean "size the sort grid from the capacity"
            self.num_keys = k
        self.bin_and_sort(max_keys)
        self.blend()

    def pixels(self, i):
        """Slice of the per-pixel buffers belonging to view i, as [C, H, W]."""
        v = self.views[i]
        o = self.pix_offset[i]
        return self.image[:, o:o + v.width * v.height].view(self.channels, v.height, v.width)

    def view_slice(self, t, i):
        v = self.views[i]
        o = self.pix_offset[i]
        return t[o:o + v.width * v.height].view(v.height, v.width)
