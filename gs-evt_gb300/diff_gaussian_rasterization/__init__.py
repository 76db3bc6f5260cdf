"""Drop-in replacement of the `diff_gaussian_rasterization` module imported by the
reference (gaussian_splatting/gaussian_renderer/__init__.py:15-18).

Same names, same call signature and the same 5-tuple return as the reference's call
sites:
  - GaussianRasterizationSettings with the 18 fields filled at
    gaussian_renderer/__init__.py:318-337 (the velocity fields default, so the legacy
    `render()` at :58-72 still constructs it);
  - GaussianRasterizer(raster_settings=...)(means3D=, means2D=, shs=, colors_precomp=,
    opacities=, scales=, rotations=, cov3D_precomp=, theta=, rho=, w=, v=)
    -> (color [3,H,W], radii [N] int32, depth [1,H,W], opacity [1,H,W],
        n_touched [N] int32)   (:362-375);
  - exactly one of shs / colors_precomp and one of (scales, rotations) / cov3D_precomp,
    else an Exception, as the rasterizer requires;
  - gradients flow to means2D (NDC units), the map tensors that require grad, and to
    theta, rho, w, v: the left-twist gradient of the rendered view chained through
    vel_transofrm and delta_time (:266-275, :301-304).

Every stage runs in libgsevt.so (sm_103a kernels); there is no CPU path.
"""
from typing import NamedTuple

import torch
import torch.nn as nn

from gsevt import engine
from gsevt._lib import lib, check
from gsevt.engine import GSFrame, MapSpec, ViewSpec, _ptr, _stream

__all__ = ["GaussianRasterizationSettings", "GaussianRasterizer", "rasterize_gaussians"]


class GaussianRasterizationSettings(NamedTuple):
    image_height: int
    image_width: int
    tanfovx: float
    tanfovy: float
    bg: torch.Tensor
    scale_modifier: float
    viewmatrix: torch.Tensor
    projmatrix: torch.Tensor
    projmatrix_raw: torch.Tensor = None
    sh_degree: int = 3
    campos: torch.Tensor = None
    prefiltered: bool = False
    angular_vel: torch.Tensor = None
    linear_vel: torch.Tensor = None
    vel_transofrm: torch.Tensor = None
    vel_transofrm_inv: torch.Tensor = None
    delta_time: float = 0.0
    debug: bool = False


# key capacity remembered per (n, width, height) so a repeated call does not regrow
_capacity_hint = {}


def _proj_raw(s):
    if s.projmatrix_raw is not None:
        return s.projmatrix_raw
    # projmatrix = viewmatrix @ projmatrix_raw in the transposed convention
    return torch.linalg.solve(s.viewmatrix, s.projmatrix)


def _campos(s):
    if s.campos is not None:
        return s.campos
    return torch.linalg.inv(s.viewmatrix)[3, :3]


def _as_f32(t):
    return None if t is None else t.detach().contiguous().float()


class _RasterizeGaussians(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means3D, means2D, shs, colors_precomp, opacities, scales, rotations, cov3D_precomp,
                theta, rho, w, v, raster_settings):
        s = raster_settings
        n = means3D.shape[0]
        H, W = int(s.image_height), int(s.image_width)
        dev = means3D.device
        xyz = _as_f32(means3D)
        opac = _as_f32(opacities).reshape(-1)
        shs_c = None if shs is None else _as_f32(shs).reshape(n, -1, 3)
        cols = None if colors_precomp is None else _as_f32(colors_precomp)
        sc = _as_f32(scales)
        rot = _as_f32(rotations)
        cov = _as_f32(cov3D_precomp)
        if cov is not None:
            sc = rot = None
        sh_coeffs = shs_c.shape[1] if shs_c is not None else 16
        # never read past the coefficients the caller supplied
        deg = min(int(s.sh_degree), 3, int(round(sh_coeffs ** 0.5)) - 1 if shs_c is not None else 3)
        if shs_c is not None and (deg + 1) ** 2 > sh_coeffs:
            deg -= 1
        m = MapSpec(n, xyz=xyz, opacity=opac, scales=sc, rotations=rot, cov3d=cov, shs=shs_c, colors=cols,
                    sh_degree=max(deg, 0), sh_coeffs=sh_coeffs,
                    scale_modifier=float(s.scale_modifier))
        settings = {"viewmatrix": s.viewmatrix, "projmatrix_raw": _proj_raw(s), "campos": _campos(s),
                    "bg": s.bg, "tanfovx": s.tanfovx, "tanfovy": s.tanfovy}
        view = ViewSpec(W, H, 0, settings=settings)
        key = (n, W, H)
        frame = GSFrame([m], [view], channels=3, key_capacity=_capacity_hint.get(key, max(1 << 20, 4 * n)),
                        want_depth=True, want_alpha=True, want_radii=True, want_n_touched=True, device=dev)
        if n > 0:
            frame.render(exact_keys=True)
            _capacity_hint[key] = max(frame.L.key_capacity, int(frame.num_keys * 1.25) + 1024)
        else:
            frame.image.copy_(s.bg.float().reshape(3, 1).expand(3, W * H))
            frame.final_T.fill_(1.0)
            frame.depth.zero_()
            frame.alpha.zero_()
        color = frame.image.view(3, H, W).clone()
        depth = frame.depth.view(1, H, W).clone()
        opacity = frame.alpha.view(1, H, W).clone()
        radii = frame.radii[:n].clone() if n > 0 else torch.zeros(0, dtype=torch.int32, device=dev)
        n_touched = frame.n_touched[:n].clone() if n > 0 else torch.zeros(0, dtype=torch.int32, device=dev)
        ctx.frame = frame
        ctx.n = n
        ctx.settings = s
        ctx.has_sh = shs is not None
        ctx.has_cov = cov3D_precomp is not None
        ctx.sh_shape = None if shs is None else shs.shape
        ctx.opac_shape = opacities.shape
        ctx.mark_non_differentiable(radii, n_touched)
        return color, radii, depth, opacity, n_touched

    @staticmethod
    def backward(ctx, grad_color, grad_radii, grad_depth, grad_opacity, grad_ntouched):
        frame, n, s = ctx.frame, ctx.n, ctx.settings
        need = ctx.needs_input_grad
        dev = frame.image.device
        outs = [None] * 13
        if n == 0:
            return tuple(outs)
        gimg = torch.zeros_like(frame.image) if grad_color is None else grad_color.detach().float().contiguous().view(3, -1)
        gdep = None if grad_depth is None else grad_depth.detach().float().contiguous().view(-1)
        gop = None if grad_opacity is None else grad_opacity.detach().float().contiguous().view(-1)
        frame.blend_backward(gimg, gdep, gop)
        xi = torch.empty(6, dtype=torch.float64, device=dev)
        g = {}
        if need[0]:
            g["means3d"] = torch.empty((n, 3), dtype=torch.float32, device=dev)
        if need[1]:
            g["means2d"] = torch.empty((n, 3), dtype=torch.float32, device=dev)
        if need[2] and ctx.has_sh:
            g["shs"] = torch.empty((n, ctx.sh_shape[1], 3), dtype=torch.float32, device=dev)
        if need[3] and not ctx.has_sh:
            g["colors"] = torch.empty((n, 3), dtype=torch.float32, device=dev)
        if need[4]:
            g["opacity"] = torch.empty(n, dtype=torch.float32, device=dev)
        if need[5] and not ctx.has_cov:
            g["scales"] = torch.empty((n, 3), dtype=torch.float32, device=dev)
        if need[6] and not ctx.has_cov:
            g["rotations"] = torch.empty((n, 4), dtype=torch.float32, device=dev)
        if need[7] and ctx.has_cov:
            g["cov3d"] = torch.empty((n, 6), dtype=torch.float32, device=dev)
        frame.preprocess_backward(xi, [g] if g else None)
        if any(need[8:12]):
            out12 = torch.empty(12, dtype=torch.float32, device=dev)
            if s.vel_transofrm is not None:
                E_t = s.vel_transofrm.detach().contiguous().float()
            else:
                E_t = torch.eye(4, dtype=torch.float32, device=dev)
            zero3 = torch.zeros(3, dtype=torch.float32, device=dev)
            lin = zero3 if s.linear_vel is None else s.linear_vel.detach().contiguous().float()
            ang = zero3 if s.angular_vel is None else s.angular_vel.detach().contiguous().float()
            dt = float(s.delta_time) if s.vel_transofrm is not None else 0.0
            check(lib().gsevt_chain_view_grad(_ptr(xi), _ptr(E_t), dt, _ptr(lin), _ptr(ang), _ptr(out12),
                                              _stream()), "gsevt_chain_view_grad")
            for k in range(4):
                if need[8 + k]:
                    outs[8 + k] = out12[3 * k:3 * k + 3].clone()
        outs[0] = g.get("means3d")
        outs[1] = g.get("means2d")
        outs[2] = g.get("shs")
        if outs[2] is not None and ctx.sh_shape is not None:
            outs[2] = outs[2].view(ctx.sh_shape)
        outs[3] = g.get("colors")
        outs[4] = g["opacity"].view(ctx.opac_shape) if "opacity" in g else None
        outs[5] = g.get("scales")
        outs[6] = g.get("rotations")
        outs[7] = g.get("cov3d")
        ctx.frame = None
        return tuple(outs)


def rasterize_gaussians(means3D, means2D, sh, colors_precomp, opacities, scales, rotations, cov3Ds_precomp,
                        raster_settings, theta=None, rho=None, w=None, v=None):
    return _RasterizeGaussians.apply(means3D, means2D, sh, colors_precomp, opacities, scales, rotations,
                                     cov3Ds_precomp, theta, rho, w, v, raster_settings)


class GaussianRasterizer(nn.Module):
    def __init__(self, raster_settings):
        super().__init__()
        self.raster_settings = raster_settings

    def markVisible(self, positions):
        """Frustum test (camera-space depth > 0.2) as a bool mask, without gradients."""
        with torch.no_grad():
            vm = self.raster_settings.viewmatrix
            p = torch.cat([positions, torch.ones_like(positions[:, :1])], dim=1) @ vm
            return p[:, 2] > 0.2

    def forward(self, means3D, means2D, opacities, shs=None, colors_precomp=None, scales=None, rotations=None,
                cov3D_precomp=None, theta=None, rho=None, w=None, v=None):
        s = self.raster_settings
        if (shs is None and colors_precomp is None) or (shs is not None and colors_precomp is not None):
            raise Exception("Please provide excatly one of either SHs or precomputed colors!")
        if ((scales is None or rotations is None) and cov3D_precomp is None) or \
                ((scales is not None or rotations is not None) and cov3D_precomp is not None):
            raise Exception("Please provide exactly one of either scale/rotation pair or precomputed 3D covariance!")
        if not means3D.is_cuda:
            raise RuntimeError("gsevt rasterizer: tensors must be on a CUDA device (there is no CPU path)")
        return rasterize_gaussians(means3D, means2D, shs, colors_precomp, opacities, scales, rotations,
                                   cov3D_precomp, s, theta, rho, w, v)
