"""render1 / render2 / build_rasterizer / run_rasterizer with the signatures of the
reference's gaussian_splatting/gaussian_renderer/__init__.py:155-383, over the drop-in
`diff_gaussian_rasterization` (libgsevt.so).  `GaussianMap` is the part of the
reference's GaussianModel (gaussian_splatting/scene/gaussian_model.py:33-100) the
renderer reads: the activated getters over a fixed, pre-loaded map.
"""
import math

import numpy as np
import torch

from diff_gaussian_rasterization import GaussianRasterizationSettings, GaussianRasterizer


class GaussianMap:
    """Activated Gaussian map: get_xyz [N,3], get_features [N,16,3], get_opacity [N,1],
    get_scaling [N,3], get_rotation [N,4] (normalised w,x,y,z), active_sh_degree.
    The getters return stored tensors; the reference recomputes the activations and
    concatenates the SH every call (gaussian_model.py:75-95)."""

    def __init__(self, xyz, features, opacity, scaling, rotation, sh_degree=3, device="cuda"):
        t = lambda a: torch.as_tensor(np.asarray(a) if not torch.is_tensor(a) else a,
                                      dtype=torch.float32).to(device).contiguous()
        self._xyz, self._features = t(xyz), t(features)
        self._opacity = t(opacity).reshape(-1, 1)
        self._scaling = t(scaling)
        rot = t(rotation)
        self._rotation = rot / rot.norm(dim=1, keepdim=True)
        self.active_sh_degree = sh_degree
        self.max_sh_degree = sh_degree

    @classmethod
    def from_synthetic(cls, m, device="cuda"):
        return cls(m["xyz"], m["sh"], m["opacity"], m["scale"], m["rot"], 3, device)

    @property
    def get_xyz(self):
        return self._xyz

    @property
    def get_features(self):
        return self._features

    @property
    def get_opacity(self):
        return self._opacity

    @property
    def get_scaling(self):
        return self._scaling

    @property
    def get_rotation(self):
        return self._rotation


def build_rasterizer(viewpoint_camera, vel_transofrm, vel_transofrm_inv, delta_time, pc, bg_color,
                     scaling_modifier):
    settings = GaussianRasterizationSettings(
        image_height=int(viewpoint_camera.image_height), image_width=int(viewpoint_camera.image_width),
        tanfovx=math.tan(viewpoint_camera.FoVx * 0.5), tanfovy=math.tan(viewpoint_camera.FoVy * 0.5),
        bg=bg_color, scale_modifier=scaling_modifier, viewmatrix=viewpoint_camera.world_view_transform,
        projmatrix=viewpoint_camera.full_proj_transform, projmatrix_raw=viewpoint_camera.projection_matrix,
        sh_degree=pc.active_sh_degree, campos=viewpoint_camera.camera_center, prefiltered=False,
        angular_vel=viewpoint_camera.angular_vel, linear_vel=viewpoint_camera.linear_vel,
        vel_transofrm=vel_transofrm, vel_transofrm_inv=vel_transofrm_inv, delta_time=delta_time, debug=False)
    return GaussianRasterizer(raster_settings=settings)


def run_rasterizer(rasterizer, mask, means3D, means2D, shs, colors_precomp, opacity, scales, rotations,
                   cov3D_precomp, theta, rho, w, v):
    if mask is not None:
        means3D, means2D, opacity = means3D[mask], means2D[mask], opacity[mask]
        shs = None if shs is None else shs[mask]
        colors_precomp = None if colors_precomp is None else colors_precomp[mask]
        scales = None if scales is None else scales[mask]
        rotations = None if rotations is None else rotations[mask]
        cov3D_precomp = None if cov3D_precomp is None else cov3D_precomp[mask]
    image, radii, depth, opac, n_touched = rasterizer(
        means3D=means3D, means2D=means2D, shs=shs, colors_precomp=colors_precomp, opacities=opacity,
        scales=scales, rotations=rotations, cov3D_precomp=cov3D_precomp, theta=theta, rho=rho, w=w, v=v)
    return {"render": image, "radii": radii, "depth": depth, "opacity": opac, "n_touched": n_touched}


def _screenspace(pc):
    p = torch.zeros_like(pc.get_xyz, requires_grad=True) + 0
    try:
        p.retain_grad()
    except Exception:
        pass
    return p


def render1(curr_viewpoint_camera, pc, bg_color, scaling_modifier=1.0, override_color=None, mask=None):
    if pc.get_xyz.shape[0] == 0:
        return None
    means2D = _screenspace(pc)
    eye = torch.eye(4, device=pc.get_xyz.device)
    rast = build_rasterizer(curr_viewpoint_camera, eye, eye, 0, pc, bg_color, scaling_modifier)
    c = curr_viewpoint_camera
    return run_rasterizer(rast, mask, pc.get_xyz, means2D, pc.get_features if override_color is None else None,
                          override_color, pc.get_opacity, pc.get_scaling, pc.get_rotation, None,
                          c.cam_rot_delta, c.cam_trans_delta, c.cam_w_delta, c.cam_v_delta)


def render2(last_viewpoint_camera, curr_viewpoint_camera, next_viewpoint_camera, pc, bg_color,
            scaling_modifier=1.0, override_color=None, mask=None):
    if pc.get_xyz.shape[0] == 0:
        return None
    means2D = _screenspace(pc)
    c = curr_viewpoint_camera
    last = build_rasterizer(last_viewpoint_camera, c.last_vel_transform.t(), c.last_vel_transform_inv.t(),
                            -c.delta_tau / 2, pc, bg_color, scaling_modifier)
    nxt = build_rasterizer(next_viewpoint_camera, c.next_vel_transform.t(), c.next_vel_transform_inv.t(),
                           c.delta_tau / 2, pc, bg_color, scaling_modifier)
    shs = pc.get_features if override_color is None else None
    args = (pc.get_xyz, means2D, shs, override_color, pc.get_opacity, pc.get_scaling, pc.get_rotation, None,
            c.cam_rot_delta, c.cam_trans_delta, c.cam_w_delta, c.cam_v_delta)
    return run_rasterizer(last, mask, *args), run_rasterizer(nxt, mask, *args)
