"""Generate tests/golden/reference_golden.npz from the reference's own Python code.

Run in a container that has the reference checkout (default /root/reference; override
with GSEVT_REFERENCE).  The GPU test machine never runs this script; it only reads the
committed .npz.  Modules the reference imports but this environment lacks (munch,
cv2, plyfile, open3d, yaml, rosbag, PIL, natsort and the rasterizer itself) are
replaced by inert stubs: none of the functions exercised here calls into them.
The reference hard-codes device="cuda" in a few tensor constructors
(gaussian_splatting/utils/general_utils.py:101,120,140) and as the Camera default
(utils/render_camera/camera.py:24); those run here on the CPU.

Pinned (reference file:line -> fixture keys):
  utils/pose.py:26-91            so3_* / v_* / se3_* / log_*
  utils/render_camera/camera.py  cam_* (matrices :68-91, velocity transforms :100-123,
                                 update_pose :133-147, update_velocity :149-155,
                                 const_vel_model :183-201, cal_weighted_velocity :157-181)
  utils/render_camera/frame.py   pair_* (pair poses and scaled cameras :61-82),
                                 dIr_* (grey + normalisation :86-94, grey :39-43)
  utils/tracker.py               loss_* (:93-103), conv_* (:65-76)
  gaussian_splatting/utils/sh_utils.py:55-118   sh_*
  gaussian_splatting/scene/gaussian_model.py:67-73 + general_utils.py:113-148  cov_*
"""
import os
import sys
import types

import numpy as np
import torch

REF = os.environ.get("GSEVT_REFERENCE", "/root/reference")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.npz")


def _stub(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    sys.modules[name] = m
    return m


def install_stubs():
    class Munch(dict):
        __getattr__ = dict.__getitem__

    _stub("munch", munchify=lambda d: Munch(d) if isinstance(d, dict) else d)
    _stub("cv2")
    _stub("plyfile", PlyData=object, PlyElement=object)
    _stub("open3d")
    _stub("yaml")
    _stub("rosbag")
    pil = _stub("PIL")
    pil.Image = _stub("PIL.Image")
    _stub("natsort", natsorted=sorted)
    _stub("diff_gaussian_rasterization", GaussianRasterizationSettings=object, GaussianRasterizer=object)
    sys.path.insert(0, REF)
    sys.path.insert(0, os.path.join(REF, "gaussian_splatting"))


class no_cuda_device:
    """Drop device='cuda' from torch.zeros while the reference's helpers run on CPU."""

    def __enter__(self):
        self.zeros = torch.zeros

        def zeros(*a, **k):
            if k.get("device") == "cuda":
                k.pop("device")
            return self.zeros(*a, **k)

        torch.zeros = zeros

    def __exit__(self, *exc):
        torch.zeros = self.zeros


def main():
    install_stubs()
    from utils import pose as rpose
    from utils.render_camera import camera as rcam
    from utils.render_camera import frame as rframe
    from utils import tracker as rtracker
    from gaussian_splatting.utils import sh_utils
    from gaussian_splatting.utils import general_utils

    # Camera defaults to device="cuda" (camera.py:24) and frame.py:75-82 relies on it
    cam_init = rcam.Camera.__init__

    def cpu_init(self, *a, **k):
        k["device"] = "cpu"
        cam_init(self, *a, **k)

    rcam.Camera.__init__ = cpu_init
    g = {}
    rng = np.random.default_rng(1234)
    d64 = torch.float64

    # --- SO(3)/SE(3) -------------------------------------------------------------
    thetas = [rng.normal(size=3) * s for s in (1e-7, 3e-6, 1e-3, 0.1, 0.5, 1.5, 3.0)]
    g["so3_theta"] = np.array(thetas)
    g["so3_exp"] = np.array([rpose.SO3_exp(torch.tensor(t, dtype=d64)).numpy() for t in thetas])
    g["v_mat"] = np.array([rpose.V(torch.tensor(t, dtype=d64)).numpy() for t in thetas])
    xis = [np.concatenate([rng.normal(size=3), t]) for t in thetas]
    g["se3_xi"] = np.array(xis)
    g["se3_exp"] = np.array([rpose.SE3_exp(torch.tensor(x, dtype=d64)).numpy() for x in xis])
    rots = [rpose.SO3_exp(torch.tensor(t, dtype=d64)) for t in thetas[2:6]]
    g["log_R"] = np.array([r.numpy() for r in rots])
    g["log_out"] = np.array([rpose.SO3_log(r.float()).numpy() for r in rots])

    # --- Camera --------------------------------------------------------------------
    R0 = rpose.SO3_exp(torch.tensor([0.1, -0.2, 0.05], dtype=d64)).float()
    t0 = torch.tensor([0.3, -0.1, 0.4])
    ang = torch.tensor([0.2, -0.1, 0.3])
    lin = torch.tensor([0.4, 0.1, -0.2])
    W, H, fx, fy = 640, 480, 600.0, 610.0
    fovx = rcam.focal2fov(fx, W)
    fovy = rcam.focal2fov(fy, H)
    dtau = 0.01
    cam = rcam.Camera(R0, t0, ang.clone(), lin.clone(), fovx, fovy, W, H, delta_tau=dtau, device="cpu")
    cam.fx, cam.fy = fx, fy
    g["cam_R"], g["cam_t"], g["cam_ang"], g["cam_lin"] = R0.numpy(), t0.numpy(), ang.numpy(), lin.numpy()
    g["cam_size_focal"] = np.array([W, H, fx, fy, dtau])
    g["cam_world_view"] = cam.world_view_transform.numpy()
    g["cam_proj"] = cam.projection_matrix.numpy()
    g["cam_full_proj"] = cam.full_proj_transform.numpy()
    g["cam_center"] = cam.camera_center.numpy()
    g["cam_last_vel"] = cam.last_vel_transform.numpy()
    g["cam_next_vel"] = cam.next_vel_transform.numpy()
    # the rendered pair (frame.py:61-82) and its scaled cameras, captured at render2
    captured = {}

    def fake_render2(last, curr, nxt, pc, bg, *a, **k):
        captured["last"], captured["next"] = last, nxt
        img = lambda s: {"render": torch.full((3, last.image_height, last.image_width), s)}
        return img(0.25), img(0.5)

    rframe.render2 = fake_render2
    for lvl in (0, 1, 2):
        rf = object.__new__(rframe.RenderFrame)
        rf.viewpoint, rf.gaussians, rf.pipeline, rf.background = cam, None, None, None
        rf.get_delta_Ir(lvl)
        for nm in ("last", "next"):
            c = captured[nm]
            g["pair_%s_l%d_R" % (nm, lvl)] = c.R.detach().numpy()
            g["pair_%s_l%d_t" % (nm, lvl)] = c.T.detach().numpy()
            g["pair_%s_l%d_size_fov" % (nm, lvl)] = np.array([c.image_width, c.image_height, c.FoVx, c.FoVy])
    # update_pose / update_velocity / update_vwRT
    with torch.no_grad():
        cam.cam_rot_delta.copy_(torch.tensor([0.01, -0.02, 0.005]))
        cam.cam_trans_delta.copy_(torch.tensor([0.03, 0.01, -0.02]))
        cam.cam_w_delta.copy_(torch.tensor([0.1, 0.0, -0.1]))
        cam.cam_v_delta.copy_(torch.tensor([-0.05, 0.02, 0.01]))
    g["upd_deltas"] = np.concatenate([cam.cam_rot_delta.detach().numpy(), cam.cam_trans_delta.detach().numpy(),
                                      cam.cam_w_delta.detach().numpy(), cam.cam_v_delta.detach().numpy()])
    cam.update_vwRT()
    g["upd_R"], g["upd_t"] = cam.R.detach().numpy(), cam.T.detach().numpy()
    g["upd_ang"], g["upd_lin"] = cam.angular_vel.detach().numpy(), cam.linear_vel.detach().numpy()
    last_status = [cam.T.detach().clone(), cam.R.detach().clone()]
    cam.const_vel_model(0.02)
    g["cvm_tau"] = np.array(0.02)
    g["cvm_R"], g["cvm_t"] = cam.R.detach().numpy(), cam.T.detach().numpy()
    cam.cal_weighted_velocity(last_status, 0.02, 0.5)
    g["cwv_ang"], g["cwv_lin"] = cam.angular_vel.detach().numpy(), cam.linear_vel.detach().numpy()

    # --- grey, normalised intensity change, loss ------------------------------------
    c_last = torch.tensor(rng.uniform(0, 1, (3, 24, 32)), dtype=torch.float32)
    c_next = torch.tensor(rng.uniform(0, 1, (3, 24, 32)), dtype=torch.float32)
    grey_l = rframe.RenderFrame.get_intensity_frame(None, c_last)
    grey_n = rframe.RenderFrame.get_intensity_frame(None, c_next)

    def fake_render2b(last, curr, nxt, pc, bg, *a, **k):
        return {"render": c_last}, {"render": c_next}

    rframe.render2 = fake_render2b
    rf = object.__new__(rframe.RenderFrame)
    rf.viewpoint, rf.gaussians, rf.pipeline, rf.background = cam, None, None, None
    # pyramid level 0 with a 32x24 "camera": only the renders matter here
    cam_small = rcam.Camera(R0, t0, ang.clone(), lin.clone(), fovx, fovy, 32, 24, delta_tau=dtau, device="cpu")
    cam_small.fx, cam_small.fy = fx, fy
    rf.viewpoint = cam_small
    s_dIr, u_dIr = rf.get_delta_Ir(0)
    g["dIr_color_last"], g["dIr_color_next"] = c_last.numpy(), c_next.numpy()
    g["dIr_grey_last"], g["dIr_grey_next"] = grey_l.numpy(), grey_n.numpy()
    g["dIr_signed"], g["dIr_unsigned"] = s_dIr.detach().numpy(), u_dIr.detach().numpy()
    E = torch.tensor(rng.normal(size=(1, 24, 32)), dtype=torch.float32)
    E = E / torch.norm(E)
    g["loss_E"] = E.numpy()
    g["loss_signed"] = rtracker.Tracker.tracking_loss(None, s_dIr, E).detach().numpy()
    g["loss_unsigned"] = rtracker.Tracker.tracking_loss(None, u_dIr, torch.abs(E)).detach().numpy()
    losses = [1.0 - 0.01 * i + 1e-5 * (i % 3) for i in range(30)]
    g["conv_losses"] = np.array(losses)
    g["conv_results"] = np.array([rtracker.Tracker.check_convergence(None, losses[:k], 1e-3) for k in range(1, 31)])
    flat = [0.5 + 1e-6 * (i % 2) for i in range(15)]
    g["conv_flat"] = np.array(flat)
    g["conv_flat_results"] = np.array([rtracker.Tracker.check_convergence(None, flat[:k], 1e-4)
                                       for k in range(1, 16)])

    # --- SH evaluation ------------------------------------------------------------------
    n = 64
    sh = rng.normal(0.0, 0.3, size=(n, 16, 3)).astype(np.float32)
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    g["sh_coeffs"], g["sh_dirs"] = sh, dirs
    for deg in range(4):
        res = sh_utils.eval_sh(deg, torch.tensor(sh, dtype=d64).transpose(1, 2), torch.tensor(dirs, dtype=d64))
        g["sh_out_deg%d" % deg] = (res + 0.5).numpy()

    # --- cov3D ----------------------------------------------------------------------------
    scale = np.exp(rng.normal(-4.0, 0.5, size=(n, 3))).astype(np.float32)
    q = rng.normal(size=(n, 4))
    q = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    with no_cuda_device():
        L = general_utils.build_scaling_rotation(torch.tensor(scale), torch.tensor(q))
        cov = general_utils.strip_symmetric(L @ L.transpose(1, 2))
    g["cov_scale"], g["cov_rot"], g["cov_out"] = scale, q, cov.numpy()

    np.savez_compressed(OUT, **g)
    print("wrote", OUT, len(g), "arrays")


if __name__ == "__main__":
    main()
