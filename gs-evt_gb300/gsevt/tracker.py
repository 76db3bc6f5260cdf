"""Plain per-view tracking path: RenderFrame and Tracker with the API of the reference's
utils/render_camera/frame.py:10-94 and utils/tracker.py:33-287, running on the drop-in
rasterizer.  Each iteration renders the (t, t + dtau) pair with two rasterizer calls,
forms the grey intensity change with torch ops, back-propagates through autograd and
steps torch.optim.Adam, exactly the reference's per-iteration structure.  The batched
path (gsevt.batched) does the same iteration in one graph-captured launch sequence.
"""
import logging
import os

import numpy as np
import torch

from .camera import Camera, focal2fov
from .events import EventFrame
from .renderer import render1, render2

GREY_WEIGHTS = (0.2989, 0.5870, 0.1140)


class RenderFrame:
    """log_eps: None for the reference's linear grey change (frame.py:86-92), or eps > 0
    for the log-intensity change ln(I_next + eps) - ln(I_last + eps) of the paper."""

    def __init__(self, viewpoint, gaussians, pipeline, background, pyramid_level, log_eps=None):
        self.viewpoint, self.gaussians, self.pipeline, self.background = viewpoint, gaussians, pipeline, background
        self.log_eps = log_eps
        self.sign_delta_Ir, self.unsign_delta_Ir = self.get_delta_Ir(pyramid_level)

    @staticmethod
    def get_intensity_frame(color_frame):
        w = torch.tensor(GREY_WEIGHTS, device=color_frame.device).view(1, 3, 1, 1)
        return (color_frame * w).sum(dim=1)

    def render(self):
        return render1(self.viewpoint, self.gaussians, self.background)

    def get_delta_Ir(self, pyramid_level=0):
        vp = self.viewpoint
        assert vp.delta_tau != 0, "delta_tau should not be zero"
        s = 0.5 ** pyramid_level
        w, h = int(vp.image_width * s), int(vp.image_height * s)
        cams = []
        for E in (vp.last_vel_transform, vp.next_vel_transform):
            T = E @ vp.curr_pose
            cams.append(Camera(T[:3, :3], T[:3, 3], vp.angular_vel, vp.linear_vel, focal2fov(vp.fx * s, w),
                               focal2fov(vp.fy * s, h), w, h, delta_tau=vp.delta_tau, device=vp.device))
        last_pkg, next_pkg = render2(cams[0], vp, cams[1], self.gaussians, self.background)
        In, Il = self.get_intensity_frame(next_pkg["render"]), self.get_intensity_frame(last_pkg["render"])
        if self.log_eps:
            In, Il = torch.log(In + self.log_eps), torch.log(Il + self.log_eps)
        d = In - Il
        n = d / torch.norm(d, p=2)
        return n, torch.abs(n)


def tracking_loss(delta_Ir, delta_Ie):
    return torch.norm(delta_Ir - delta_Ie)


def check_convergence(losses, threshold=1e-4):
    """Mean |slope| of the last 10 loss steps below the threshold (tracker.py:65-76)."""
    if len(losses) <= 10:
        return False
    return bool(np.mean(np.abs(np.diff(losses[-11:]))) < threshold)


def make_optimizer(viewpoint, lrs):
    groups = [{"params": [viewpoint.cam_rot_delta], "lr": lrs["cam_rot_delta"]},
              {"params": [viewpoint.cam_trans_delta], "lr": lrs["cam_trans_delta"]},
              {"params": [viewpoint.cam_w_delta], "lr": lrs["cam_w_delta"]},
              {"params": [viewpoint.cam_v_delta], "lr": lrs["cam_v_delta"]}]
    return torch.optim.Adam(groups)


def plain_iteration(viewpoint, gaussians, background, optimizer, lvl, opt_vel, sign_Ie, unsign_Ie,
                    lr_fraction=None, lrs=None, read_loss=True, log_eps=None):
    """One tracking iteration of the plain path (tracker.py:177-222); log_eps selects the
    log-intensity change (RenderFrame)."""
    viewpoint.cam_w_delta.requires_grad_(bool(opt_vel))
    viewpoint.cam_v_delta.requires_grad_(bool(opt_vel))
    if opt_vel and lr_fraction is not None and lrs is not None:
        names = ["cam_rot_delta", "cam_trans_delta", "cam_w_delta", "cam_v_delta"]
        for g, name in zip(optimizer.param_groups, names):
            f = lr_fraction if name in ("cam_rot_delta", "cam_trans_delta") else 1 - lr_fraction
            g["lr"] = lrs[name] * f
    rf = RenderFrame(viewpoint, gaussians, None, background, lvl, log_eps=log_eps)
    loss = tracking_loss(rf.sign_delta_Ir, sign_Ie) if opt_vel else tracking_loss(rf.unsign_delta_Ir, unsign_Ie)
    loss.backward()
    val = loss.item() if read_loss else loss.detach()
    with torch.no_grad():
        optimizer.step()
        if opt_vel:
            viewpoint.update_vwRT()
        else:
            viewpoint.update_pose()
        optimizer.zero_grad()
    return val, rf


class Tracker:
    """Tracker(config, event_arrays, viewpoint, gaussians, pipeline, background, device)
    .tracking() — per frame: constant-velocity prediction, event pyramid, coarse
    (pose, unsigned loss) then fine (pose + velocity, signed loss) Adam stages per
    pyramid level with slope-based convergence (tracker.py:105-287).  Poses are returned
    as a list of (timestamp, R, t); with config["Tracking"]["save_path"] they are also
    written as the reference writes them (tracking_pose_tum.txt, and one overlay image per
    frame in tracking_frames/frame_<i>.png, utils/tracker.py:106-108, 258-270)."""

    def __init__(self, config, event_arrays, viewpoint, gaussians, pipeline, background, device="cuda"):
        self.config, self.event_arrays = config, event_arrays
        self.viewpoint, self.gaussians, self.pipeline, self.background = viewpoint, gaussians, pipeline, background
        self.device = device
        ev = config["Event"]
        self.img_width, self.img_height = ev["img_width"], ev["img_height"]
        self.gaussian_kernel_size = ev["gaussian_kernel_size"]
        self.intrinsic = np.array(ev["intrinsic"]["data"]).reshape(3, 3)
        self.distortion_factors = np.array(ev["distortion_factors"])
        opt = config["Optimizer"]
        self.converged_threshold, self.max_optim_iter = opt["converged_threshold"], opt["max_optim_iter"]
        self.lrs = {k: opt[k] for k in ("cam_rot_delta", "cam_trans_delta", "cam_w_delta", "cam_v_delta")}
        self.pyramid_lvl = 3
        self.log = logging.getLogger("gsevt.tracker")
        tracking_cfg = (config.get("Tracking") or {}) if hasattr(config, "get") else {}
        self.save_path = tracking_cfg.get("save_path")
        # optional (not a key of the reference's configs): eps of the log-intensity change
        self.log_eps = tracking_cfg.get("log_grey_eps")
        self.trajectory = []
        self.iterations = 0

    def check_convergence(self, losses, threshold=1e-4):
        return check_convergence(losses, threshold)

    def tracking_loss(self, delta_Ir, delta_Ie, mask=None, huber=False):
        r = delta_Ir * mask - delta_Ie if mask is not None else delta_Ir - delta_Ie
        if huber:
            return torch.nn.functional.huber_loss(r, torch.zeros_like(r), delta=0.002, reduction="none").sum()
        return torch.norm(r)

    def tracking(self):
        from . import io as gio
        vp = self.viewpoint
        last_delta_tau = 0.0
        fraction_num = self.max_optim_iter / 2
        if self.save_path:
            os.makedirs(os.path.join(self.save_path, "tracking_frames"), exist_ok=True)
        for frame_idx, ea in enumerate(self.event_arrays):
            optimizer = make_optimizer(vp, self.lrs)
            delta_tau = ea.duration()
            vp.delta_tau = delta_tau
            vp.const_vel_model((delta_tau + last_delta_tau) / 2)
            initial = [vp.T.detach().clone(), vp.R.detach().clone()]
            ef = EventFrame(self.img_width, self.img_height, self.intrinsic, self.distortion_factors,
                            self.gaussian_kernel_size, ea, device=self.device, levels=self.pyramid_lvl)
            for lvl in range(self.pyramid_lvl - 1, -1, -1):
                opt_vel = lvl != self.pyramid_lvl - 1
                start_vel = 0
                for g, name in zip(optimizer.param_groups, self.lrs):
                    g["lr"] = self.lrs[name]
                losses, it = [], 0
                while True:
                    frac = None
                    if opt_vel:
                        k = it - start_vel
                        frac = k / fraction_num if 1 <= k <= fraction_num else 1
                    val, rf = plain_iteration(vp, self.gaussians, self.background, optimizer, lvl, opt_vel,
                                              ef.sign_pyramid[lvl], ef.unsign_pyramid[lvl], frac, self.lrs,
                                              log_eps=self.log_eps)
                    self.iterations += 1
                    losses.append(val)
                    if self.check_convergence(losses, self.converged_threshold):
                        if not opt_vel:
                            opt_vel, start_vel = True, it
                        else:
                            break
                    limit = self.max_optim_iter if not opt_vel else start_vel + self.max_optim_iter
                    if it >= limit:
                        self.log.error("optimisation exceeded max_optim_iter at level %d", lvl)
                        break
                    it += 1
            if frame_idx >= 5:
                vp.cal_weighted_velocity(initial, (delta_tau + last_delta_tau) / 2, 0.5)
            last_delta_tau = delta_tau
            self.trajectory.append((ea.time(), vp.R.detach().cpu().numpy(), vp.T.detach().cpu().numpy()))
            if self.save_path:
                # the last render of the finest level against the frame's signed event frame
                img = gio.event_overlay(ef.sign_pyramid[0], rf.sign_delta_Ir)
                gio.write_png(os.path.join(self.save_path, "tracking_frames", "frame_%d.png" % frame_idx), img)
        if self.save_path:
            gio.write_tum(os.path.join(self.save_path, "tracking_pose_tum.txt"), self.trajectory)
        return self.trajectory
