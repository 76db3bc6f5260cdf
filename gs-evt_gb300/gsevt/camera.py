"""Camera with learnable pose / velocity deltas: the API of the reference's
utils/render_camera/camera.py:9-219 (same constructor, properties and update methods),
so the plain per-view tracking path can run the reference's per-iteration structure on
top of the drop-in rasterizer.  Arithmetic is torch float32 on the camera's device, as
in the reference.
"""
import math

import torch
from torch import nn


def _skew(x):
    z = torch.zeros((), dtype=x.dtype, device=x.device)
    return torch.stack([torch.stack([z, -x[2], x[1]]), torch.stack([x[2], z, -x[0]]),
                        torch.stack([-x[1], x[0], z])])


def so3_exp(theta):
    """Rodrigues with the small-angle branch below 1e-5 (utils/pose.py:26-41)."""
    W = _skew(theta)
    W2 = W @ W
    a = torch.norm(theta)
    I = torch.eye(3, dtype=theta.dtype, device=theta.device)
    if a < 1e-5:
        return I + W + 0.5 * W2
    return I + (torch.sin(a) / a) * W + ((1 - torch.cos(a)) / (a * a)) * W2


def so3_left_jacobian(theta):
    W = _skew(theta)
    W2 = W @ W
    a = torch.norm(theta)
    I = torch.eye(3, dtype=theta.dtype, device=theta.device)
    if a < 1e-5:
        return I + 0.5 * W + (1.0 / 6.0) * W2
    return I + W * ((1 - torch.cos(a)) / (a * a)) + W2 * ((a - torch.sin(a)) / (a ** 3))


def se3_exp(xi):
    """xi = [rho, theta] -> 4x4 (utils/pose.py:79-91)."""
    T = torch.eye(4, dtype=xi.dtype, device=xi.device)
    T[:3, :3] = so3_exp(xi[3:])
    T[:3, 3] = so3_left_jacobian(xi[3:]) @ xi[:3]
    return T


def so3_log(R):
    c = torch.clamp((torch.trace(R) - 1.0) / 2.0, -1.0, 1.0)
    th = torch.acos(c)
    if th.abs() < 1e-5:
        return torch.zeros(3, device=R.device, dtype=R.dtype)
    axis = torch.stack([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / (2 * torch.sin(th))
    return th * axis


def focal2fov(focal, pixels):
    return 2 * math.atan(pixels / (2 * focal))


def projection_matrix(znear, zfar, fovx, fovy):
    """graphics_utils.py:49-69 (camera -> clip, un-transposed)."""
    top = math.tan(fovy / 2) * znear
    right = math.tan(fovx / 2) * znear
    P = torch.zeros(4, 4)
    P[0, 0] = 2.0 * znear / (2 * right)
    P[1, 1] = 2.0 * znear / (2 * top)
    P[3, 2] = 1.0
    P[2, 2] = zfar / (zfar - znear)
    P[2, 3] = -(zfar * znear) / (zfar - znear)
    return P


class Camera(nn.Module):
    def __init__(self, R, t, angular_vel, linear_vel, fovx, fovy, image_width, image_height, delta_tau=0,
                 device="cuda"):
        super().__init__()
        self.device = torch.device(device)
        self.R = torch.as_tensor(R, dtype=torch.float32).to(self.device)
        self.T = torch.as_tensor(t, dtype=torch.float32).to(self.device)
        self.angular_vel = torch.as_tensor(angular_vel, dtype=torch.float32).to(self.device)
        self.linear_vel = torch.as_tensor(linear_vel, dtype=torch.float32).to(self.device)
        self.FoVx, self.FoVy = fovx, fovy
        self.image_width, self.image_height = image_width, image_height
        self.zfar, self.znear = 100.0, 0.01
        self.delta_tau = delta_tau
        z = lambda: torch.zeros(3, device=self.device)
        self.cam_rot_delta = nn.Parameter(z(), requires_grad=True)
        self.cam_trans_delta = nn.Parameter(z(), requires_grad=True)
        self.cam_w_delta = nn.Parameter(z(), requires_grad=False)
        self.cam_v_delta = nn.Parameter(z(), requires_grad=False)

    @property
    def projection_matrix(self):
        return projection_matrix(self.znear, self.zfar, self.FoVx, self.FoVy).transpose(0, 1).to(self.device)

    @property
    def world_view_transform(self):
        Rt = torch.eye(4, device=self.device)
        Rt[:3, :3] = self.R
        Rt[:3, 3] = self.T
        return Rt.transpose(0, 1)

    @property
    def full_proj_transform(self):
        return self.world_view_transform @ self.projection_matrix

    @property
    def camera_center(self):
        return -(self.R.transpose(0, 1) @ self.T)

    @property
    def curr_pose(self):
        T = torch.eye(4, device=self.device)
        T[:3, :3] = self.R
        T[:3, 3] = self.T
        return T

    def compute_motion_vectors(self):
        return self.angular_vel * (self.delta_tau / 2), self.linear_vel * (self.delta_tau / 2)

    @property
    def last_vel_transform(self):
        rv, tv = self.compute_motion_vectors()
        return se3_exp(torch.cat([-tv, -rv]))

    @property
    def last_vel_transform_inv(self):
        return torch.linalg.inv(self.last_vel_transform)

    @property
    def next_vel_transform(self):
        rv, tv = self.compute_motion_vectors()
        return se3_exp(torch.cat([tv, rv]))

    @property
    def next_vel_transform_inv(self):
        return torch.linalg.inv(self.next_vel_transform)

    def update_RT(self, R, t):
        self.R = R.to(self.device)
        self.T = t.to(self.device)

    def update_vwRT(self):
        self.update_velocity()
        self.update_pose()

    def update_pose(self):
        T = se3_exp(torch.cat([self.cam_trans_delta, self.cam_rot_delta])) @ self.curr_pose
        self.update_RT(T[:3, :3], T[:3, 3])
        self.cam_rot_delta.data.fill_(0)
        self.cam_trans_delta.data.fill_(0)

    def update_velocity(self):
        self.angular_vel = self.angular_vel + self.cam_w_delta.data
        self.linear_vel = self.linear_vel + self.cam_v_delta.data
        self.cam_w_delta.data.fill_(0)
        self.cam_v_delta.data.fill_(0)

    def cal_weighted_velocity(self, last_data, delta_tau, weight):
        last = torch.eye(4, device=self.device)
        last[:3, :3] = last_data[1]
        last[:3, 3] = last_data[0]
        delta = self.curr_pose.detach() @ torch.inverse(last)
        lv = delta[:3, 3] / delta_tau
        av = so3_log(delta[:3, :3]) / delta_tau
        self.linear_vel = weight * lv + (1 - weight) * self.linear_vel
        self.angular_vel = weight * av + (1 - weight) * self.angular_vel

    def const_vel_model(self, tau):
        D = se3_exp(torch.cat([self.linear_vel * tau, self.angular_vel * tau]))
        T = D @ self.curr_pose
        self.last_R, self.last_T = self.R.clone(), self.T.clone()
        self.update_RT(T[:3, :3], T[:3, 3])

    @staticmethod
    def init_from_yaml(config):
        """Camera.init_from_yaml (camera.py:203-219) over a plain dict config."""
        g, tr = config["Gaussian"], config["Tracking"]
        W, H = g["img_width"], g["img_height"]
        dev = g["model_params"]["device"]
        R = torch.tensor(tr["initial_pose"]["rot"]["data"], dtype=torch.float32).reshape(3, 3)
        t = torch.tensor(tr["initial_pose"]["trans"]["data"], dtype=torch.float32).reshape(3)
        lin = torch.tensor(tr["initial_vel"]["linear_vel"], dtype=torch.float32)
        ang = torch.tensor(tr["initial_vel"]["angular_vel"], dtype=torch.float32)
        cp = g["calib_params"]
        cam = Camera(R, t, ang, lin, focal2fov(cp["fx"], W), focal2fov(cp["fy"], H), W, H, device=dev)
        cam.fx, cam.fy = cp["fx"], cp["fy"]
        cam.update_pose()
        return cam
