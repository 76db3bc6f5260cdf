"""FP64 pose algebra of the oracle — test infrastructure only.

Restates, in numpy float64, the reference's pose and camera algebra:
  - skew_sym_mat, SO3_exp (small-angle branch < 1e-5), SO3_log, V, SE3_exp(deltaT=[rho, theta]):
    utils/pose.py:13-91
  - Camera.world_view_transform / projection_matrix / full_proj_transform / camera_center:
    utils/render_camera/camera.py:68-91 with graphics_utils.py:33-69 (getWorld2View2,
    getProjectionMatrix, znear 0.01, zfar 100, camera.py:58-59) and focal2fov (:100-101)
  - last/next velocity transforms SE3_exp(-/+[v, w] dtau/2): camera.py:100-123
  - update_pose (left-multiply SE3_exp([rho, theta])): camera.py:133-147
  - update_velocity: camera.py:149-155; const_vel_model: camera.py:183-201;
    cal_weighted_velocity: camera.py:157-181
  - the rendered pair poses E(-/+) @ T: utils/render_camera/frame.py:68-82
These functions are pinned against fixtures generated from the reference Python
(tests/golden/make_golden.py).  The exact SE(3) left Jacobian used for the velocity
gradient chain is the published closed form (Barfoot & Furgale, IEEE T-RO 2014).
"""
import math

import numpy as np


def skew(x):
    x = np.asarray(x, dtype=np.float64)
    return np.array([[0.0, -x[2], x[1]], [x[2], 0.0, -x[0]], [-x[1], x[0], 0.0]])


def so3_exp(theta):
    theta = np.asarray(theta, dtype=np.float64)
    W = skew(theta)
    W2 = W @ W
    a = np.linalg.norm(theta)
    if a < 1e-5:
        return np.eye(3) + W + 0.5 * W2
    return np.eye(3) + (math.sin(a) / a) * W + ((1.0 - math.cos(a)) / (a * a)) * W2


def so3_log(R):
    c = (np.trace(R) - 1.0) / 2.0
    c = min(1.0, max(-1.0, c))
    th = math.acos(c)
    if abs(th) < 1e-5:
        return np.zeros(3)
    axis = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / (2.0 * math.sin(th))
    return th * axis


def so3_left_jacobian(theta):
    """V(theta) of utils/pose.py:61-76 (the SO(3) left Jacobian)."""
    theta = np.asarray(theta, dtype=np.float64)
    W = skew(theta)
    W2 = W @ W
    a = np.linalg.norm(theta)
    if a < 1e-5:
        return np.eye(3) + 0.5 * W + (1.0 / 6.0) * W2
    return np.eye(3) + W * ((1.0 - math.cos(a)) / a ** 2) + W2 * ((a - math.sin(a)) / a ** 3)


def se3_exp(xi):
    """xi = [rho(3), theta(3)] -> 4x4, as utils/pose.py:79-91."""
    xi = np.asarray(xi, dtype=np.float64)
    T = np.eye(4)
    T[:3, :3] = so3_exp(xi[3:])
    T[:3, 3] = so3_left_jacobian(xi[3:]) @ xi[:3]
    return T


def se3_left_jacobian(xi):
    """Exact 6x6 left Jacobian of SE(3) for xi = [rho, theta] (Barfoot & Furgale 2014):
    exp(xi + d) ~= exp(J_l(xi) d) exp(xi)."""
    xi = np.asarray(xi, dtype=np.float64)
    rho, phi = xi[:3], xi[3:]
    J = so3_left_jacobian(phi)
    a = np.linalg.norm(phi)
    P, Rh = skew(phi), skew(rho)
    if a < 1e-4:
        Q = 0.5 * Rh + (1.0 / 6.0) * (P @ Rh + Rh @ P + P @ Rh @ P) \
            + (1.0 / 24.0) * (P @ P @ Rh + Rh @ P @ P - 3.0 * P @ Rh @ P) \
            + (1.0 / 120.0) * (P @ Rh @ P @ P + P @ P @ Rh @ P)
    else:
        a2, a3, a4, a5 = a * a, a ** 3, a ** 4, a ** 5
        c1 = (a - math.sin(a)) / a3
        c2 = (a2 + 2.0 * math.cos(a) - 2.0) / (2.0 * a4)
        c3 = (2.0 * a - 3.0 * math.sin(a) + a * math.cos(a)) / (2.0 * a5)
        Q = 0.5 * Rh + c1 * (P @ Rh + Rh @ P + P @ Rh @ P) \
            + c2 * (P @ P @ Rh + Rh @ P @ P - 3.0 * P @ Rh @ P) \
            + c3 * (P @ Rh @ P @ P + P @ P @ Rh @ P)
    Jl = np.zeros((6, 6))
    Jl[:3, :3] = J
    Jl[:3, 3:] = Q
    Jl[3:, 3:] = J
    return Jl


def se3_adjoint(T):
    """Ad(T) for twists ordered [rho, theta]: exp(Ad(T) xi) = T exp(xi) T^-1."""
    R, t = T[:3, :3], T[:3, 3]
    A = np.zeros((6, 6))
    A[:3, :3] = R
    A[:3, 3:] = skew(t) @ R
    A[3:, 3:] = R
    return A


def focal2fov(focal, pixels):
    return 2.0 * math.atan(pixels / (2.0 * focal))


def projection_matrix(fovx, fovy, znear=0.01, zfar=100.0):
    """getProjectionMatrix (graphics_utils.py:49-69), un-transposed (camera -> clip)."""
    th_y, th_x = math.tan(fovy / 2.0), math.tan(fovx / 2.0)
    top, right = th_y * znear, th_x * znear
    bottom, left = -top, -right
    P = np.zeros((4, 4))
    P[0, 0] = 2.0 * znear / (right - left)
    P[1, 1] = 2.0 * znear / (top - bottom)
    P[0, 2] = (right + left) / (right - left)
    P[1, 2] = (top + bottom) / (top - bottom)
    P[3, 2] = 1.0
    P[2, 2] = zfar / (zfar - znear)
    P[2, 3] = -(zfar * znear) / (zfar - znear)
    return P


def camera_center(R, t):
    """-R^T t (camera.py:89-91 computes it as the inverse of the view matrix)."""
    return -np.asarray(R).T @ np.asarray(t)


def view_vector(R, t, W, H, fx, fy, dtype=np.float32):
    """Oracle view layout: R[9] row-major, t[3], Praw[16] row-major, campos[3], tanfx, tanfy."""
    fovx, fovy = focal2fov(fx, W), focal2fov(fy, H)
    P = projection_matrix(fovx, fovy)
    v = np.concatenate([np.asarray(R, np.float64).reshape(9), np.asarray(t, np.float64).reshape(3),
                        P.reshape(16), camera_center(R, t),
                        [math.tan(fovx * 0.5), math.tan(fovy * 0.5)]])
    return v.astype(dtype)


def vel_transforms(lin_vel, ang_vel, delta_tau):
    """(last, next) = SE3_exp(-/+[v, w] dtau/2)  (camera.py:100-123)."""
    rv = np.asarray(ang_vel, np.float64) * (delta_tau / 2.0)
    tv = np.asarray(lin_vel, np.float64) * (delta_tau / 2.0)
    return se3_exp(np.concatenate([-tv, -rv])), se3_exp(np.concatenate([tv, rv]))


def pose_matrix(R, t):
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def pair_poses(R, t, lin_vel, ang_vel, delta_tau):
    """Rendered poses of the (t, t + dtau) pair: E(-/+) @ T  (frame.py:68-73)."""
    El, En = vel_transforms(lin_vel, ang_vel, delta_tau)
    T = pose_matrix(R, t)
    return El @ T, En @ T


def tracked_pair_poses(R, t, lin_vel, ang_vel, delta_tau, rho, theta, dv, dw):
    """Rendered poses as functions of the optimised deltas: the pose delta left-multiplies
    the current pose (camera.py:133-147) and the velocity deltas add to the velocity
    (camera.py:149-155)."""
    T = se3_exp(np.concatenate([rho, theta])) @ pose_matrix(R, t)
    El, En = vel_transforms(np.asarray(lin_vel) + dv, np.asarray(ang_vel) + dw, delta_tau)
    return El @ T, En @ T


def chain_pose_gradient(g_last, g_next, lin_vel, ang_vel, delta_tau):
    """Exact chain from per-view left-twist gradients g_v = dL/dxi_v ([rho, theta] order) to
    the 12 optimised deltas (theta, rho, w, v) of the current camera.
    T_v = E_v(u) exp(delta) T, E_v = exp(s h u), u = [v, w], h = dtau/2, s = -1/+1."""
    u = np.concatenate([np.asarray(lin_vel, np.float64), np.asarray(ang_vel, np.float64)])
    h = delta_tau / 2.0
    g_pose = np.zeros(6)
    g_vel = np.zeros(6)
    for s, g in ((-1.0, np.asarray(g_last, np.float64)), (1.0, np.asarray(g_next, np.float64))):
        E = se3_exp(s * h * u)
        g_pose += se3_adjoint(E).T @ g
        g_vel += s * h * (se3_left_jacobian(s * h * u).T @ g)
    # order returned: theta, rho, w, v (the reference's parameter names)
    return g_pose[3:], g_pose[:3], g_vel[3:], g_vel[:3]


def update_pose(R, t, rho, theta):
    T = se3_exp(np.concatenate([rho, theta])) @ pose_matrix(R, t)
    return T[:3, :3], T[:3, 3]


def const_vel_model(R, t, lin_vel, ang_vel, tau):
    """camera.py:183-201: new pose = SE3_exp([v, w] tau) @ T."""
    D = se3_exp(np.concatenate([np.asarray(lin_vel) * tau, np.asarray(ang_vel) * tau]))
    T = D @ pose_matrix(R, t)
    return T[:3, :3], T[:3, 3]


def cal_weighted_velocity(R, t, last_R, last_t, lin_vel, ang_vel, delta_tau, weight):
    """camera.py:157-181."""
    delta = pose_matrix(R, t) @ np.linalg.inv(pose_matrix(last_R, last_t))
    lv = delta[:3, 3] / delta_tau
    av = so3_log(delta[:3, :3]) / delta_tau
    return (weight * lv + (1 - weight) * np.asarray(lin_vel),
            weight * av + (1 - weight) * np.asarray(ang_vel))
