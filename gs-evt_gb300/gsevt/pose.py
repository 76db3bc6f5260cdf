"""Host-side FP64 SE(3) algebra for building view tables and initial tracker states.

Conventions follow the reference: twists are [rho (translation), theta (rotation)]
(utils/pose.py:79-91), poses are world -> camera with the update T <- exp(xi) T
(utils/render_camera/camera.py:133-147), the rendered pair is E(-/+ [v, w] dtau/2) T
(camera.py:100-123), projection matrices follow graphics_utils.py:49-69 with
znear 0.01, zfar 100 (camera.py:58-59).  The device keeps the same algebra in FP64
(csrc/track.cu).
"""
import math

import numpy as np


def hat(v):
    x, y, z = (float(a) for a in v)
    return np.array([[0.0, -z, y], [z, 0.0, -x], [-y, x, 0.0]])


def _coeffs(angle):
    """(sin a / a, (1 - cos a) / a^2, (a - sin a) / a^3) with the reference's small-angle
    branch below 1e-5 (utils/pose.py:35-36, 70-71)."""
    if angle < 1e-5:
        return 1.0, 0.5, 1.0 / 6.0
    s, c = math.sin(angle), math.cos(angle)
    return s / angle, (1.0 - c) / angle ** 2, (angle - s) / angle ** 3


def exp_so3(theta):
    K = hat(theta)
    a, b, _ = _coeffs(float(np.linalg.norm(theta)))
    return np.eye(3) + a * K + b * (K @ K)


def left_jacobian_so3(theta):
    K = hat(theta)
    _, b, c = _coeffs(float(np.linalg.norm(theta)))
    return np.eye(3) + b * K + c * (K @ K)


def exp_se3(xi):
    xi = np.asarray(xi, np.float64)
    T = np.eye(4)
    T[:3, :3] = exp_so3(xi[3:])
    T[:3, 3] = left_jacobian_so3(xi[3:]) @ xi[:3]
    return T


def matrix(R, t):
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def focal2fov(focal, pixels):
    return 2.0 * math.atan(pixels / (2.0 * focal))


def projection_matrix(fovx, fovy, znear=0.01, zfar=100.0):
    tx, ty = math.tan(fovx / 2.0), math.tan(fovy / 2.0)
    P = np.zeros((4, 4))
    P[0, 0] = 1.0 / tx
    P[1, 1] = 1.0 / ty
    P[2, 2] = zfar / (zfar - znear)
    P[2, 3] = -(zfar * znear) / (zfar - znear)
    P[3, 2] = 1.0
    return P


def pair_poses(R, t, lin_vel, ang_vel, delta_tau):
    h = 0.5 * delta_tau
    u = np.concatenate([np.asarray(lin_vel, np.float64), np.asarray(ang_vel, np.float64)])
    T = matrix(R, t)
    return exp_se3(-h * u) @ T, exp_se3(h * u) @ T


def campos(R, t):
    return -np.asarray(R).T @ np.asarray(t)


def so3_log(R):
    c = min(1.0, max(-1.0, (np.trace(R) - 1.0) / 2.0))
    th = math.acos(c)
    if abs(th) < 1e-5:
        return np.zeros(3)
    return th * np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / (2.0 * math.sin(th))


def rotation_error_deg(Ra, Rb):
    """Angle of Ra Rb^T in degrees, as atan2(sin, cos) of the relative rotation (the trace
    alone loses angles below ~0.03 degrees to rounding when either matrix is FP32)."""
    D = np.asarray(Ra, np.float64) @ np.asarray(Rb, np.float64).T
    s = 0.5 * np.linalg.norm([D[2, 1] - D[1, 2], D[0, 2] - D[2, 0], D[1, 0] - D[0, 1]])
    c = 0.5 * (np.trace(D) - 1.0)
    return math.degrees(math.atan2(s, c))
