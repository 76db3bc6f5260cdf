"""Seeded synthetic inputs standing in for the VECTOR sequences (the reference's data,
README.md:23,55, is not available): Gaussian maps, pinhole cameras, ground-truth
motion, perturbed initial states and event windows.

Distributions (shapes from configs/VECTOR/*.yaml: SH degree 3, 640x480, up to 30k
events per frame; sizes from the benchmark configurations):
  - means uniform in the box x in [-2, 2], y in [-1.5, 1.5], z in [1, 4] m in front of
    the ground-truth camera at t = 0 (a 4 x 3 x 3 m box; every point 1..5 m away);
  - log-scales N(-4, 0.5) per axis; rotations uniform unit quaternions (w, x, y, z);
  - opacity sigmoid(N(0, 1)); SH DC ~ N(0.5, 0.2), higher bands ~ N(0, 0.05);
  - ground-truth pose identity at t = 0, ground-truth velocity twist N(0, 0.3) per axis;
  - initial pose = ground truth perturbed by a twist of 5 cm / 3 degrees in random
    directions, initial velocity = ground truth + N(0, 0.1) per axis;
  - events: grey log-intensity rendered at the two ground-truth poses of the window,
    dL = log(I_next + 1e-3) - log(I_last + 1e-3), signal events distributed over pixels in
    proportion to |dL| / C with C = 0.2 (the count is then scaled to the requested
    total, of which 5 % are uniform noise events of random polarity), polarity
    sign(dL), timestamps uniform over the window.
"""
import math

import numpy as np

from . import pose as P


def sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def make_map(n, seed):
    rng = np.random.default_rng(seed)
    lo = np.array([-2.0, -1.5, 1.0])
    hi = np.array([2.0, 1.5, 4.0])
    xyz = rng.uniform(lo, hi, size=(n, 3))
    scale = np.exp(rng.normal(-4.0, 0.5, size=(n, 3)))
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    opacity = sigmoid(rng.normal(0.0, 1.0, size=n))
    sh = np.zeros((n, 16, 3))
    sh[:, 0, :] = rng.normal(0.5, 0.2, size=(n, 3))
    sh[:, 1:, :] = rng.normal(0.0, 0.05, size=(n, 15, 3))
    f = np.float32
    return dict(xyz=xyz.astype(f), scale=scale.astype(f), rot=q.astype(f), opacity=opacity.astype(f),
                sh=sh.astype(f))


class PinholeCamera:
    """Centred pinhole camera: tan(fov/2) = size / (2 f) (focal2fov,
    graphics_utils.py:100-101) and the reference's projection matrix."""

    def __init__(self, width, height, fx, fy=None):
        self.width, self.height = int(width), int(height)
        self.fx = float(fx)
        self.fy = float(fy if fy is not None else fx)
        self.fovx = P.focal2fov(self.fx, self.width)
        self.fovy = P.focal2fov(self.fy, self.height)
        self.tanfovx = math.tan(self.fovx * 0.5)
        self.tanfovy = math.tan(self.fovy * 0.5)
        self.proj = P.projection_matrix(self.fovx, self.fovy)

    def scaled(self, level):
        s = 0.5 ** level
        return PinholeCamera(int(self.width * s), int(self.height * s), self.fx * s, self.fy * s)


class Scenario:
    """One tracking problem: map, camera, ground truth and perturbed initial state."""

    def __init__(self, n, seed, width, height, focal, n_events, delta_tau=0.01, rot_deg=3.0, trans_m=0.05):
        self.seed = seed
        self.map = make_map(n, seed)
        self.camera = PinholeCamera(width, height, focal)
        rng = np.random.default_rng(seed + 1000)
        self.delta_tau = float(delta_tau)
        self.gt_R, self.gt_t = np.eye(3), np.zeros(3)
        self.gt_lin = rng.normal(0.0, 0.3, 3)
        self.gt_ang = rng.normal(0.0, 0.3, 3)
        self.init_R, self.init_t = perturb(self.gt_R, self.gt_t, rng, trans_m, rot_deg)
        self.init_lin = self.gt_lin + rng.normal(0.0, 0.1, 3)
        self.init_ang = self.gt_ang + rng.normal(0.0, 0.1, 3)
        self.n_events = int(n_events)

    def gt_pair(self):
        return P.pair_poses(self.gt_R, self.gt_t, self.gt_lin, self.gt_ang, self.delta_tau)


def perturb(R, t, rng, trans_m, rot_deg):
    d = rng.normal(size=3)
    d *= trans_m / np.linalg.norm(d)
    a = rng.normal(size=3)
    a *= math.radians(rot_deg) / np.linalg.norm(a)
    T = P.exp_se3(np.concatenate([d, a])) @ P.matrix(R, t)
    return T[:3, :3], T[:3, 3]


def hypotheses(R, t, count, seed, max_trans=0.2, max_rot_deg=10.0):
    """`count` pose hypotheses perturbed by 0..max_trans m and 0..max_rot_deg degrees."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        f = i / max(count - 1, 1)
        out.append(perturb(R, t, rng, max(f * max_trans, 1e-6), max(f * max_rot_deg, 1e-6)))
    return out


def synth_events(I_last, I_next, n_events, seed, contrast=0.2, noise_frac=0.05, delta_tau=0.01, eps=1e-3):
    """Event window from two grey renders ([H, W] arrays).  Returns x, y (uint16),
    polarity (uint8, 1 = positive), ts (int64 microseconds, sorted)."""
    rng = np.random.default_rng(seed)
    H, W = I_last.shape
    dl = np.log(np.asarray(I_next, np.float64) + eps) - np.log(np.asarray(I_last, np.float64) + eps)
    lam = np.abs(dl).reshape(-1) / contrast
    n_noise = int(round(n_events * noise_frac))
    n_sig = n_events - n_noise
    tot = lam.sum()
    if tot <= 0:
        counts = np.zeros(H * W, np.int64)
        n_noise = n_events
    else:
        counts = rng.multinomial(n_sig, lam / tot)
    idx = np.repeat(np.arange(H * W), counts)
    pol = (dl.reshape(-1)[idx] > 0).astype(np.uint8)
    nidx = rng.integers(0, H * W, size=n_noise)
    npol = rng.integers(0, 2, size=n_noise).astype(np.uint8)
    idx = np.concatenate([idx, nidx])
    pol = np.concatenate([pol, npol])
    ts = np.sort(rng.integers(0, int(delta_tau * 1e6) + 1, size=idx.shape[0])).astype(np.int64)
    perm = rng.permutation(idx.shape[0])
    idx, pol = idx[perm], pol[perm]
    return (idx % W).astype(np.uint16), (idx // W).astype(np.uint16), pol, ts


class SinusoidTrajectory:
    """Ground-truth motion of one synthetic sequence: T(tau) = exp(sin(2 pi f tau) zeta) with
    zeta = [a_t u, a_r k] for unit axes u (translation) and k (rotation) drawn from the
    seed, a_t = 0.5 m and a_r = 20 degrees at f = 0.2 Hz by default (world -> camera poses,
    identity at tau = 0).  The path is a one-parameter subgroup, so the left twist rate
    that the tracker's velocity model uses (T(tau + h) = exp(h [v, w]) T(tau)) is exactly
    2 pi f cos(2 pi f tau) zeta."""

    def __init__(self, seed, amp_m=0.5, amp_deg=20.0, freq_hz=0.2):
        rng = np.random.default_rng(seed)
        u = rng.normal(size=3)
        k = rng.normal(size=3)
        self.zeta = np.concatenate([amp_m * u / np.linalg.norm(u), math.radians(amp_deg) * k / np.linalg.norm(k)])
        self.omega = 2.0 * math.pi * freq_hz

    def pose(self, tau):
        T = P.exp_se3(math.sin(self.omega * tau) * self.zeta)
        return T[:3, :3].copy(), T[:3, 3].copy()

    def velocity(self, tau):
        """(linear, angular) twist rate at tau, in the tracker's convention."""
        xi = self.omega * math.cos(self.omega * tau) * self.zeta
        return xi[:3].copy(), xi[3:].copy()


def synth_events_device(I_last, I_next, n_events, generator, contrast=0.2, noise_frac=0.05, eps=1e-3):
    """Device form of synth_events for [H, W] torch images (same model: signal events
    distributed over pixels in proportion to |ln(I_next + eps) - ln(I_last + eps)| / C,
    polarity its sign, plus uniform noise events of random polarity), drawn with a torch
    generator on the images' device.  Returns x, y (uint16 tensors) and polarity (uint8
    tensor); event order is irrelevant to the event frame."""
    import torch
    H, W = I_last.shape
    dl = (torch.log(I_next.double() + eps) - torch.log(I_last.double() + eps)).reshape(-1)
    lam = dl.abs() / contrast
    n_noise = int(round(n_events * noise_frac))
    n_sig = n_events - n_noise
    dev = I_last.device
    if float(lam.sum()) > 0 and n_sig > 0:
        idx = torch.multinomial(lam.float(), n_sig, replacement=True, generator=generator)
        pol = (dl[idx] > 0).to(torch.uint8)
    else:
        idx = torch.zeros(0, dtype=torch.int64, device=dev)
        pol = torch.zeros(0, dtype=torch.uint8, device=dev)
        n_noise = n_events
    nidx = torch.randint(0, H * W, (n_noise,), generator=generator, device=dev)
    npol = torch.randint(0, 2, (n_noise,), generator=generator, device=dev).to(torch.uint8)
    idx = torch.cat([idx, nidx])
    pol = torch.cat([pol, npol])
    # coordinates below 2^15: the int16 bits are the uint16 values
    return (idx % W).to(torch.int16).view(torch.uint16), (idx // W).to(torch.int16).view(torch.uint16), pol
