"""Shared test helpers: small seeded scenes, oracle view vectors and workspace access."""
import math

import numpy as np

from gsevt import synthetic
from gsevt import pose as gpose


def scene(n=2000, W=96, H=64, f=80.0, seed=0):
    m = synthetic.make_map(n, seed)
    cam = synthetic.PinholeCamera(W, H, f)
    return m, cam


def random_pose(seed, trans=0.05, rot_deg=3.0):
    rng = np.random.default_rng(seed)
    return synthetic.perturb(np.eye(3), np.zeros(3), rng, trans, rot_deg)


def view_vector(R, t, cam, dtype=np.float32):
    """Oracle view layout: R[9] t[3] Praw[16] campos[3] tanfx tanfy (the first 33 floats of
    gsevt_view)."""
    v = np.concatenate([np.asarray(R, np.float64).reshape(9), np.asarray(t, np.float64).reshape(3),
                        cam.proj.reshape(16), gpose.campos(R, t), [cam.tanfovx, cam.tanfovy]])
    return v.astype(dtype)


def cov6(m):
    from oracle import oracle
    return oracle.cov3d(m["scale"], m["rot"])


def grey_bg(bg):
    bg = np.asarray(bg, np.float32)
    return np.array([np.float32(np.float32(0.2989) * bg[0] + np.float32(0.587) * bg[1]) + np.float32(0.114) * bg[2]],
                    np.float32)


def pair_views(R, t, lin, ang, dtau):
    Tl, Tn = gpose.pair_poses(R, t, lin, ang, dtau)
    return (Tl[:3, :3], Tl[:3, 3]), (Tn[:3, :3], Tn[:3, 3])


def oracle_pair_loss_f64(m, cam, R, t, lin, ang, dtau, E, recs, unsigned=False, cov=None, log_eps=None):
    """FP64 frozen pair loss for pose (R, t) and velocity (lin, ang)."""
    from oracle import oracle
    (Rl, tl), (Rn, tn) = pair_views(R, t, lin, ang, dtau)
    imgs = []
    for (Rv, tv), rec in zip(((Rl, tl), (Rn, tn)), recs):
        v = view_vector(Rv, tv, cam, np.float64)
        out, _, _ = oracle.frozen_render(rec, m["xyz"], m["opacity"], v, cam.width, cam.height, [0.0], 1,
                                         sh=m["sh"], cov_pre=cov, scale=None if cov is not None else m["scale"],
                                         rot=None if cov is not None else m["rot"])
        imgs.append(out[0])
    return oracle.loss_f64(imgs[0], imgs[1], E, unsigned, log_eps=log_eps)
