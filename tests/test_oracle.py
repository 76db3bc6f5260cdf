"""CPU tests of the oracle: pinned against fixtures generated from the reference's own
Python (tests/golden/make_golden.py), plus self-consistency checks (exp error bound,
SE(3) Jacobians, FP64 analytic gradient vs central finite differences, sort stability,
event frame)."""
import math
import os

import numpy as np
import pytest

from oracle import oracle
from oracle import pose as opose
from gsevt import pose as gpose
from gsevt import synthetic
import helpers

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.npz"))


# ----------------------------------------------------------------------- exp --
def test_exp2f_error_bound():
    ys = np.linspace(-126.0, 0.0, 40001).astype(np.float32)
    ys = np.concatenate([ys, np.float32([-8.0, -8.5, -7.5, -1e-7, -0.0, -0.5, -1.5, -0.4999999, -125.9])])
    got = np.array([oracle.exp2f(y) for y in ys], np.float64)
    ref = np.exp2(ys.astype(np.float64))
    ulp = np.abs(got - ref) / np.spacing(np.float32(ref).astype(np.float32)).astype(np.float64)
    assert ulp.max() <= 1.0, ulp.max()
    # below the range (and NaN) the argument is raised to -126
    tiny = np.float32(2.0 ** -126)
    assert oracle.exp2f(-126.5) == tiny and oracle.exp2f(-1e30) == tiny and oracle.exp2f(float("nan")) == tiny
    # integers are exact
    assert all(oracle.exp2f(float(-k)) == np.float32(2.0 ** -k) for k in range(0, 126))


_EXP2_PROBE = r"""
#include <omp.h>
#include "common.cuh"
extern "C" long long exp2_mismatches(float (*ref)(float), unsigned long long lo, unsigned long long hi)
{
    long long bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static, 1 << 16)
    for (long long b = (long long)lo; b <= (long long)hi; ++b) {
        const float y = gs_bits_float((uint32_t)b);
        bad += gs_float_bits(gs_exp2f(y)) != gs_float_bits(ref(y));
    }
    return bad;
}
extern "C" float exp2_one(float y) { return gs_exp2f(y); }
"""


def test_kernel_exp2f_equals_the_oracle_on_every_float(tmp_path):
    """The kernels' 2^y (gs_exp2f in csrc/common.cuh: rint(y) by the 1.5 2^23 addition and
    the scale as an exponent-field addition) against the oracle's or_exp2f (rintf and a
    multiply by 2^k) on every float in [-126, 0] and on the clamped arguments below it.
    The same source is compiled for the host here; the blend parity tests on the GPU then
    tie the device instance to the oracle's images bit for bit."""
    import ctypes
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src, so = tmp_path / "exp2_probe.cu", tmp_path / "exp2_probe.so"
    src.write_text(_EXP2_PROBE)
    cmd = [nvcc, "-shared", "-O2", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-fopenmp",
           "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(root, "include"), "-I", os.path.join(root, "gs-evt_gb300", "csrc"),
           str(src), "-o", str(so), "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    probe = ctypes.CDLL(str(so))
    probe.exp2_mismatches.restype = ctypes.c_longlong
    probe.exp2_mismatches.argtypes = [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_ulonglong]
    probe.exp2_one.restype = ctypes.c_float
    probe.exp2_one.argtypes = [ctypes.c_float]
    ref = ctypes.cast(oracle.lib().or_exp2f_export, ctypes.c_void_p)
    # -0.0 (0x80000000) up to -126.0 (0xC2FC0000): every float of the blends' range
    assert probe.exp2_mismatches(ref, 0x80000000, 0xC2FC0000) == 0
    assert probe.exp2_mismatches(ref, 0x00000000, 0x00000000) == 0  # +0.0
    for y in (-126.00001, -126.5, -127.0, -1e30, float("-inf"), float("nan")):
        assert probe.exp2_one(y) == np.float32(2.0 ** -126) == oracle.exp2f(y)


# ------------------------------------------------------------- pose golden --
@pytest.mark.parametrize("mod", [opose, "product"])
def test_pose_algebra_golden(mod):
    exp_so3 = opose.so3_exp if mod is opose else gpose.exp_so3
    jl = opose.so3_left_jacobian if mod is opose else gpose.left_jacobian_so3
    exp_se3 = opose.se3_exp if mod is opose else gpose.exp_se3
    log = opose.so3_log if mod is opose else gpose.so3_log
    for th, R, V in zip(GOLD["so3_theta"], GOLD["so3_exp"], GOLD["v_mat"]):
        np.testing.assert_allclose(exp_so3(th), R, atol=1e-14)
        np.testing.assert_allclose(jl(th), V, atol=1e-14)
    for xi, T in zip(GOLD["se3_xi"], GOLD["se3_exp"]):
        np.testing.assert_allclose(exp_se3(xi), T, atol=1e-13)
    for R, w in zip(GOLD["log_R"], GOLD["log_out"]):
        np.testing.assert_allclose(log(R), w, atol=2e-6)


def test_camera_golden():
    R, t = GOLD["cam_R"].astype(np.float64), GOLD["cam_t"].astype(np.float64)
    W, H, fx, fy, dtau = GOLD["cam_size_focal"]
    fovx, fovy = opose.focal2fov(fx, W), opose.focal2fov(fy, H)
    P = opose.projection_matrix(fovx, fovy)
    np.testing.assert_allclose(opose.pose_matrix(R, t).T, GOLD["cam_world_view"], atol=1e-6)
    np.testing.assert_allclose(P.T, GOLD["cam_proj"], atol=1e-6)
    np.testing.assert_allclose((P @ opose.pose_matrix(R, t)).T, GOLD["cam_full_proj"], atol=1e-5)
    np.testing.assert_allclose(opose.camera_center(R, t), GOLD["cam_center"], atol=1e-6)
    lin, ang = GOLD["cam_lin"], GOLD["cam_ang"]
    El, En = opose.vel_transforms(lin, ang, dtau)
    np.testing.assert_allclose(El, GOLD["cam_last_vel"], atol=1e-7)
    np.testing.assert_allclose(En, GOLD["cam_next_vel"], atol=1e-7)
    for lvl in (0, 1, 2):
        Tl, Tn = opose.pair_poses(R, t, lin, ang, dtau)
        s = 0.5 ** lvl
        w, h = int(W * s), int(H * s)
        for nm, T in (("last", Tl), ("next", Tn)):
            np.testing.assert_allclose(T[:3, :3], GOLD["pair_%s_l%d_R" % (nm, lvl)], atol=1e-6)
            np.testing.assert_allclose(T[:3, 3], GOLD["pair_%s_l%d_t" % (nm, lvl)], atol=1e-6)
            np.testing.assert_allclose([w, h, opose.focal2fov(fx * s, w), opose.focal2fov(fy * s, h)],
                                       GOLD["pair_%s_l%d_size_fov" % (nm, lvl)], rtol=1e-12)
        # the product's pair poses agree too
        Pl, Pn = gpose.pair_poses(R, t, lin, ang, dtau)
        np.testing.assert_allclose(Pl, Tl, atol=1e-14)
        np.testing.assert_allclose(Pn, Tn, atol=1e-14)


def test_pose_updates_golden():
    R, t = GOLD["cam_R"].astype(np.float64), GOLD["cam_t"].astype(np.float64)
    d = GOLD["upd_deltas"].astype(np.float64)
    rot, trans, w, v = d[0:3], d[3:6], d[6:9], d[9:12]
    ang = GOLD["cam_ang"] + w
    lin = GOLD["cam_lin"] + v
    R2, t2 = opose.update_pose(R, t, trans, rot)
    np.testing.assert_allclose(R2, GOLD["upd_R"], atol=2e-6)
    np.testing.assert_allclose(t2, GOLD["upd_t"], atol=2e-6)
    np.testing.assert_allclose(ang, GOLD["upd_ang"], atol=1e-7)
    np.testing.assert_allclose(lin, GOLD["upd_lin"], atol=1e-7)
    R3, t3 = opose.const_vel_model(GOLD["upd_R"].astype(np.float64), GOLD["upd_t"].astype(np.float64),
                                   GOLD["upd_lin"], GOLD["upd_ang"], float(GOLD["cvm_tau"]))
    np.testing.assert_allclose(R3, GOLD["cvm_R"], atol=2e-6)
    np.testing.assert_allclose(t3, GOLD["cvm_t"], atol=2e-6)
    lv, av = opose.cal_weighted_velocity(GOLD["cvm_R"].astype(np.float64), GOLD["cvm_t"].astype(np.float64),
                                         GOLD["upd_R"].astype(np.float64), GOLD["upd_t"].astype(np.float64),
                                         GOLD["upd_lin"], GOLD["upd_ang"], float(GOLD["cvm_tau"]), 0.5)
    np.testing.assert_allclose(lv, GOLD["cwv_lin"], atol=2e-4)
    np.testing.assert_allclose(av, GOLD["cwv_ang"], atol=2e-4)


def test_sh_golden():
    for deg in range(4):
        got = oracle.sh_eval(GOLD["sh_coeffs"], GOLD["sh_dirs"], deg)
        np.testing.assert_allclose(got, GOLD["sh_out_deg%d" % deg], rtol=1e-12, atol=1e-12)


def test_cov3d_golden():
    got = oracle.cov3d(GOLD["cov_scale"], GOLD["cov_rot"])
    ref = GOLD["cov_out"]
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.max(np.abs(got - ref) / scale) < 2e-6


def test_grey_normalisation_loss_golden():
    w = np.float32([0.2989, 0.5870, 0.1140])
    for nm in ("last", "next"):
        c = GOLD["dIr_color_" + nm]
        np.testing.assert_allclose((c * w[:, None, None]).sum(0), GOLD["dIr_grey_" + nm][0], atol=1e-6)
    gl, gn = GOLD["dIr_grey_last"][0], GOLD["dIr_grey_next"][0]
    d = gn.astype(np.float64) - gl
    np.testing.assert_allclose(d / np.linalg.norm(d), GOLD["dIr_signed"][0], atol=1e-6)
    np.testing.assert_allclose(np.abs(d / np.linalg.norm(d)), GOLD["dIr_unsigned"][0], atol=1e-6)
    E = GOLD["loss_E"][0]
    assert abs(oracle.loss(gl, gn, E, False) - float(GOLD["loss_signed"])) < 1e-5
    assert abs(oracle.loss(gl, gn, np.abs(E), True) - float(GOLD["loss_unsigned"])) < 1e-5


@pytest.mark.parametrize("unsigned", [False, True])
def test_log_grey_loss_and_image_gradients(unsigned):
    """Log-intensity mode of the pair loss (dI = ln(I_next + eps) - ln(I_last + eps)): the C
    oracle equals the numpy FP64 form, and its image gradients (which carry 1 / (I + eps))
    match central finite differences; eps -> 0 is not taken, and without log_eps the
    linear form is unchanged."""
    rng = np.random.default_rng(9)
    H, W, eps = 12, 16, 1e-3
    Il = rng.uniform(0.0, 1.0, (H, W)).astype(np.float32)
    In = (Il + rng.normal(0.0, 0.05, (H, W))).clip(0.0, None).astype(np.float32)
    E = rng.normal(size=(H, W)).astype(np.float32)
    E /= np.linalg.norm(E.astype(np.float64))
    if unsigned:
        E = np.abs(E)
    L, gn, gl = oracle.loss(Il, In, E, unsigned, grads=True, log_eps=eps)
    assert abs(L - oracle.loss_f64(Il, In, E, unsigned, log_eps=eps)) < 1e-12
    assert abs(oracle.loss(Il, In, E, unsigned) - oracle.loss_f64(Il, In, E, unsigned)) < 1e-12
    assert abs(L - oracle.loss(Il, In, E, unsigned)) > 1e-3  # the two modes differ
    h = 1e-7
    for k in rng.choice(H * W, 12, replace=False):
        for img, g in ((In, gn), (Il, gl)):
            a = img.astype(np.float64).copy()
            b = a.copy()
            a.reshape(-1)[k] += h
            b.reshape(-1)[k] -= h
            args = (a, In.astype(np.float64)) if img is Il else (Il.astype(np.float64), a)
            argsb = (b, In.astype(np.float64)) if img is Il else (Il.astype(np.float64), b)
            fd = (oracle.loss_f64(*args, E, unsigned, log_eps=eps) - oracle.loss_f64(*argsb, E, unsigned,
                                                                                      log_eps=eps)) / (2 * h)
            assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, g[k])


def test_convergence_golden():
    from gsevt.tracker import check_convergence
    L = list(GOLD["conv_losses"])
    assert [check_convergence(L[:k], 1e-3) for k in range(1, 31)] == list(GOLD["conv_results"])
    F = list(GOLD["conv_flat"])
    assert [check_convergence(F[:k], 1e-4) for k in range(1, 16)] == list(GOLD["conv_flat_results"])


# ---------------------------------------------------------------- SE(3) -----
def test_se3_left_jacobian_and_adjoint():
    rng = np.random.default_rng(3)
    for s in (1e-6, 1e-2, 0.5, 2.0):
        x = rng.normal(size=6) * s
        J = opose.se3_left_jacobian(x)
        for k in range(6):
            e = np.zeros(6)
            e[k] = 1e-6
            A = opose.se3_exp(x + e) @ np.linalg.inv(opose.se3_exp(x))
            B = opose.se3_exp(-x + 0 * e)
            num = (A - np.eye(4)) / 1e-6
            col = np.array([num[0, 3], num[1, 3], num[2, 3], num[2, 1], num[0, 2], num[1, 0]])
            np.testing.assert_allclose(col, J[:, k], atol=2e-5)
        T = opose.se3_exp(rng.normal(size=6))
        xi = rng.normal(size=6) * 1e-3
        np.testing.assert_allclose(T @ opose.se3_exp(xi) @ np.linalg.inv(T),
                                   opose.se3_exp(opose.se3_adjoint(T) @ xi), atol=1e-12)


# ----------------------------------------------------- FP64 gradient vs FD --
def _frozen_case(n=400, W=48, H=32, f=40.0, seed=5, nch=1):
    m, cam = helpers.scene(n, W, H, f, seed)
    R, t = helpers.random_pose(seed)
    cov = helpers.cov6(m)
    v32 = helpers.view_vector(R, t, cam)
    res = oracle.rasterize_view(m["xyz"], cov, m["sh"], m["opacity"], v32, W, H, [0.0] * nch, nch=nch,
                                record=True)
    return m, cam, R, t, res


def test_frozen_render_matches_fp32():
    m, cam, R, t, res = _frozen_case(nch=3)
    v64 = helpers.view_vector(R, t, cam, np.float64)
    out, D, A = oracle.frozen_render(res, m["xyz"], m["opacity"], v64, cam.width, cam.height, [0, 0, 0], 3,
                                     sh=m["sh"], scale=m["scale"], rot=m["rot"])
    np.testing.assert_allclose(out, res["image"], atol=2e-5)
    np.testing.assert_allclose(D, res["depth"], atol=2e-4)
    np.testing.assert_allclose(A, res["alpha"], atol=2e-5)


def test_frozen_pose_gradient_fd():
    m, cam, R, t, res = _frozen_case()
    W, H = cam.width, cam.height
    rng = np.random.default_rng(0)
    wimg = rng.normal(size=(1, H, W))

    def L(Rv, tv):
        v = helpers.view_vector(Rv, tv, cam, np.float64)
        out, _, _ = oracle.frozen_render(res, m["xyz"], m["opacity"], v, W, H, [0.0], 1, sh=m["sh"],
                                         scale=m["scale"], rot=m["rot"])
        return float((out * wimg).sum())

    v = helpers.view_vector(R, t, cam, np.float64)
    g, _ = oracle.frozen_backward(res, m["xyz"], m["opacity"], v, W, H, [0.0], 1, wimg, sh=m["sh"],
                                  scale=m["scale"], rot=m["rot"])
    T = opose.pose_matrix(R, t)
    h = 1e-6
    fd = np.zeros(6)
    for k in range(6):
        e = np.zeros(6)
        e[k] = h
        Tp, Tm = opose.se3_exp(e) @ T, opose.se3_exp(-e) @ T
        fd[k] = (L(Tp[:3, :3], Tp[:3, 3]) - L(Tm[:3, :3], Tm[:3, 3])) / (2 * h)
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-9 * np.abs(fd).max())


def test_frozen_map_gradients_fd():
    m, cam, R, t, res = _frozen_case(n=200)
    W, H = cam.width, cam.height
    rng = np.random.default_rng(1)
    wimg = rng.normal(size=(3, H, W))
    wd, wa = rng.normal(size=(H, W)), rng.normal(size=(H, W))
    v = helpers.view_vector(R, t, cam, np.float64)
    res3 = oracle.rasterize_view(m["xyz"], helpers.cov6(m), m["sh"], m["opacity"], helpers.view_vector(R, t, cam),
                                 W, H, [0.1, 0.2, 0.3], nch=3, record=True)

    def L(mm):
        out, D, A = oracle.frozen_render(res3, mm["xyz"], mm["opacity"], v, W, H, [0.1, 0.2, 0.3], 3,
                                         sh=mm["sh"], scale=mm["scale"], rot=mm["rot"])
        return float((out * wimg).sum() + (D * wd).sum() + (A * wa).sum())

    _, mg = oracle.frozen_backward(res3, m["xyz"], m["opacity"], v, W, H, [0.1, 0.2, 0.3], 3, wimg, sh=m["sh"],
                                   scale=m["scale"], rot=m["rot"], dL_ddepth=wd, dL_dalpha=wa, map_grads=True)
    touched = np.nonzero(res3["pre"]["touched"])[0][:12]
    h = 1e-4
    for name, key, shape in (("xyz", "means3d", 3), ("opacity", "opac", 1), ("scale", "scale", 3),
                             ("rot", "rot", 4), ("sh", "sh", 48)):
        for gi in touched[:4]:
            for c in range(min(shape, 4)):
                mp = {k: v_.astype(np.float64).copy() for k, v_ in m.items()}
                mm = {k: v_.astype(np.float64).copy() for k, v_ in m.items()}
                idx = (gi,) if shape == 1 else (gi, c) if name != "sh" else (gi, c // 3, c % 3)
                base = float(m[name][idx])
                step = h * max(abs(base), 1e-2)
                # the oracle reads float32 maps: perturb to exactly representable values
                xp, xm = float(np.float32(base + step)), float(np.float32(base - step))
                mp[name][idx] = xp
                mm[name][idx] = xm
                fd = (L(mp) - L(mm)) / (xp - xm)
                an = mg[key][gi] if shape == 1 else mg[key][gi, c]
                assert abs(an - fd) <= 1e-4 * abs(fd) + 1e-6, (name, gi, c, an, fd)


def test_pair_chain_fd():
    """Chain from per-view twist gradients to (theta, rho, w, v) against FD on the pose
    and velocity deltas of utils/render_camera/camera.py."""
    rng = np.random.default_rng(2)
    R, t = helpers.random_pose(7)
    lin, ang, dtau = rng.normal(size=3), rng.normal(size=3), 0.05
    gl, gn = rng.normal(size=6), rng.normal(size=6)

    def L(d):
        Tl, Tn = opose.tracked_pair_poses(R, t, lin, ang, dtau, d[3:6], d[0:3], d[9:12], d[6:9])
        T0l, T0n = opose.pair_poses(R, t, lin, ang, dtau)
        # linear functional of the left twists of the two rendered views
        xl = _log_se3(Tl @ np.linalg.inv(T0l))
        xn = _log_se3(Tn @ np.linalg.inv(T0n))
        return gl @ xl + gn @ xn

    th, rh, w, v = opose.chain_pose_gradient(gl, gn, lin, ang, dtau)
    an = np.concatenate([th, rh, w, v])
    fd = np.zeros(12)
    for k in range(12):
        e = np.zeros(12)
        e[k] = 1e-6
        fd[k] = (L(e) - L(-e)) / 2e-6
    np.testing.assert_allclose(an, fd, rtol=1e-6, atol=1e-8)


def _log_se3(T):
    # rotation vector without the reference's 1e-5 cut-off, so tiny FD steps survive
    R = T[:3, :3]
    a = math.acos(min(1.0, max(-1.0, (np.trace(R) - 1.0) / 2.0)))
    v = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2.0
    w = v * (a / math.sin(a) if a > 1e-4 else 1.0 + a * a / 6.0)
    V = opose.so3_left_jacobian(w)
    return np.concatenate([np.linalg.solve(V, T[:3, 3]), w])


# --------------------------------------------------------- sort and events --
def test_sort_stable_and_ranges():
    rng = np.random.default_rng(0)
    keys = (rng.integers(0, 50, 5000).astype(np.uint64) << np.uint64(32)) | rng.integers(0, 4, 5000).astype(np.uint64)
    vals = np.arange(5000, dtype=np.uint32)
    k2, v2 = oracle.sort_pairs(keys, vals, 40)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k2, keys[order]) and np.array_equal(v2, vals[order])
    r = oracle.ranges(k2, 64)
    for tile in range(64):
        sel = np.nonzero((k2 >> np.uint64(32)) == tile)[0]
        if sel.size:
            assert r[tile, 0] == sel[0] and r[tile, 1] == sel[-1] + 1
        else:
            assert r[tile, 0] == 0 and r[tile, 1] == 0


def test_event_frame_oracle():
    rng = np.random.default_rng(0)
    W, H = 40, 30
    n = 3000
    x = rng.integers(0, W, n).astype(np.uint16)
    y = rng.integers(0, H, n).astype(np.uint16)
    p = rng.integers(0, 2, n).astype(np.uint8)
    s, u, c = oracle.event_frame(W, H, x, y, p, 9)
    ref = np.zeros((H, W), np.int32)
    np.add.at(ref, (y.astype(int), x.astype(int)), np.where(p > 0, 1, -1))
    assert np.array_equal(c, ref)
    sigma = 0.3 * ((9 - 1) * 0.5 - 1) + 0.8
    k = np.exp(-((np.arange(9) - 4.0) ** 2) / (2 * sigma ** 2))
    k /= k.sum()
    pad = np.pad(ref.astype(np.float64), 4, mode="edge")
    tmp = sum(k[j] * pad[:, j:j + W] for j in range(9))
    blur = sum(k[j] * tmp[j:j + H, :] for j in range(9))
    np.testing.assert_allclose(s, blur / np.linalg.norm(blur), atol=1e-7)
    np.testing.assert_allclose(u, np.abs(s))
    assert abs(np.linalg.norm(s.astype(np.float64)) - 1.0) < 1e-6
    z, _, _ = oracle.event_frame(W, H, x[:0], y[:0], p[:0], 9)
    assert not z.any()


def test_pyramid_nearest():
    img = np.arange(480 * 640, dtype=np.float32).reshape(480, 640)
    lv = oracle.pyramid(img, 3)
    assert [a.shape for a in lv] == [(480, 640), (240, 320), (120, 160)]
    assert np.array_equal(lv[1], img[::2, ::2]) and np.array_equal(lv[2], img[::4, ::4])
    odd = np.arange(260 * 346, dtype=np.float32).reshape(260, 346)
    l2 = oracle.pyramid(odd, 3)[2]
    assert l2.shape == (65, 86)
    assert l2[0, 85] == odd[0, int(np.floor(85 * 346 / 86))]


def test_synthetic_events_counts():
    rng = np.random.default_rng(0)
    a = rng.uniform(0.2, 1.0, (24, 32))
    b = a * np.exp(rng.normal(0, 0.2, a.shape))
    x, y, p, ts = synthetic.synth_events(a, b, 3000, 1)
    assert x.shape[0] == 3000 and ts.shape[0] == 3000 and np.all(np.diff(ts) >= 0)
    assert x.max() < 32 and y.max() < 24


def test_undistort_oracle():
    """Zero distortion is the identity; otherwise the result equals an independent numpy
    evaluation of the same OpenCV model (FP64 map, 1/32-pixel rounding, bilinear, zero
    border)."""
    rng = np.random.default_rng(4)
    W, H = 64, 48
    img = rng.normal(size=(H, W)).astype(np.float32)
    cam0 = (60.0, 61.0, 31.5, 23.2, 0.0, 0.0, 0.0, 0.0, 0.0)
    assert np.array_equal(oracle.undistort(img, cam0), img)
    cam = (60.0, 61.0, 31.5, 23.2, -0.031982, 0.041966, -0.000507, -0.001031, 0.0)  # desk_normal1 factors
    got = oracle.undistort(img, cam)
    fx, fy, cx, cy, k1, k2, p1, p2, k3 = cam
    v, u = np.mgrid[0:H, 0:W].astype(np.float64)
    x, y = (u - cx) / fx, (v - cy) / fy
    r2 = x * x + y * y
    kr = 1 + ((k3 * r2 + k2) * r2 + k1) * r2
    xd = x * kr + p1 * 2 * x * y + p2 * (r2 + 2 * x * x)
    yd = y * kr + p1 * (r2 + 2 * y * y) + p2 * 2 * x * y
    iu = np.rint((fx * xd + cx) * 32).astype(np.int64)
    iv = np.rint((fy * yd + cy) * 32).astype(np.int64)
    ix, iy = iu >> 5, iv >> 5
    ax, ay = (iu & 31) / 32.0, (iv & 31) / 32.0
    ref = np.zeros((H, W))
    for dy in (0, 1):
        for dx in (0, 1):
            sx, sy = ix + dx, iy + dy
            ok = (sx >= 0) & (sy >= 0) & (sx < W) & (sy < H)
            w = (ax if dx else 1 - ax) * (ay if dy else 1 - ay)
            ref[ok] += w[ok] * img[sy[ok], sx[ok]]
    np.testing.assert_allclose(got, ref, atol=1e-5)
    assert not np.array_equal(got, img)
