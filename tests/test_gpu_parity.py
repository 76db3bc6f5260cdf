"""GPU parity: the CUDA path through the C ABI against the CPU oracle on the same seeded
inputs.  Integer and index outputs (radii, tile rects, duplicated keys, sort order,
tile ranges, contributor counts) must be bit-exact; images are compared bit-exactly
as well (same operation order, same deterministic exp), and gradients against the
oracle's FP64 analytic gradient (itself checked against central finite differences
on the CPU) within the tolerances stated in each test."""
import ctypes as C
import math

import numpy as np
import pytest
import torch

from oracle import oracle
from oracle import pose as opose
from gsevt import _lib
from gsevt import pose as gpose
from gsevt.engine import GSFrame, MapSpec, ViewSpec
import helpers

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda")
IMG_ATOL, IMG_RTOL = 1e-5, 1e-4   # images (FP32): the parity tolerance for floating-point images
GRAD_RTOL = 1e-4                   # pose / velocity gradients (norm-relative)


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def _region(frame, name, dtype, count):
    off = _lib.workspace_offsets(frame.L)[name]
    nbytes = count * torch.empty((), dtype=dtype).element_size()
    return frame.workspace[off:off + nbytes].view(dtype)


def _map_spec(m, packed=False):
    n = m["xyz"].shape[0]
    if packed:
        from gsevt.engine import pack_map
        pk = pack_map(_t(m["xyz"]), _t(m["opacity"]), _t(m["sh"]), scales=_t(m["scale"]), rotations=_t(m["rot"]))
        return MapSpec(n, packed=pk), pk
    return MapSpec(n, xyz=_t(m["xyz"]), opacity=_t(m["opacity"]), scales=_t(m["scale"]), rotations=_t(m["rot"]),
                   shs=_t(m["sh"])), None


def _view(R, t, cam, map_index=0, bg=(0.0, 0.0, 0.0), pair=-1, role=0):
    return ViewSpec(cam.width, cam.height, map_index, bg=bg, R=R, t=t, P=cam.proj, campos=gpose.campos(R, t),
                    tanfovx=cam.tanfovx, tanfovy=cam.tanfovy, pair=pair, pair_role=role)


def _bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.uint32)
    b = np.ascontiguousarray(b, np.float32).view(np.uint32)
    return np.array_equal(a, b)


@pytest.fixture(scope="module")
def small():
    m, cam = helpers.scene(20000, 320, 240, 300.0, seed=0)
    R, t = helpers.random_pose(11)
    return m, cam, R, t


@pytest.mark.parametrize("packed", [False, True])
def test_single_view_bit_exact(small, packed):
    m, cam, R, t = small
    W, H = cam.width, cam.height
    n = m["xyz"].shape[0]
    ms, keep = _map_spec(m, packed)
    bg = (0.1, 0.2, 0.3)
    fr = GSFrame([ms], [_view(R, t, cam, bg=bg)], channels=3, want_depth=True, want_alpha=True, want_radii=True,
                 want_n_touched=True, want_n_contrib=True, device=DEV)
    fr.render(exact_keys=True)
    torch.cuda.synchronize()
    res = oracle.rasterize_view(m["xyz"], helpers.cov6(m), m["sh"], m["opacity"], helpers.view_vector(R, t, cam),
                                W, H, list(bg), nch=3)
    pre = res["pre"]
    vis = pre["touched"] > 0
    assert vis.sum() > 1000
    # preprocess: radii, tile rects, means, depths, conics, colours
    assert np.array_equal(fr.radii[:n].cpu().numpy(), pre["radii"])
    binv = _region(fr, "bin", torch.int32, 4 * n).view(n, 4).cpu().numpy()
    assert np.array_equal(binv[:, 0], pre["touched"])
    rect = pre["rect"][vis]
    assert np.array_equal(binv[vis, 1] & 0xffff, rect[:, 0]) and np.array_equal(binv[vis, 2] >> 16, rect[:, 3])
    rec = _region(fr, "recA", torch.float32, 8 * n).view(n, 8).cpu().numpy()  # 32-byte records
    A, B = rec[vis, :4], rec[vis, 4:]
    Cc = _region(fr, "recC", torch.float32, 4 * n).view(n, 4).cpu().numpy()[vis]
    assert _bits_equal(A[:, :2], pre["mean2d"][vis]) and _bits_equal(A[:, 2], pre["depth"][vis])
    assert _bits_equal(A[:, 3], pre["grey"][vis])
    assert _bits_equal(B[:, :3], pre["conic"][vis]) and _bits_equal(Cc[:, :3], pre["rgb"][vis])
    # keys, sort order, ranges
    K = fr.num_keys
    assert K == res["keys"].shape[0]
    buf = ((fr.L.sort_bits - 32 + 7) // 8) & 1
    tiles = _region(fr, "keys%d" % buf, torch.int32, K).cpu().numpy().view(np.uint32)
    vals = _region(fr, "vals%d" % buf, torch.int32, K).cpu().numpy().view(np.uint32)
    # same order as the stable sort of the full (tile | depth) keys, ties included
    assert np.array_equal(tiles, (res["keys"] >> np.uint64(32)).astype(np.uint32))
    assert np.array_equal(vals, res["vals"])
    rng = _region(fr, "ranges", torch.int32, 2 * fr.L.total_tiles).view(-1, 2).cpu().numpy().view(np.uint32)
    assert np.array_equal(rng, res["ranges"])
    # blend outputs
    img = fr.image.view(3, H, W).cpu().numpy()
    assert _bits_equal(img, res["image"])
    assert _bits_equal(fr.final_T.view(H, W).cpu().numpy(), res["final_T"])
    assert _bits_equal(fr.depth.view(H, W).cpu().numpy(), res["depth"])
    assert _bits_equal(fr.alpha.view(H, W).cpu().numpy(), res["alpha"])
    assert np.array_equal(fr.n_contrib.view(H, W).cpu().numpy(), res["n_contrib"])
    assert np.array_equal(fr.n_touched[:n].cpu().numpy(), res["n_touched"])


def test_multi_view_multi_map(small):
    """Views of different sizes and two maps in one frame: every view matches its own
    single-view oracle render bit for bit."""
    m0, cam0, R, t = small
    m1, cam1 = helpers.scene(7000, 200, 136, 180.0, seed=4)
    cams = [cam0, cam0, cam1]
    poses = [(R, t), helpers.random_pose(12), helpers.random_pose(13)]
    s0, _ = _map_spec(m0, True)
    s1, _ = _map_spec(m1, False)
    views = [_view(poses[0][0], poses[0][1], cam0, 0), _view(poses[1][0], poses[1][1], cam0, 0),
             _view(poses[2][0], poses[2][1], cam1, 1)]
    fr = GSFrame([s0, s1], views, channels=1, want_n_contrib=True, device=DEV)
    fr.render(exact_keys=True)
    torch.cuda.synchronize()
    for i, (mm, cam, (Rv, tv)) in enumerate(zip([m0, m0, m1], cams, poses)):
        res = oracle.rasterize_view(mm["xyz"], helpers.cov6(mm), mm["sh"], mm["opacity"],
                                    helpers.view_vector(Rv, tv, cam), cam.width, cam.height, [0.0], nch=1)
        got = fr.pixels(i)[0].cpu().numpy()
        assert _bits_equal(got, res["image"][0]), i
        assert np.array_equal(fr.view_slice(fr.n_contrib, i).cpu().numpy(), res["n_contrib"]), i


def test_empty_and_culled():
    m, cam = helpers.scene(500, 64, 48, 60.0, seed=1)
    R = gpose.exp_so3([0.0, math.pi, 0.0])  # looking away from the map
    t = np.zeros(3)
    s, _ = _map_spec(m)
    fr = GSFrame([s], [_view(R, t, cam, bg=(0.5, 0.25, 0.0))], channels=3, want_radii=True, device=DEV)
    fr.render(exact_keys=True)
    assert fr.num_keys == 0
    img = fr.image.view(3, 48, 64).cpu().numpy()
    assert np.all(img[0] == 0.5) and np.all(img[1] == 0.25) and np.all(img[2] == 0.0)
    assert not fr.radii[:500].any()


def test_key_overflow_is_reported_not_faulting(small):
    m, cam, R, t = small
    s, _ = _map_spec(m)
    fr = GSFrame([s], [_view(R, t, cam)], channels=1, key_capacity=1000, device=DEV)
    fr.preprocess()
    st, k = fr.status()
    assert k > 1000 and st & _lib.STATUS_KEY_OVERFLOW
    fr.bin_and_sort(0)
    fr.blend()
    torch.cuda.synchronize()
    st2, _ = fr.status()
    assert st2 & _lib.STATUS_KEY_OVERFLOW and not st2 & _lib.STATUS_SORT_TIMEOUT


# ------------------------------------------------------------------ adjoint --
def _pair_setup(n=20000, W=320, H=240, f=300.0, seed=0, pose_seed=21, unsigned=False):
    m, cam = helpers.scene(n, W, H, f, seed)
    R, t = helpers.random_pose(pose_seed)
    rng = np.random.default_rng(pose_seed)
    lin, ang, dtau = rng.normal(0, 0.3, 3), rng.normal(0, 0.3, 3), 0.02
    E = rng.normal(size=(H, W)).astype(np.float32)
    E /= np.linalg.norm(E.astype(np.float64))
    if unsigned:
        E = np.abs(E)
    return m, cam, R, t, lin, ang, dtau, E


def _pair_frame(m, cam, R, t, lin, ang, dtau, E, unsigned=False, log_eps=None):
    (Rl, tl), (Rn, tn) = helpers.pair_views(R, t, lin, ang, dtau)
    s, keep = _map_spec(m, True)
    Et = _t(E.reshape(-1))
    views = [_view(Rl, tl, cam, 0, pair=0, role=0), _view(Rn, tn, cam, 0, pair=0, role=1)]
    fr = GSFrame([s], views, channels=1,
                 pairs=[{"last": 0, "next": 1, "event": Et, "unsigned": unsigned, "log_eps": log_eps}], device=DEV)
    fr._keep = (keep, Et)
    return fr, ((Rl, tl), (Rn, tn))


@pytest.mark.parametrize("size", [(320, 240, 300.0, 20000), (640, 480, 500.0, 60000)])
def test_alpha_support_rectangles_keep_images_bit_exact(size):
    """Frames with tracking pairs bin each Gaussian only into the tiles its alpha support
    (o * exp(-q/2) >= 1/255) can reach; frames without pairs use the 3-sigma rectangles.
    The same two views rendered both ways give bit-identical images with fewer pairs."""
    W, H, f, n = size
    m, cam, R, t, lin, ang, dtau, E = _pair_setup(n=n, W=W, H=H, f=f, seed=3, pose_seed=70)
    fr, views = _pair_frame(m, cam, R, t, lin, ang, dtau, E)
    fr.render(exact_keys=True)
    s, keep = _map_spec(m, True)
    plain = GSFrame([s], [_view(Rv, tv, cam, 0) for (Rv, tv) in views], channels=1, device=DEV)
    plain.render(exact_keys=True)
    torch.cuda.synchronize()
    assert fr.status()[0] == 0 and plain.status()[0] == 0
    assert 0 < fr.num_keys < plain.num_keys
    for i in range(2):
        assert torch.equal(fr.pixels(i), plain.pixels(i)), i


@pytest.mark.parametrize("unsigned,log_eps", [(False, None), (True, None), (False, 1e-3), (True, 1e-3)])
def test_pair_loss_and_twist_gradients(unsigned, log_eps):
    """Pair loss and per-view twist gradients against the oracle, for the linear grey change
    and the log-intensity change (log_eps).  Loss: 1e-6 relative (FP32 per-thread partials,
    FP64 above); in log mode 1e-5 (the device takes CUDA's logf of the FP32 pixel, the oracle
    an FP64 log).  Gradients: 1e-4 norm-relative against the FP64 oracle adjoint."""
    m, cam, R, t, lin, ang, dtau, E = _pair_setup(unsigned=unsigned)
    fr, views = _pair_frame(m, cam, R, t, lin, ang, dtau, E, unsigned, log_eps)
    fr.render(exact_keys=True)
    loss = torch.zeros(1, dtype=torch.float64, device=DEV)
    fr.loss(loss)
    fr.blend_backward()
    xi = torch.zeros((2, 6), dtype=torch.float64, device=DEV)
    fr.preprocess_backward(xi)
    torch.cuda.synchronize()
    W, H = cam.width, cam.height
    recs, imgs = [], []
    for (Rv, tv) in views:
        r = oracle.rasterize_view(m["xyz"], helpers.cov6(m), m["sh"], m["opacity"], helpers.view_vector(Rv, tv, cam),
                                  W, H, [0.0], nch=1, record=True)
        recs.append(r)
        imgs.append(r["image"][0])
    for i in range(2):
        assert _bits_equal(fr.pixels(i)[0].cpu().numpy(), imgs[i])
    L_ref, gn, gl = oracle.loss(imgs[0], imgs[1], E, unsigned, grads=True, log_eps=log_eps)
    tol = 1e-5 if log_eps else 1e-6
    print("pair loss (unsigned=%s, log_eps=%s): rel err %.2e" % (unsigned, log_eps, abs(loss.item() - L_ref) / L_ref))
    assert abs(loss.item() - L_ref) <= tol * abs(L_ref)
    xi = xi.cpu().numpy()
    for i, ((Rv, tv), g) in enumerate(zip(views, (gl, gn))):
        g_ref, _ = oracle.frozen_backward(recs[i], m["xyz"], m["opacity"], helpers.view_vector(Rv, tv, cam, np.float64),
                                          W, H, [0.0], 1, g.reshape(1, H, W), sh=m["sh"], scale=m["scale"],
                                          rot=m["rot"])
        err = np.linalg.norm(xi[i] - g_ref) / np.linalg.norm(g_ref)
        assert err < GRAD_RTOL, (i, err, xi[i], g_ref)


@pytest.mark.parametrize("log_eps", [None, 1e-3])
def test_twelve_vector_against_finite_differences(log_eps):
    """Chained (theta, rho, w, v) gradient of the pair loss against FP64 central finite
    differences (step 1e-6) of the oracle's frozen-decision pair loss, at several poses,
    for the linear and the log-intensity change."""
    worst = 0.0
    for k in range(4):
        m, cam, R, t, lin, ang, dtau, E = _pair_setup(n=6000, W=160, H=120, f=150.0, seed=2, pose_seed=40 + k)
        from gsevt.batched import BatchedTracker, Problem
        prob = Problem(0, R, t, lin, ang, dtau, cam.width, cam.height, cam.fx, cam.fy, _t(E.reshape(-1)),
                       lr=(0.0, 0.0, 0.0, 0.0), opt_vel=True, log_eps=log_eps)
        bt = BatchedTracker([m], [prob], device=DEV)
        # the float32 views the device derived from its FP64 pose state
        table = bt.frame.view_table.cpu().numpy().view(np.float32).reshape(2, -1)[:, :33].copy()
        bt.step()
        st = bt.states()
        g_gpu = st["grad"][0]
        recs = [oracle.rasterize_view(m["xyz"], helpers.cov6(m), m["sh"], m["opacity"], table[i], cam.width,
                                      cam.height, [0.0], nch=1, record=True) for i in range(2)]
        L_ref = oracle.loss(recs[0]["image"][0], recs[1]["image"][0], E, log_eps=log_eps)
        assert abs(st["loss"][0] - L_ref) < (1e-5 if log_eps else 1e-6) * L_ref

        def L(d):
            T = opose.se3_exp(np.concatenate([d[3:6], d[0:3]])) @ opose.pose_matrix(R, t)
            return helpers.oracle_pair_loss_f64(m, cam, T[:3, :3], T[:3, 3], lin + d[9:12], ang + d[6:9], dtau, E,
                                                recs, log_eps=log_eps)

        fd = np.zeros(12)
        for j in range(12):
            e = np.zeros(12)
            e[j] = 1e-6
            fd[j] = (L(e) - L(-e)) / 2e-6
        for grp in range(4):
            a, b = g_gpu[3 * grp:3 * grp + 3], fd[3 * grp:3 * grp + 3]
            err = np.linalg.norm(a - b) / np.linalg.norm(b)
            worst = max(worst, err)
            assert err < GRAD_RTOL, (k, grp, a, b, err)
    print("worst 12-vector relative error vs FD (log_eps=%s): %.3g" % (log_eps, worst))


# ----------------------------------------------------------------- drop-in --
def test_drop_in_rasterizer_matches_oracle_and_grads():
    from diff_gaussian_rasterization import GaussianRasterizationSettings, GaussianRasterizer
    from gsevt.camera import Camera
    m, cam = helpers.scene(8000, 160, 120, 150.0, seed=3)
    R, t = helpers.random_pose(5)
    W, H = cam.width, cam.height
    c = Camera(torch.tensor(R, dtype=torch.float32), torch.tensor(t, dtype=torch.float32), torch.zeros(3),
               torch.zeros(3), cam.fovx, cam.fovy, W, H, device="cuda")
    bg = torch.tensor([0.0, 0.0, 0.0], device=DEV)
    s = GaussianRasterizationSettings(
        image_height=H, image_width=W, tanfovx=math.tan(c.FoVx * 0.5), tanfovy=math.tan(c.FoVy * 0.5), bg=bg,
        scale_modifier=1.0, viewmatrix=c.world_view_transform, projmatrix=c.full_proj_transform,
        projmatrix_raw=c.projection_matrix, sh_degree=3, campos=c.camera_center, prefiltered=False,
        angular_vel=c.angular_vel, linear_vel=c.linear_vel, vel_transofrm=torch.eye(4, device=DEV),
        vel_transofrm_inv=torch.eye(4, device=DEV), delta_time=0, debug=False)
    xyz = _t(m["xyz"]).requires_grad_(True)
    means2D = torch.zeros_like(xyz, requires_grad=True)
    opac = _t(m["opacity"]).reshape(-1, 1).requires_grad_(True)
    sh = _t(m["sh"]).requires_grad_(True)
    sc = _t(m["scale"]).requires_grad_(True)
    rot = _t(m["rot"]).requires_grad_(True)
    color, radii, depth, alpha, n_touched = GaussianRasterizer(s)(
        means3D=xyz, means2D=means2D, shs=sh, colors_precomp=None, opacities=opac, scales=sc, rotations=rot,
        cov3D_precomp=None, theta=c.cam_rot_delta, rho=c.cam_trans_delta, w=c.cam_w_delta, v=c.cam_v_delta)
    # the view the drop-in builds from float32 settings tensors
    Rf = c.R.cpu().numpy().astype(np.float64)
    tf = c.T.cpu().numpy().astype(np.float64)
    v32 = np.concatenate([Rf.reshape(9), tf, c.projection_matrix.cpu().numpy().T.reshape(16),
                          c.camera_center.cpu().numpy(), [s.tanfovx, s.tanfovy]]).astype(np.float32)
    res = oracle.rasterize_view(m["xyz"], helpers.cov6(m), m["sh"], m["opacity"], v32, W, H, [0, 0, 0], nch=3,
                                record=True)
    assert _bits_equal(color.detach().cpu().numpy(), res["image"])
    assert np.array_equal(radii.cpu().numpy(), res["pre"]["radii"])
    assert np.array_equal(n_touched.cpu().numpy(), res["n_touched"])
    rng = np.random.default_rng(0)
    wc = rng.normal(size=(3, H, W))
    wd = rng.normal(size=(1, H, W)) * 0.1
    wa = rng.normal(size=(1, H, W))
    loss = (color * _t(wc.astype(np.float32))).sum() + (depth * _t(wd.astype(np.float32))).sum() + \
        (alpha * _t(wa.astype(np.float32))).sum()
    loss.backward()
    g_xi, mg = oracle.frozen_backward(res, m["xyz"], m["opacity"], v32.astype(np.float64), W, H, [0, 0, 0], 3, wc,
                                      sh=m["sh"], scale=m["scale"], rot=m["rot"], dL_ddepth=wd[0], dL_dalpha=wa[0],
                                      map_grads=True)

    def rel(a, b):
        return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30)

    assert rel(c.cam_trans_delta.grad.cpu().numpy(), g_xi[:3]) < GRAD_RTOL
    assert rel(c.cam_rot_delta.grad.cpu().numpy(), g_xi[3:]) < GRAD_RTOL
    assert rel(xyz.grad.cpu().numpy(), mg["means3d"]) < 1e-3
    assert rel(means2D.grad[:, :2].cpu().numpy(), mg["mean2d"]) < 1e-3
    assert rel(opac.grad.cpu().numpy()[:, 0], mg["opac"]) < 1e-3
    assert rel(sh.grad.cpu().numpy().reshape(-1, 48), mg["sh"]) < 1e-3
    assert rel(sc.grad.cpu().numpy(), mg["scale"]) < 1e-3
    assert rel(rot.grad.cpu().numpy(), mg["rot"]) < 1e-3


# ------------------------------------------------------------------ events --
def test_event_frame_gpu_vs_oracle():
    from gsevt.events import event_frames
    rng = np.random.default_rng(0)
    W, H, n = 640, 480, 200000
    x = rng.integers(0, W, n).astype(np.uint16)
    y = rng.integers(0, H, n).astype(np.uint16)
    p = rng.integers(0, 2, n).astype(np.uint8)
    sig, uns = event_frames(_t(x), _t(y), _t(p), W, H, 9, 3, DEV)
    s_ref, u_ref, _ = oracle.event_frame(W, H, x, y, p, 9)
    s0 = sig[0][0].cpu().numpy()
    np.testing.assert_allclose(s0, s_ref, atol=1e-6 * np.abs(s_ref).max())
    np.testing.assert_array_equal(uns[0][0].cpu().numpy(), np.abs(s0))
    lv = oracle.pyramid(s0, 3)
    for l in (1, 2):
        np.testing.assert_array_equal(sig[l][0].cpu().numpy(), lv[l])
    z, _ = event_frames(_t(x[:0]), _t(y[:0]), _t(p[:0]), W, H, 9, 1, DEV)
    assert not z[0].any()
    # with the desk_normal1 intrinsics and distortion (configs/VECTOR/desk_normal1_config.yaml)
    cam = (327.32749, 327.46184, 304.97749, 235.37621, -0.031982, 0.041966, -0.000507, -0.001031, 0.0)
    sig_d, _ = event_frames(_t(x), _t(y), _t(p), W, H, 9, 1, DEV, camera=cam)
    sd_ref, _, _ = oracle.event_frame(W, H, x, y, p, 9, camera=cam)
    np.testing.assert_allclose(sig_d[0][0].cpu().numpy(), sd_ref, atol=1e-6 * np.abs(sd_ref).max())
    assert np.abs(sd_ref - s_ref).max() > 1e-3 * np.abs(s_ref).max()


# ------------------------------------------------------- batched vs plain --
@pytest.mark.parametrize("log_eps", [None, 1e-3])
def test_batched_iteration_matches_plain_path(log_eps):
    from gsevt.batched import BatchedTracker, Problem
    from gsevt.camera import Camera
    from gsevt.renderer import GaussianMap
    from gsevt.tracker import make_optimizer, plain_iteration
    m, cam, R, t, lin, ang, dtau, E = _pair_setup(n=20000, W=320, H=240, f=300.0, seed=0, pose_seed=60)
    Et = _t(E)
    lrs = {"cam_rot_delta": 0.004, "cam_trans_delta": 0.004, "cam_w_delta": 0.002, "cam_v_delta": 0.002}
    # plain: reference-style per-view calls, torch glue, torch Adam
    c = Camera(torch.tensor(R, dtype=torch.float32), torch.tensor(t, dtype=torch.float32),
               torch.tensor(ang, dtype=torch.float32), torch.tensor(lin, dtype=torch.float32), cam.fovx, cam.fovy,
               cam.width, cam.height, delta_tau=dtau, device="cuda")
    c.fx, c.fy = cam.fx, cam.fy
    gm = GaussianMap.from_synthetic(m)
    opt = make_optimizer(c, lrs)
    bgc = torch.zeros(3, device=DEV)
    L_plain, _ = plain_iteration(c, gm, bgc, opt, 0, True, Et.view(1, cam.height, cam.width), None,
                                 log_eps=log_eps)
    # batched
    prob = Problem(0, R, t, lin, ang, dtau, cam.width, cam.height, cam.fx, cam.fy, Et.reshape(-1), opt_vel=True,
                   log_eps=log_eps)
    bt = BatchedTracker([m], [prob], device=DEV)
    bt.step()
    st = bt.states()
    assert abs(st["loss"][0] - L_plain) < 1e-5 * abs(L_plain)
    np.testing.assert_allclose(st["R"][0], c.R.cpu().numpy(), atol=2e-6)
    np.testing.assert_allclose(st["t"][0], c.T.cpu().numpy(), atol=2e-6)
    np.testing.assert_allclose(st["ang_vel"][0], c.angular_vel.cpu().numpy(), atol=2e-6)
    np.testing.assert_allclose(st["lin_vel"][0], c.linear_vel.cpu().numpy(), atol=2e-6)


@pytest.mark.parametrize("depth_kpt,pair_kpt,coop_sort", [(4, 4, 0), (8, 8, 1), (12, 4, 1)])
def test_sort_tuning_choices_keep_order_bit_exact(small, depth_kpt, pair_kpt, coop_sort):
    """Every sort configuration the autotuner may pick (onesweep keys per thread 4 / 8 / 12,
    the cooperative sort allowed or not) gives the oracle's keys, sort order, ranges and
    image bit for bit.  A 2M key capacity makes the tile sort run the onesweep passes."""
    m, cam, R, t = small
    W, H = cam.width, cam.height
    s, _ = _map_spec(m, True)
    fr = GSFrame([s], [_view(R, t, cam)], channels=1, key_capacity=2_000_000, device=DEV)
    fr.set_tuning(depth_sort_kpt=depth_kpt, pair_sort_kpt=pair_kpt, coop_sort=coop_sort)
    fr.render(exact_keys=True)
    torch.cuda.synchronize()
    assert fr.status()[0] == 0
    res = oracle.rasterize_view(m["xyz"], helpers.cov6(m), m["sh"], m["opacity"], helpers.view_vector(R, t, cam),
                                W, H, [0.0], nch=1)
    K = fr.num_keys
    buf = ((fr.L.sort_bits - 32 + 7) // 8) & 1
    vals = _region(fr, "vals%d" % buf, torch.int32, K).cpu().numpy().view(np.uint32)
    assert np.array_equal(vals, res["vals"])
    rng = _region(fr, "ranges", torch.int32, 2 * fr.L.total_tiles).view(-1, 2).cpu().numpy().view(np.uint32)
    assert np.array_equal(rng, res["ranges"])
    assert _bits_equal(fr.pixels(0)[0].cpu().numpy(), res["image"][0])


def test_batched_step_without_the_cooperative_sort_matches():
    """The batched step with the cooperative sort turned off (visible-slot compaction,
    onesweep depth sort, coarse duplication and the super-tile sort as separate kernels, the
    path of frames above 8192 slots per SM) renders the same images, loss and gradient."""
    from gsevt.batched import BatchedTracker, Problem
    m, cam, R, t, lin, ang, dtau, E = _pair_setup(n=20000, W=320, H=240, f=300.0, seed=0, pose_seed=33)
    out = []
    for coop in (0, 1):
        prob = Problem(0, R, t, lin, ang, dtau, cam.width, cam.height, cam.fx, cam.fy, _t(E.reshape(-1)),
                       lr=(0.0, 0.0, 0.0, 0.0), opt_vel=True)
        bt = BatchedTracker([m], [prob], device=DEV)
        bt.frame.set_tuning(coop_sort=coop, depth_sort_kpt=8)
        bt.step()
        torch.cuda.synchronize()
        assert bt.check_status()[0] == 0
        out.append((bt.frame.image.clone(), bt.states()))
    (i0, s0), (i1, s1) = out
    assert torch.equal(i0.view(torch.int32), i1.view(torch.int32))
    assert s0["loss"][0] == s1["loss"][0]
    assert np.linalg.norm(s0["grad"][0] - s1["grad"][0]) <= 1e-5 * np.linalg.norm(s0["grad"][0])
