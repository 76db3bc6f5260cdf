"""GPU parity at the benchmark sizes: the production code paths at 300k and 500k
Gaussians, 640x480, against the CPU oracle on the same seeded inputs.

  - the plain drop-in at 300k (seed 1, f = 600): radii, tile rectangles, duplicated keys,
    sort order, tile ranges, n_touched, contributor counts and images bit-exact; the
    (t, t + dtau) pair rendered through render2 and differentiated by autograd gives the
    theta / rho / w / v gradients of the FP64 oracle adjoint within 1e-4;
  - the graphed batched step at 500k (seed 2): at 20 random poses both views' images are
    bit-exact and the chained 12-vector matches FP64 central finite differences (step
    1e-6) of the oracle's pair loss within 1e-4 per parameter group.  At this size (one
    pair, 1M slots) the depth sort, the compaction and the super-tile binning run as one
    cooperative launch, a branch the small scenes do not take with 256+ super-tiles;
  - convergence: after 100 fine-stage iterations at 500k the batched and the plain path
    end within 1 mm / 0.05 degrees of each other.

Each test prints its worst error."""
import math

import numpy as np
import pytest
import torch

from oracle import oracle
from oracle import pose as opose
from gsevt import _lib
from gsevt import pose as gpose
from gsevt import synthetic
from gsevt.engine import GSFrame, MapSpec, ViewSpec, pack_map
from gsevt.events import event_frames
import helpers

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda")
GRAD_RTOL = 1e-4      # pose / velocity gradients (norm-relative per parameter group)
GREY = (0.2989, 0.5870, 0.1140)


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def _region(frame, name, dtype, count):
    off = _lib.workspace_offsets(frame.L)[name]
    nbytes = count * torch.empty((), dtype=dtype).element_size()
    return frame.workspace[off:off + nbytes].view(dtype)


def _bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.uint32)
    b = np.ascontiguousarray(b, np.float32).view(np.uint32)
    return np.array_equal(a, b)


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def _events(sc, pk, n_events):
    """Signed event frame of the scenario's ground-truth window (1 level)."""
    W, H = sc.camera.width, sc.camera.height
    cam = sc.camera
    views = [ViewSpec(W, H, 0, R=T[:3, :3], t=T[:3, 3], P=cam.proj, campos=gpose.campos(T[:3, :3], T[:3, 3]),
                      tanfovx=cam.tanfovx, tanfovy=cam.tanfovy) for T in sc.gt_pair()]
    fr = GSFrame([MapSpec(sc.map["xyz"].shape[0], packed=pk)], views, channels=1, device=DEV)
    fr.render(exact_keys=True)
    a, b = fr.pixels(0)[0].cpu().numpy(), fr.pixels(1)[0].cpu().numpy()
    ex, ey, ep, _ = synthetic.synth_events(a, b, n_events, sc.seed + 77, delta_tau=sc.delta_tau)
    sig, _ = event_frames(_t(ex), _t(ey), _t(ep), W, H, 9, 1, DEV)
    return sig[0][0].contiguous()


@pytest.fixture(scope="module")
def c2():
    sc = synthetic.Scenario(300_000, 1, 640, 480, 600.0, 1_000_000)
    m = sc.map
    pk = pack_map(_t(m["xyz"]), _t(m["opacity"]), _t(m["sh"]), scales=_t(m["scale"]), rotations=_t(m["rot"]))
    return sc, pk, helpers.cov6(m)


@pytest.fixture(scope="module")
def c3():
    sc = synthetic.Scenario(500_000, 2, 640, 480, 600.0, 1_000_000)
    m = sc.map
    pk = pack_map(_t(m["xyz"]), _t(m["opacity"]), _t(m["sh"]), scales=_t(m["scale"]), rotations=_t(m["rot"]))
    E = _events(sc, pk, sc.n_events)
    return sc, pk, helpers.cov6(m), E


def test_plain_drop_in_frame_300k_bit_exact(c2):
    """One RGB view at the initial pose through the drop-in's frame path (raw map tensors,
    3-sigma binning, full tile sort): every integer output and every image bit-exact."""
    sc, _, cov = c2
    m, cam = sc.map, sc.camera
    W, H = cam.width, cam.height
    n = m["xyz"].shape[0]
    R, t = sc.init_R, sc.init_t
    bg = (0.0, 0.0, 0.0)
    spec = MapSpec(n, xyz=_t(m["xyz"]), opacity=_t(m["opacity"]), scales=_t(m["scale"]), rotations=_t(m["rot"]),
                   shs=_t(m["sh"]))
    view = ViewSpec(W, H, 0, bg=bg, R=R, t=t, P=cam.proj, campos=gpose.campos(R, t), tanfovx=cam.tanfovx,
                    tanfovy=cam.tanfovy)
    fr = GSFrame([spec], [view], channels=3, want_depth=True, want_alpha=True, want_radii=True,
                 want_n_touched=True, want_n_contrib=True, device=DEV)
    fr.render(exact_keys=True)
    torch.cuda.synchronize()
    assert fr.status()[0] == 0
    res = oracle.rasterize_view(m["xyz"], cov, m["sh"], m["opacity"], helpers.view_vector(R, t, cam), W, H,
                                list(bg), nch=3)
    pre = res["pre"]
    vis = pre["touched"] > 0
    K = fr.num_keys
    print("300k drop-in frame: %d visible, %d keys" % (int(vis.sum()), K))
    assert vis.sum() > 100_000 and K == res["keys"].shape[0]
    assert np.array_equal(fr.radii[:n].cpu().numpy(), pre["radii"])
    binv = _region(fr, "bin", torch.int32, 4 * n).view(n, 4).cpu().numpy()
    assert np.array_equal(binv[:, 0], pre["touched"])
    rect = pre["rect"][vis]
    assert np.array_equal(binv[vis, 1] & 0xffff, rect[:, 0]) and np.array_equal(binv[vis, 1] >> 16, rect[:, 1])
    assert np.array_equal(binv[vis, 2] & 0xffff, rect[:, 2]) and np.array_equal(binv[vis, 2] >> 16, rect[:, 3])
    buf = ((fr.L.sort_bits - 32 + 7) // 8) & 1
    tiles = _region(fr, "keys%d" % buf, torch.int32, K).cpu().numpy().view(np.uint32)
    vals = _region(fr, "vals%d" % buf, torch.int32, K).cpu().numpy().view(np.uint32)
    assert np.array_equal(tiles, (res["keys"] >> np.uint64(32)).astype(np.uint32))
    assert np.array_equal(vals, res["vals"])
    rng = _region(fr, "ranges", torch.int32, 2 * fr.L.total_tiles).view(-1, 2).cpu().numpy().view(np.uint32)
    assert np.array_equal(rng, res["ranges"])
    assert _bits_equal(fr.image.view(3, H, W).cpu().numpy(), res["image"])
    assert _bits_equal(fr.final_T.view(H, W).cpu().numpy(), res["final_T"])
    assert _bits_equal(fr.depth.view(H, W).cpu().numpy(), res["depth"])
    assert _bits_equal(fr.alpha.view(H, W).cpu().numpy(), res["alpha"])
    assert np.array_equal(fr.n_contrib.view(H, W).cpu().numpy(), res["n_contrib"])
    assert np.array_equal(fr.n_touched[:n].cpu().numpy(), res["n_touched"])


def test_plain_drop_in_pair_gradients_300k(c2):
    """The reference's render2 -> grey -> normalised dI -> loss -> backward, through the
    drop-in GaussianRasterizer at 300k: both RGB renders bit-exact, the loss within 1e-5 and
    the theta, rho, w, v gradients within 1e-4 of the FP64 oracle adjoint chained exactly."""
    from gsevt.camera import Camera, focal2fov
    from gsevt.renderer import GaussianMap, render2
    from gsevt.tracker import RenderFrame
    sc, pk, cov = c2
    m, cam = sc.map, sc.camera
    W, H = cam.width, cam.height
    E = _events(sc, pk, sc.n_events)
    vp = Camera(torch.tensor(sc.init_R, dtype=torch.float32), torch.tensor(sc.init_t, dtype=torch.float32),
                torch.tensor(sc.init_ang, dtype=torch.float32), torch.tensor(sc.init_lin, dtype=torch.float32),
                cam.fovx, cam.fovy, W, H, delta_tau=sc.delta_tau, device="cuda")
    vp.fx, vp.fy = cam.fx, cam.fy
    for p in (vp.cam_w_delta, vp.cam_v_delta):
        p.requires_grad_(True)
    gm = GaussianMap.from_synthetic(m)
    # GaussianMap re-normalises the quaternions on the device (as get_rotation does); the
    # oracle takes the covariances of exactly those rotations
    cov = oracle.cov3d(m["scale"], gm.get_rotation.detach().cpu().numpy())
    bg = torch.zeros(3, device=DEV)
    cams = []
    for Ev in (vp.last_vel_transform, vp.next_vel_transform):
        T = Ev @ vp.curr_pose
        cams.append(Camera(T[:3, :3], T[:3, 3], vp.angular_vel, vp.linear_vel, focal2fov(vp.fx, W),
                           focal2fov(vp.fy, H), W, H, delta_tau=vp.delta_tau, device="cuda"))
    last_pkg, next_pkg = render2(cams[0], vp, cams[1], gm, bg)
    d = RenderFrame.get_intensity_frame(next_pkg["render"][None]) - \
        RenderFrame.get_intensity_frame(last_pkg["render"][None])
    n_r = d / torch.norm(d, p=2)
    loss = torch.norm(n_r - E[None])
    loss.backward()
    recs, greys = [], []
    for c, pkg in zip(cams, (last_pkg, next_pkg)):
        v32 = np.concatenate([c.R.cpu().numpy().astype(np.float64).reshape(9), c.T.cpu().numpy().astype(np.float64),
                              c.projection_matrix.cpu().numpy().T.reshape(16), c.camera_center.cpu().numpy(),
                              [math.tan(c.FoVx * 0.5), math.tan(c.FoVy * 0.5)]]).astype(np.float32)
        r = oracle.rasterize_view(m["xyz"], cov, m["sh"], m["opacity"], v32, W, H, [0.0, 0.0, 0.0], nch=3,
                                  record=True)
        assert _bits_equal(pkg["render"].detach().cpu().numpy(), r["image"])
        recs.append((r, v32))
        img = r["image"].astype(np.float64)
        greys.append(GREY[0] * img[0] + GREY[1] * img[1] + GREY[2] * img[2])
    L_ref, gn, gl = oracle.loss(greys[0], greys[1], E.cpu().numpy(), False, grads=True)
    assert abs(loss.item() - L_ref) <= 1e-5 * abs(L_ref), (loss.item(), L_ref)
    g_views = []
    for (r, v32), g in zip(recs, (gl, gn)):
        g3 = np.stack([w * g.reshape(H, W) for w in GREY])
        gx, _ = oracle.frozen_backward(r, m["xyz"], m["opacity"], v32.astype(np.float64), W, H, [0.0, 0.0, 0.0], 3,
                                       g3, sh=m["sh"], cov_pre=cov)
        g_views.append(gx)
    lin = vp.linear_vel.detach().cpu().numpy().astype(np.float64)
    ang = vp.angular_vel.detach().cpu().numpy().astype(np.float64)
    ref = opose.chain_pose_gradient(g_views[0], g_views[1], lin, ang, float(vp.delta_tau))
    got = [vp.cam_rot_delta.grad, vp.cam_trans_delta.grad, vp.cam_w_delta.grad, vp.cam_v_delta.grad]
    errs = [_rel(g.cpu().numpy(), r) for g, r in zip(got, ref)]
    print("300k drop-in pair: loss %.9f, gradient errors theta/rho/w/v %s" % (L_ref, ["%.2e" % e for e in errs]))
    assert max(errs) < GRAD_RTOL, errs


def test_batched_step_500k_images_and_fd_at_20_poses(c3):
    """The CUDA-graph batched iteration at 500k, 640x480: at 20 random poses (5 cm / 3 deg
    from ground truth, velocity ground truth + N(0, 0.1)) both rendered views are bit-exact
    against the oracle, the loss agrees to 1e-6, and the chained (theta, rho, w, v) gradient
    matches FP64 central finite differences of the oracle's frozen pair loss (step 1e-6)
    within 1e-4 per parameter group."""
    from gsevt.batched import BatchedTracker, Problem
    sc, pk, cov, E = c3
    m, cam = sc.map, sc.camera
    W, H = cam.width, cam.height
    n = m["xyz"].shape[0]
    En = E.cpu().numpy()
    worst, worst_loss = 0.0, 0.0
    for k in range(20):
        rng = np.random.default_rng(500 + k)
        R, t = synthetic.perturb(sc.gt_R, sc.gt_t, rng, 0.05, 3.0)
        lin = sc.gt_lin + rng.normal(0.0, 0.1, 3)
        ang = sc.gt_ang + rng.normal(0.0, 0.1, 3)
        prob = Problem(0, R, t, lin, ang, sc.delta_tau, W, H, cam.fx, cam.fy, E.reshape(-1), lr=(0.0, 0.0, 0.0, 0.0),
                       opt_vel=True)
        bt = BatchedTracker([{"packed": pk, "n": n}], [prob], device=DEV)
        table = bt.frame.view_table.cpu().numpy().view(np.float32).reshape(2, -1)[:, :33].copy()
        bt.capture(warmup=1)
        bt.graph.replay()
        torch.cuda.synchronize()
        assert bt.check_status()[0] == 0
        st = bt.states()
        recs = []
        for i in range(2):
            r = oracle.rasterize_view(m["xyz"], cov, m["sh"], m["opacity"], table[i], W, H, [0.0], nch=1, record=True)
            assert _bits_equal(bt.frame.pixels(i)[0].cpu().numpy(), r["image"][0]), (k, i)
            recs.append(r)
        L_ref = oracle.loss(recs[0]["image"][0], recs[1]["image"][0], En)
        worst_loss = max(worst_loss, abs(st["loss"][0] - L_ref) / abs(L_ref))
        assert abs(st["loss"][0] - L_ref) <= 1e-6 * abs(L_ref), (k, st["loss"][0], L_ref)

        def L(dv):
            T = opose.se3_exp(np.concatenate([dv[3:6], dv[0:3]])) @ opose.pose_matrix(R, t)
            return helpers.oracle_pair_loss_f64(m, cam, T[:3, :3], T[:3, 3], lin + dv[9:12], ang + dv[6:9],
                                                sc.delta_tau, En, recs, cov=cov)

        fd = np.zeros(12)
        for j in range(12):
            e = np.zeros(12)
            e[j] = 1e-6
            fd[j] = (L(e) - L(-e)) / 2e-6
        g = st["grad"][0]
        for grp in range(4):
            err = _rel(g[3 * grp:3 * grp + 3], fd[3 * grp:3 * grp + 3])
            worst = max(worst, err)
            assert err < GRAD_RTOL, (k, grp, g[3 * grp:3 * grp + 3], fd[3 * grp:3 * grp + 3], err)
        del bt
    print("500k graphed step, 20 poses: images bit-exact; worst loss rel err %.2e; worst 12-vector rel err "
          "vs FD %.2e" % (worst_loss, worst))


def test_batched_converges_like_plain_500k(c3):
    """100 fine-stage Adam iterations from the scenario's 5 cm / 3 degree perturbation at
    500k, 640x480: the graphed batched path and the plain per-view drop-in path end within
    1 mm / 0.05 degrees of each other."""
    from gsevt.batched import BatchedTracker, Problem
    from gsevt.camera import Camera
    from gsevt.renderer import GaussianMap
    from gsevt.tracker import make_optimizer, plain_iteration
    sc, pk, _, E = c3
    cam = sc.camera
    n = sc.map["xyz"].shape[0]
    iters = 100
    prob = Problem(0, sc.init_R, sc.init_t, sc.init_lin, sc.init_ang, sc.delta_tau, cam.width, cam.height,
                   cam.fx, cam.fy, E.reshape(-1), opt_vel=True)
    bt = BatchedTracker([{"packed": pk, "n": n}], [prob], device=DEV)
    bt.capture(warmup=0)
    bt.run(iters)
    st = bt.states()
    assert bt.check_status()[0] == 0
    c = Camera(torch.tensor(sc.init_R, dtype=torch.float32), torch.tensor(sc.init_t, dtype=torch.float32),
               torch.tensor(sc.init_ang, dtype=torch.float32), torch.tensor(sc.init_lin, dtype=torch.float32),
               cam.fovx, cam.fovy, cam.width, cam.height, delta_tau=sc.delta_tau, device="cuda")
    c.fx, c.fy = cam.fx, cam.fy
    lrs = {"cam_rot_delta": 0.004, "cam_trans_delta": 0.004, "cam_w_delta": 0.002, "cam_v_delta": 0.002}
    opt = make_optimizer(c, lrs)
    gm = GaussianMap.from_synthetic(sc.map)
    bg = torch.zeros(3, device=DEV)
    for _ in range(iters):
        plain_iteration(c, gm, bg, opt, 0, True, E[None], None, read_loss=False)
    Rp, tp = c.R.cpu().numpy().astype(np.float64), c.T.cpu().numpy().astype(np.float64)
    dt = float(np.linalg.norm(st["t"][0] - tp))
    dr = gpose.rotation_error_deg(st["R"][0], Rp)
    moved = float(np.linalg.norm(st["t"][0] - sc.init_t))
    print("500k convergence: batched vs plain %.3f mm / %.4f deg after %d iterations (moved %.1f mm)"
          % (1e3 * dt, dr, iters, 1e3 * moved))
    assert moved > 1e-3
    assert dt < 1e-3 and dr < 0.05, (dt, dr)
