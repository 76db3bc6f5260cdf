"""GPU tests of the tracking layer: batched launches of many problems against single
launches, batched vs plain convergence, the per-frame tracker loop, and the device
event frame inside the tracker."""
import math

import numpy as np
import pytest
import torch

from gsevt import _lib
from gsevt import pose as gpose
from gsevt import synthetic
from gsevt.batched import BatchedTracker, Problem
from gsevt.camera import Camera
from gsevt.engine import GSFrame, MapSpec, ViewSpec, pack_map
from gsevt.events import EventArray, event_frames
from gsevt.renderer import GaussianMap
from gsevt.tracker import Tracker, make_optimizer, plain_iteration

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def _scenario(n, W, H, f, seed, n_events):
    sc = synthetic.Scenario(n, seed, W, H, f, n_events)
    m = sc.map
    pk = pack_map(_t(m["xyz"]), _t(m["opacity"]), _t(m["sh"]), scales=_t(m["scale"]), rotations=_t(m["rot"]))
    Tl, Tn = sc.gt_pair()
    cam = sc.camera
    views = [ViewSpec(W, H, 0, R=T[:3, :3], t=T[:3, 3], P=cam.proj, campos=gpose.campos(T[:3, :3], T[:3, 3]),
                      tanfovx=cam.tanfovx, tanfovy=cam.tanfovy) for T in (Tl, Tn)]
    fr = GSFrame([MapSpec(n, packed=pk)], views, channels=1, device=DEV)
    fr.render(exact_keys=True)
    a, b = fr.pixels(0)[0].cpu().numpy(), fr.pixels(1)[0].cpu().numpy()
    ex, ey, ep, ts = synthetic.synth_events(a, b, n_events, seed + 77, delta_tau=sc.delta_tau)
    sig, uns = event_frames(_t(ex), _t(ey), _t(ep), W, H, 9, 3, DEV)
    return sc, pk, sig, uns, EventArray(ex, ey, ep, ts)


def test_batched_problems_match_single_launches():
    """Three problems over two maps of different image sizes in one launch give the same
    losses (bit-identical) and 12-vector gradients as one launch per problem."""
    s0, pk0, sig0, uns0, _ = _scenario(20000, 320, 240, 300.0, 3, 30000)
    s1, pk1, sig1, uns1, _ = _scenario(15000, 256, 192, 220.0, 4, 30000)
    maps = [{"packed": pk0, "n": 20000}, {"packed": pk1, "n": 15000}]
    def prob(sc, mi, E, seed):
        R, t = synthetic.perturb(sc.gt_R, sc.gt_t, np.random.default_rng(seed), 0.05, 3.0)
        c = sc.camera
        return Problem(mi, R, t, sc.init_lin, sc.init_ang, sc.delta_tau, c.width, c.height, c.fx, c.fy,
                       E.reshape(-1), opt_vel=True)

    probs = [prob(s0, 0, sig0[0], 10), prob(s1, 1, sig1[0], 11), prob(s0, 0, sig0[0], 12)]
    bt = BatchedTracker(maps, probs, device=DEV)
    bt.step()
    st = bt.states()
    # problems are reordered by map: 0, 2 (map 0) then 1 (map 1)
    for slot, pi in enumerate(bt.order):
        single = BatchedTracker([maps[probs[pi].map_index]],
                                [Problem(0, probs[pi].R, probs[pi].t, probs[pi].lin_vel, probs[pi].ang_vel,
                                         probs[pi].delta_tau, probs[pi].width, probs[pi].height, probs[pi].fx,
                                         probs[pi].fy, probs[pi].event_signed, opt_vel=True)], device=DEV)
        single.step()
        ss = single.states()
        # the forward is deterministic; the adjoint's per-Gaussian sums use FP32 atomics
        # across tiles, so gradients agree to rounding, not bit for bit
        assert ss["loss"][0] == st["loss"][slot], (pi, ss["loss"][0], st["loss"][slot])
        g1, g2 = ss["grad"][0], st["grad"][slot]
        assert np.linalg.norm(g1 - g2) <= 1e-5 * np.linalg.norm(g1), (pi, g1, g2)
        np.testing.assert_allclose(ss["R"][0], st["R"][slot], atol=1e-7)
        np.testing.assert_allclose(ss["t"][0], st["t"][slot], atol=1e-7)


def _ws_region(frame, name, dtype, count):
    off = _lib.workspace_offsets(frame.L)[name]
    nbytes = count * torch.empty((), dtype=dtype).element_size()
    return frame.workspace[off:off + nbytes].view(dtype)


@pytest.mark.parametrize("sizes", [((320, 240, 300.0, 20000), (256, 192, 220.0, 15000)),
                                   ((640, 480, 600.0, 20000), (1280, 720, 900.0, 15000)),
                                   ((64, 48, 60.0, 60000), (96, 64, 80.0, 40000))])
def test_super_tile_lists_match_tile_sort(sizes):
    """The batched step bins through 4x4-tile super-tiles; its per-tile lists, ranges and
    images equal the full stable tile sort of gsevt_bin_and_sort on the same views (the
    third case: small dense views whose single super-tiles hold 20-34k Gaussians)."""
    (w0, h0, f0, n0), (w1, h1, f1, n1) = sizes
    s0, pk0, sig0, _, _ = _scenario(n0, w0, h0, f0, 5, 30000)
    s1, pk1, sig1, _, _ = _scenario(n1, w1, h1, f1, 6, 30000)
    maps = [{"packed": pk0, "n": n0}, {"packed": pk1, "n": n1}]
    def prob(sc, mi, E, seed):
        R, t = synthetic.perturb(sc.gt_R, sc.gt_t, np.random.default_rng(seed), 0.05, 3.0)
        c = sc.camera
        return Problem(mi, R, t, sc.init_lin, sc.init_ang, sc.delta_tau, c.width, c.height, c.fx, c.fy,
                       E.reshape(-1), opt_vel=True)
    probs = [prob(s0, 0, sig0[0], 20), prob(s1, 1, sig1[0], 21), prob(s0, 0, sig0[0], 22)]
    bt = BatchedTracker(maps, probs, device=DEV)
    fr = bt.frame
    L = fr.L
    views0 = fr.view_table.clone()
    bt.step()
    torch.cuda.synchronize()
    st, _ = fr.status()
    assert st == 0, st
    # the super-tile sort ends in buffer (passes & 1); the fine lists are in the other one
    # (one pass for the 32 super-tiles of the small pair, two for the 320 of the large one)
    bound = L.super_tiles
    assert bound == sum(((v.width + 63) // 64) * ((v.height + 63) // 64) for v in fr.views)
    bits = max(1, int(bound - 1).bit_length())
    fine_buf = (((bits + 7) // 8) & 1) ^ 1
    T = L.total_tiles
    img_c = fr.image.clone()
    rng_c = _ws_region(fr, "ranges", torch.int32, 2 * T).view(T, 2).clone().cpu().numpy()
    vals_c = _ws_region(fr, "vals%d" % fine_buf, torch.int32, L.key_capacity).clone().cpu().numpy()
    # the full tile sort on the same view table
    fr.view_table.copy_(views0)
    fr.preprocess()
    fr.bin_and_sort()
    fr.blend()
    torch.cuda.synchronize()
    st, K = fr.status()
    assert st == 0, st
    tile_buf = ((L.sort_bits - 32 + 7) // 8) & 1
    rng_f = _ws_region(fr, "ranges", torch.int32, 2 * T).view(T, 2).cpu().numpy()
    vals_f = _ws_region(fr, "vals%d" % tile_buf, torch.int32, L.key_capacity).cpu().numpy()
    assert (rng_f[:, 1] - rng_f[:, 0]).sum() == K
    np.testing.assert_array_equal(rng_c[:, 1] - rng_c[:, 0], rng_f[:, 1] - rng_f[:, 0])
    for t in range(T):
        a, b = rng_c[t]
        c, d = rng_f[t]
        if b > a:
            assert np.array_equal(vals_c[a:b], vals_f[c:d]), t
    assert torch.equal(img_c, fr.image)


def test_super_tile_overflow_is_reported_not_faulting():
    """A key capacity far below the frame's pairs: the batched step flags the overflow,
    keeps every write and every tile range inside the buffers, and the GPU stays usable."""
    s0, pk0, sig0, _, _ = _scenario(20000, 320, 240, 300.0, 5, 30000)
    R, t = synthetic.perturb(s0.gt_R, s0.gt_t, np.random.default_rng(3), 0.05, 3.0)
    c = s0.camera
    prob = Problem(0, R, t, s0.init_lin, s0.init_ang, s0.delta_tau, c.width, c.height, c.fx, c.fy,
                   sig0[0].reshape(-1), opt_vel=True)
    bt = BatchedTracker([{"packed": pk0, "n": 20000}], [prob], key_capacity=1000, device=DEV)
    bt.step()
    torch.cuda.synchronize()
    st, k = bt.frame.status()
    assert k > 1000 and st & _lib.STATUS_KEY_OVERFLOW and not st & _lib.STATUS_SORT_TIMEOUT
    T = bt.frame.L.total_tiles
    rng = _ws_region(bt.frame, "ranges", torch.int32, 2 * T).view(T, 2).cpu().numpy()
    assert (rng[:, 1] >= rng[:, 0]).all() and rng.max() <= 1000


def test_layout_with_too_few_super_tiles_is_reported_not_faulting():
    """A layout whose super_tiles is below the views' super-tile count: the step flags
    GSEVT_STATUS_LAYOUT, every access stays in bounds (ids clamped, tile ranges inside the
    buffers) and the GPU stays usable for a correct step afterwards."""
    s0, pk0, sig0, _, _ = _scenario(20000, 320, 240, 300.0, 5, 30000)
    R, t = synthetic.perturb(s0.gt_R, s0.gt_t, np.random.default_rng(8), 0.05, 3.0)
    c = s0.camera
    prob = Problem(0, R, t, s0.init_lin, s0.init_ang, s0.delta_tau, c.width, c.height, c.fx, c.fy,
                   sig0[0].reshape(-1), opt_vel=True)
    maps = [{"packed": pk0, "n": 20000}]
    bt = BatchedTracker(maps, [prob], device=DEV)
    assert bt.frame._frame.L.super_tiles == 40
    bt.frame._frame.L.super_tiles = 3  # the workspace was sized for 40; fewer ids only shrink regions
    bt.step()
    torch.cuda.synchronize()
    st, _ = bt.frame.status()
    assert st & _lib.STATUS_LAYOUT
    T = bt.frame.L.total_tiles
    rng = _ws_region(bt.frame, "ranges", torch.int32, 2 * T).view(T, 2).cpu().numpy()
    assert (rng[:, 1] >= rng[:, 0]).all() and rng.max() <= bt.frame.L.key_capacity
    good = BatchedTracker(maps, [prob], device=DEV)
    good.step()
    torch.cuda.synchronize()
    assert good.frame.status()[0] == 0


def test_batched_step_with_a_problem_that_sees_nothing():
    """A problem whose camera faces away from the map (no visible Gaussian, empty super-tile
    groups, zero pairs) batched with a normal one: the normal problem's loss and gradient
    equal its single launch, the empty one's pose does not move, and nothing faults."""
    s0, pk0, sig0, _, _ = _scenario(20000, 320, 240, 300.0, 9, 30000)
    c = s0.camera
    R, t = synthetic.perturb(s0.gt_R, s0.gt_t, np.random.default_rng(4), 0.05, 3.0)
    flip = np.diag([-1.0, 1.0, -1.0])  # 180 degrees about the camera y axis
    Rb, tb = flip @ s0.gt_R, flip @ s0.gt_t
    good = Problem(0, R, t, s0.init_lin, s0.init_ang, s0.delta_tau, c.width, c.height, c.fx, c.fy,
                   sig0[0].reshape(-1), opt_vel=True)
    blind = Problem(0, Rb, tb, s0.init_lin, s0.init_ang, s0.delta_tau, c.width, c.height, c.fx, c.fy,
                    sig0[0].reshape(-1), opt_vel=True)
    maps = [{"packed": pk0, "n": 20000}]
    bt = BatchedTracker(maps, [good, blind], device=DEV)
    bt.step()
    torch.cuda.synchronize()
    st = bt.states()
    single = BatchedTracker(maps, [good], device=DEV)
    single.step()
    ss = single.states()
    assert ss["loss"][0] == st["loss"][0]
    assert np.linalg.norm(ss["grad"][0] - st["grad"][0]) <= 1e-5 * np.linalg.norm(ss["grad"][0])
    assert np.all(st["grad"][1] == 0.0)
    np.testing.assert_allclose(st["R"][1], Rb, atol=1e-12)
    np.testing.assert_allclose(st["t"][1], tb, atol=1e-12)


def test_batched_converges_like_plain():
    """100 fine-stage Adam iterations from a 5 cm / 3 degree perturbation: the batched
    adjoint path and the plain per-view drop-in path end within 1 mm / 0.05 degrees."""
    sc, pk, sig, uns, _ = _scenario(20000, 320, 240, 300.0, 0, 30000)
    cam = sc.camera
    E = sig[0]
    iters = 100
    prob = Problem(0, sc.init_R, sc.init_t, sc.init_lin, sc.init_ang, sc.delta_tau, cam.width, cam.height,
                   cam.fx, cam.fy, E.reshape(-1), opt_vel=True)
    bt = BatchedTracker([{"packed": pk, "n": 20000}], [prob], device=DEV)
    bt.capture(warmup=0)
    bt.run(iters)
    st = bt.states()
    c = Camera(torch.tensor(sc.init_R, dtype=torch.float32), torch.tensor(sc.init_t, dtype=torch.float32),
               torch.tensor(sc.init_ang, dtype=torch.float32), torch.tensor(sc.init_lin, dtype=torch.float32),
               cam.fovx, cam.fovy, cam.width, cam.height, delta_tau=sc.delta_tau, device="cuda")
    c.fx, c.fy = cam.fx, cam.fy
    lrs = {"cam_rot_delta": 0.004, "cam_trans_delta": 0.004, "cam_w_delta": 0.002, "cam_v_delta": 0.002}
    opt = make_optimizer(c, lrs)
    gm = GaussianMap.from_synthetic(sc.map)
    bg = torch.zeros(3, device=DEV)
    for _ in range(iters):
        plain_iteration(c, gm, bg, opt, 0, True, E, None, read_loss=False)
    Rp, tp = c.R.cpu().numpy().astype(np.float64), c.T.cpu().numpy().astype(np.float64)
    dt = np.linalg.norm(st["t"][0] - tp)
    dr = gpose.rotation_error_deg(st["R"][0], Rp)
    moved = np.linalg.norm(st["t"][0] - sc.init_t)
    assert moved > 1e-3  # the optimisation did move the pose
    assert dt < 1e-3 and dr < 0.05, (dt, dr)


def test_plain_tracker_loop_runs(tmp_path):
    """Tracker(...).tracking() over two event windows: coarse and fine stages, convergence
    checks, constant-velocity prediction; poses stay finite and move.  With a save path it
    writes the reference's outputs: the TUM trajectory and one overlay PNG per frame."""
    sc, pk, sig, uns, ea = _scenario(8000, 160, 120, 150.0, 5, 20000)
    cam = sc.camera
    cfg = {"Event": {"img_width": cam.width, "img_height": cam.height, "gaussian_kernel_size": 9,
                     "intrinsic": {"data": [cam.fx, 0, cam.width / 2, 0, cam.fy, cam.height / 2, 0, 0, 1]},
                     "distortion_factors": [0, 0, 0, 0, 0]},
           "Optimizer": {"cam_rot_delta": 0.004, "cam_trans_delta": 0.004, "cam_w_delta": 0.002,
                         "cam_v_delta": 0.002, "converged_threshold": 1e-4, "max_optim_iter": 12},
           "Tracking": {"save_path": str(tmp_path)}}
    c = Camera(torch.tensor(sc.init_R, dtype=torch.float32), torch.tensor(sc.init_t, dtype=torch.float32),
               torch.tensor(sc.init_ang, dtype=torch.float32), torch.tensor(sc.init_lin, dtype=torch.float32),
               cam.fovx, cam.fovy, cam.width, cam.height, device="cuda")
    c.fx, c.fy = cam.fx, cam.fy
    tr = Tracker(cfg, [ea, ea], c, GaussianMap.from_synthetic(sc.map), None, torch.zeros(3, device=DEV), "cuda")
    traj = tr.tracking()
    assert len(traj) == 2 and tr.iterations >= 2 * 3
    for ts, R, t in traj:
        assert np.all(np.isfinite(R)) and np.all(np.isfinite(t))
        assert abs(np.linalg.det(R) - 1.0) < 1e-4
    from gsevt import io as gio
    lines = open(tmp_path / "tracking_pose_tum.txt").read().splitlines()
    assert len(lines) == 2 and all(len(l.split()) == 8 for l in lines)
    for i in range(2):
        img = gio.read_png_rgb(str(tmp_path / "tracking_frames" / ("frame_%d.png" % i)))
        assert img.shape == (cam.height, cam.width, 3) and img.max() > 0


def test_event_pyramid_levels_in_tracker_frame():
    """EventFrame keeps the reference attributes and returns the nearest pyramid."""
    from gsevt.events import EventFrame
    sc, pk, sig, uns, ea = _scenario(4000, 128, 96, 120.0, 6, 20000)
    ef = EventFrame(128, 96, np.eye(3), np.zeros(5), 9, ea)
    assert ef.sign_delta_Ie.shape == (1, 96, 128)
    assert [p.shape for p in ef.sign_pyramid] == [(1, 96, 128), (1, 48, 64), (1, 24, 32)]
    assert torch.equal(ef.sign_pyramid[1][0], ef.sign_delta_Ie[0, ::2, ::2])
    assert torch.equal(ef.unsign_delta_Ie, ef.sign_delta_Ie.abs())
    assert abs(float(ef.sign_delta_Ie.double().norm()) - 1.0) < 1e-5


def _sequence(sc, pk, n, frames, n_events, seed):
    """Event windows along the scenario's constant-velocity ground truth."""
    from gsevt.pose import exp_se3, matrix
    cam = sc.camera
    u = np.concatenate([sc.gt_lin, sc.gt_ang])
    wins = []
    for k in range(frames):
        Tk = exp_se3(u * sc.delta_tau * k) @ matrix(sc.gt_R, sc.gt_t)
        Tl, Tn = gpose.pair_poses(Tk[:3, :3], Tk[:3, 3], sc.gt_lin, sc.gt_ang, sc.delta_tau)
        views = [ViewSpec(cam.width, cam.height, 0, R=T[:3, :3], t=T[:3, 3], P=cam.proj,
                          campos=gpose.campos(T[:3, :3], T[:3, 3]), tanfovx=cam.tanfovx, tanfovy=cam.tanfovy)
                 for T in (Tl, Tn)]
        fr = GSFrame([MapSpec(n, packed=pk)], views, channels=1, device=DEV)
        fr.render(exact_keys=True)
        a, b = fr.pixels(0)[0].cpu().numpy(), fr.pixels(1)[0].cpu().numpy()
        ex, ey, ep, ts = synthetic.synth_events(a, b, n_events, seed + k, delta_tau=sc.delta_tau)
        wins.append(EventArray(ex, ey, ep, ts + int(k * sc.delta_tau * 1e6)))
    return wins


@pytest.mark.parametrize("threshold", [0.0, 1e9])
def test_batched_sequence_tracker_matches_plain_tracker(threshold, tmp_path):
    """Per-frame loop (constant-velocity prediction, 3 pyramid levels, coarse/fine stages,
    velocity learning-rate ramp, iteration limits, slope convergence) on the device for
    three problems over two maps, against the plain Tracker run per problem.  The two
    thresholds make every stage length independent of last-bit loss values: 0 never
    converges (each level runs to its iteration limit), 1e9 converges as soon as 11
    losses exist (coarse -> fine after 11 iterations, fine ends 10 later)."""
    from gsevt.batched import BatchedSequenceTracker
    from gsevt.pose import exp_se3, matrix
    frames, max_iter = 2, 16
    s0, pk0, _, _, _ = _scenario(20000, 320, 240, 300.0, 7, 30000)
    s1, pk1, _, _, _ = _scenario(15000, 256, 192, 220.0, 8, 30000)
    w0 = _sequence(s0, pk0, 20000, frames, 30000, 100)
    w1 = _sequence(s1, pk1, 15000, frames, 30000, 200)
    # starts 1-2 cm / 0.5-1 deg from the ground truth, so that both paths keep track over
    # both frames and their ground-truth errors are comparable
    rng = np.random.default_rng(9)
    inits = []
    for sc, dt, dr in ((s0, 0.01, 0.5), (s1, 0.01, 0.5), (s0, 0.02, 1.0)):
        R, t = synthetic.perturb(sc.gt_R, sc.gt_t, rng, dt, dr)
        inits.append((R, t, sc.init_lin, sc.init_ang))
    cams = [(0, 320, 240, 300.0, 300.0), (1, 256, 192, 220.0, 220.0), (0, 320, 240, 300.0, 300.0)]
    wins = [[w0[k], w1[k], w0[k]] for k in range(frames)]
    bst = BatchedSequenceTracker([{"packed": pk0, "n": 20000}, {"packed": pk1, "n": 15000}], cams,
                                 max_optim_iter=max_iter, converged_threshold=threshold, poll_every=1,
                                 device=DEV)
    traj = bst.track(inits, wins, overlay_dir=str(tmp_path))
    from gsevt import io as gio
    for pi, (mi, W, H, fx, fy) in enumerate(cams):
        for k in range(frames):
            img = gio.read_png_rgb(str(tmp_path / ("problem_%d" % pi) / ("frame_%d.png" % k)))
            assert img.shape == (H, W, 3) and img.max() > 0
    for pi, (sc, win) in enumerate(((s0, w0), (s1, w1), (s0, w0))):
        cam = sc.camera
        R0, t0, lv, av = inits[pi]
        cfg = {"Event": {"img_width": cam.width, "img_height": cam.height, "gaussian_kernel_size": 9,
                         "intrinsic": {"data": [cam.fx, 0, cam.width / 2, 0, cam.fy, cam.height / 2, 0, 0, 1]},
                         "distortion_factors": [0, 0, 0, 0, 0]},
               "Optimizer": {"cam_rot_delta": 0.004, "cam_trans_delta": 0.004, "cam_w_delta": 0.002,
                             "cam_v_delta": 0.002, "converged_threshold": threshold, "max_optim_iter": max_iter}}
        c = Camera(torch.tensor(R0, dtype=torch.float32), torch.tensor(t0, dtype=torch.float32),
                   torch.tensor(av, dtype=torch.float32), torch.tensor(lv, dtype=torch.float32),
                   cam.fovx, cam.fovy, cam.width, cam.height, device="cuda")
        c.fx, c.fy = cam.fx, cam.fy
        tr = Tracker(cfg, win, c, GaussianMap.from_synthetic(sc.map), None, torch.zeros(3, device=DEV), "cuda")
        ref = tr.tracking()
        # identical stage lengths: coarse -> fine switch, level ends and iteration limits
        assert bst.problem_iterations[pi] == tr.iterations, (pi, bst.problem_iterations[pi], tr.iterations)
        # Adam normalises each gradient component, so a last-bit difference in a small
        # component (FP32 atomics in the adjoint) can change a step by up to the learning
        # rate (4 mm, 0.23 deg).  Frame 0 agrees to a few such steps; later frames start
        # from velocities learned in frame 0, so there the batched path is held to the
        # plain path's ground-truth error instead
        _, Rb, tb = traj[pi][0]
        _, Rp, tp = ref[0]
        assert np.linalg.norm(tb - tp) < 1.2e-2, (pi, tb, tp)
        assert gpose.rotation_error_deg(Rb, Rp.astype(np.float64)) < 0.7, pi
        u = np.concatenate([sc.gt_lin, sc.gt_ang])
        for k in range(frames):
            Tk = exp_se3(u * sc.delta_tau * k) @ matrix(sc.gt_R, sc.gt_t)
            _, Rb, tb = traj[pi][k]
            _, Rp, tp = ref[k]
            eb, ep = np.linalg.norm(tb - Tk[:3, 3]), np.linalg.norm(tp - Tk[:3, 3])
            rb = gpose.rotation_error_deg(Rb, Tk[:3, :3])
            rp = gpose.rotation_error_deg(Rp.astype(np.float64), Tk[:3, :3])
            assert eb < ep + 1.5e-2 and rb < rp + 0.7, (pi, k, eb, ep, rb, rp)


@pytest.mark.parametrize("n,W,H", [(20000, 346, 260), (200000, 320, 240)])
def test_blend_staging_and_schedule_choices_agree(n, W, H):
    """The tracker blends staged with TMA tile::gather4 tensor copies (gsevt_tuning
    blend_staging 2) and / or run as resident blocks taking tiles from one longest-first
    queue (blend_schedule 1), and the tracker adjoint and the grey forward with two pixels
    per lane (adjoint_pixels 2, forward_pixels 2; with blend_schedule 1 their blocks take
    the tiles longest first), give the images of the one-pixel launch bit for bit and the same
    loss; the twist gradients agree to FP32 atomic-order noise.  200k Gaussians at 320x240
    make tile lists of several 256-record batches, so the double buffering, the wait for an
    issued batch when a block stops early, and the mbarrier phases carried from tile to tile
    in a resident block all run; 346x260 leaves partial tiles and partial 8x8 warp blocks
    at the right and bottom edges."""
    sc = synthetic.Scenario(n, 5, W, H, 300.0, 30000)
    m, cam = sc.map, sc.camera
    pk = pack_map(_t(m["xyz"]), _t(m["opacity"]), _t(m["sh"]), scales=_t(m["scale"]), rotations=_t(m["rot"]))
    rng = np.random.default_rng(4)
    E = rng.normal(size=cam.width * cam.height).astype(np.float32)
    E /= np.linalg.norm(E.astype(np.float64))
    out = []
    for staging, schedule, pixels, fpixels in ((1, 0, 1, 1), (2, 0, 1, 1), (3, 0, 1, 1), (1, 1, 1, 1), (2, 1, 1, 1),
                                               (3, 1, 1, 1), (1, 0, 2, 1), (2, 1, 2, 1), (1, 0, 2, 2), (1, 0, 1, 2),
                                               (1, 1, 2, 2)):
        p = Problem(0, sc.init_R, sc.init_t, sc.init_lin, sc.init_ang, sc.delta_tau, cam.width, cam.height, cam.fx,
                    cam.fy, _t(E), lr=(0.0, 0.0, 0.0, 0.0), opt_vel=True)
        bt = BatchedTracker([{"packed": pk, "n": n}], [p], device=DEV, tuning="defaults")
        bt.frame.set_tuning(blend_staging=staging, blend_schedule=schedule, adjoint_pixels=pixels,
                            forward_pixels=fpixels)
        for _ in range(2):  # lr = 0: the second step repeats the first on reused buffers
            bt.step()
        torch.cuda.synchronize()
        assert bt.check_status()[0] == 0
        out.append((bt.frame.image.clone(), bt.states()))
    img1, s1 = out[0]
    for img2, s2 in out[1:]:
        assert torch.equal(img1.view(torch.int32), img2.view(torch.int32))
        assert s1["loss"][0] == s2["loss"][0]
        g1, g2 = s1["grad"][0], s2["grad"][0]
        assert np.linalg.norm(g1 - g2) <= 1e-5 * np.linalg.norm(g1), (g1, g2)


def test_large_frames_run_the_multi_block_scans():
    """Frames above 8192 scan blocks (here five 640x480 views of an 800k map, 4 M slots, and
    three tracking problems of it, 4.8 M slots) compact and bin through the three-launch
    block-sum scan instead of the one-block scan: every view of the frame is bit-exact
    against the oracle, and each problem of the batched step has the loss it has when run
    alone (which uses the cooperative sort)."""
    from oracle import oracle
    import helpers
    n, W, H = 800_000, 640, 480
    sc = synthetic.Scenario(n, 9, W, H, 600.0, 100000)
    m, cam = sc.map, sc.camera
    pk = pack_map(_t(m["xyz"]), _t(m["opacity"]), _t(m["sh"]), scales=_t(m["scale"]), rotations=_t(m["rot"]))
    rng = np.random.default_rng(2)
    poses = [synthetic.perturb(sc.gt_R, sc.gt_t, rng, 0.1, 5.0) for _ in range(5)]
    views = [ViewSpec(W, H, 0, R=R, t=t, P=cam.proj, campos=gpose.campos(R, t), tanfovx=cam.tanfovx,
                      tanfovy=cam.tanfovy) for R, t in poses]
    fr = GSFrame([MapSpec(n, packed=pk)], views, channels=1, device=DEV)
    assert fr.L.num_scan_blocks > 8192
    fr.render(exact_keys=True)
    torch.cuda.synchronize()
    assert fr.status()[0] == 0
    cov = helpers.cov6(m)
    for i in (0, 4):
        R, t = poses[i]
        res = oracle.rasterize_view(m["xyz"], cov, m["sh"], m["opacity"], helpers.view_vector(R, t, cam), W, H,
                                    [0.0], nch=1)
        got = fr.pixels(i)[0].cpu().numpy()
        assert np.array_equal(got.view(np.uint32), res["image"][0].view(np.uint32)), i
    del fr
    E = rng.normal(size=W * H).astype(np.float32)
    E /= np.linalg.norm(E.astype(np.float64))

    def probs(sel):
        return [Problem(0, poses[i][0], poses[i][1], sc.gt_lin, sc.gt_ang, sc.delta_tau, W, H, cam.fx, cam.fy, _t(E),
                        lr=(0.0, 0.0, 0.0, 0.0), opt_vel=True) for i in sel]

    big = BatchedTracker([{"packed": pk, "n": n}], probs([0, 1, 2]), device=DEV, tuning="defaults")
    assert big.frame.L.num_scan_blocks > 8192
    big.step()
    torch.cuda.synchronize()
    assert big.check_status()[0] == 0
    lb = big.states()["loss"]
    for k in range(3):
        one = BatchedTracker([{"packed": pk, "n": n}], probs([k]), device=DEV, tuning="defaults")
        one.step()
        assert one.states()["loss"][0] == lb[k], k
