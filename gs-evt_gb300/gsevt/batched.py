"""Batched adjoint tracking path.

Many tracking problems (the (t, t + dtau) pair of one pose, dozens of pose hypotheses
of one map, or concurrent sequences with different maps and resolutions) are rendered
as one frame of views: every stage is one launch over all views, the loss and the
adjoint go straight to the per-view twist, and the FP64 chain, Adam step and pose /
velocity update run on the device (gsevt_track_step_batched).  `capture()` records one
iteration as a CUDA graph; `run()` replays it without any host synchronisation.

Pose state per problem lives in device memory (gsevt_pose_state, FP64).
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check, lib
from .engine import GSFrame, MapSpec, ViewSpec, pack_map, _ptr, _stream
from .pose import projection_matrix, focal2fov

DEFAULT_LR = (0.004, 0.004, 0.002, 0.002)  # theta, rho, w, v (configs/VECTOR/*.yaml)


class Problem:
    """One tracking problem: map index, current pose / velocity, event frames, camera."""

    def __init__(self, map_index, R, t, lin_vel, ang_vel, delta_tau, width, height, fx, fy, event_signed,
                 event_unsigned=None, lr=DEFAULT_LR, opt_vel=True, unsigned=False, log_eps=None):
        self.map_index = map_index
        self.R, self.t = np.asarray(R, np.float64), np.asarray(t, np.float64)
        self.lin_vel, self.ang_vel = np.asarray(lin_vel, np.float64), np.asarray(ang_vel, np.float64)
        self.delta_tau = float(delta_tau)
        self.width, self.height, self.fx, self.fy = int(width), int(height), float(fx), float(fy)
        self.event_signed = event_signed.reshape(-1).contiguous().float()
        self.event_unsigned = None if event_unsigned is None else event_unsigned.reshape(-1).contiguous().float()
        self.lr, self.opt_vel, self.unsigned = lr, bool(opt_vel), bool(unsigned)
        # None: the reference's linear grey change; eps > 0: ln(I_next + eps) - ln(I_last + eps)
        self.log_eps = log_eps


def _field(name):
    return getattr(_lib.PoseState, name).offset


class BatchedTracker:
    def __init__(self, maps, problems, key_capacity=None, device="cuda", key_margin=1.3, tuning="table"):
        """maps: list of dicts with xyz, opacity, sh, scale, rot (numpy or tensors) or
        already-packed tensors under "packed" with "n".  tuning: "table" (the autotuner's
        choice for this workload shape when its table has one, else the defaults),
        "defaults", or a dict of gsevt_tuning fields."""
        self.device = torch.device(device)
        order = sorted(range(len(problems)), key=lambda i: problems[i].map_index)
        self.problems = [problems[i] for i in order]
        self.order = order
        self.packed, specs = [], []
        for m in maps:
            if "packed" in m:
                pk, n = m["packed"], int(m["n"])
            else:
                t = lambda a: torch.as_tensor(np.asarray(a) if not torch.is_tensor(a) else a,
                                              dtype=torch.float32).to(self.device).contiguous()
                n = int(np.asarray(m["xyz"]).shape[0]) if not torch.is_tensor(m["xyz"]) else m["xyz"].shape[0]
                # rotations are taken as given: unit (w, x, y, z) quaternions, as the
                # rasterizer receives them from GaussianModel.get_rotation
                pk = pack_map(t(m["xyz"]), t(m["opacity"]), t(m["sh"]), scales=t(m["scale"]),
                              rotations=t(m["rot"]))
            self.packed.append(pk)
            specs.append(MapSpec(n, packed=pk, sh_degree=3))
        views, pairs = [], []
        for i, p in enumerate(self.problems):
            fovx, fovy = focal2fov(p.fx, p.width), focal2fov(p.fy, p.height)
            P = projection_matrix(fovx, fovy)
            for role in (0, 1):
                views.append(ViewSpec(p.width, p.height, p.map_index, R=np.eye(3), t=np.zeros(3), P=P,
                                      campos=np.zeros(3), tanfovx=np.tan(fovx / 2), tanfovy=np.tan(fovy / 2),
                                      pair=i, pair_role=role))
            pairs.append({"last": 2 * i, "next": 2 * i + 1, "event": p.event_signed, "event_abs": p.event_unsigned,
                          "unsigned": p.unsigned, "pose": i, "log_eps": p.log_eps})
        self.frame = GSFrame(specs, views, channels=1, pairs=pairs, key_capacity=key_capacity or (1 << 20),
                             device=self.device)
        self.num = len(self.problems)
        self.loss = torch.zeros(self.num, dtype=torch.float64, device=self.device)
        self._init_states()
        self.graph = None
        if key_capacity is None:
            self.fit_capacity(key_margin)
        self.tuning_source = "defaults"
        if isinstance(tuning, dict):
            self.frame.set_tuning(**tuning)
            self.tuning_source = "given"
        elif tuning == "table":
            from . import tuner
            choice = tuner.lookup(self.frame.L)
            if choice:
                self.frame.set_tuning(**choice)
                self.tuning_source = "table"

    # ---------------------------------------------------------------- state --
    def _init_states(self):
        arr = (_lib.PoseState * self.num)()
        for i, p in enumerate(self.problems):
            s = arr[i]
            for k in range(9):
                s.R[k] = float(p.R.reshape(9)[k])
            for k in range(3):
                s.t[k], s.lin_vel[k], s.ang_vel[k] = float(p.t[k]), float(p.lin_vel[k]), float(p.ang_vel[k])
            s.delta_tau = p.delta_tau
            for k in range(4):
                s.lr[k], s.lr_scale[k] = float(p.lr[k]), 1.0
            s.opt_vel = int(p.opt_vel)
            s.last_view, s.next_view = 2 * i, 2 * i + 1
            s.fx, s.fy = p.fx, p.fy
        raw = bytes(arr)
        self.state = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(self.device)
        self._sz = C.sizeof(_lib.PoseState)
        check(lib().gsevt_track_init_views(_ptr(self.frame.view_table), _ptr(self.state), self.num, _stream()),
              "gsevt_track_init_views")

    def _f64(self, name, count):
        o = _field(name) // 8
        return self.state.view(torch.float64).view(self.num, self._sz // 8)[:, o:o + count]

    def _i32(self, name, count):
        o = _field(name) // 4
        return self.state.view(torch.int32).view(self.num, self._sz // 4)[:, o:o + count]

    def set_stage(self, opt_vel=None, lr_scale=None):
        """Switch coarse/fine stage or the learning-rate multipliers on the device."""
        if opt_vel is not None:
            self._i32("opt_vel", 1).fill_(int(opt_vel))
        if lr_scale is not None:
            self._f64("lr_scale", 4).copy_(torch.as_tensor(lr_scale, dtype=torch.float64).expand(self.num, 4))

    def states(self):
        """Host copy of the pose states as numpy arrays (synchronises)."""
        st = self.state.view(torch.float64).view(self.num, self._sz // 8).cpu().numpy()
        i32 = self.state.view(torch.int32).view(self.num, self._sz // 4).cpu().numpy()
        g = lambda n, c: st[:, _field(n) // 8:_field(n) // 8 + c]
        return dict(R=g("R", 9).reshape(-1, 3, 3), t=g("t", 3), lin_vel=g("lin_vel", 3), ang_vel=g("ang_vel", 3),
                    loss=g("loss", 1)[:, 0], grad=g("grad", 12),
                    iter=i32[:, _field("iter") // 4])

    def states_raw(self):
        i32 = self.state.view(torch.int32).view(self.num, self._sz // 4).cpu().numpy()
        return {"frozen": i32[:, _field("frozen") // 4], "level_iter": i32[:, _field("level_iter") // 4]}

    # ----------------------------------------------------------------- run --
    def fit_capacity(self, margin=1.3):
        f = self.frame
        f.preprocess()
        _, k = f.status()
        cap = int(k * margin) + 65536
        if cap != f.L.key_capacity:
            f.grow(cap)
        self.num_keys = k
        self.graph = None

    def step(self):
        check(lib().gsevt_track_step_batched(self.frame.fref, _ptr(self.state), self.num, _ptr(self.loss),
                                             _stream()), "gsevt_track_step_batched")

    def capture(self, warmup=2):
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(warmup):
                self.step()
        torch.cuda.current_stream().wait_stream(s)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.step()
        return self.graph

    def run(self, iters):
        for _ in range(iters):
            if self.graph is not None:
                self.graph.replay()
            else:
                self.step()

    def check_status(self):
        st, k = self.frame.status()
        return st, k


class BatchedSequenceTracker:
    """The reference's per-frame tracking loop (utils/tracker.py:105-287) for many problems at
    once: per frame, constant-velocity prediction (camera.py:183-201), the event pyramid,
    then per pyramid level 2 -> 0 the coarse / fine Adam stages with slope convergence, run
    on the device for all problems in lockstep (finished problems are frozen), and after
    five frames the weighted velocity update (camera.py:157-181).

    cameras: list of (map_index, width, height, fx, fy) per problem.  log_eps selects the
    log-intensity change (as Problem).  One frame per pyramid
    level shares the maps and one device pose-state array; each level's iteration is a
    CUDA graph captured once and replayed for every frame."""

    def __init__(self, maps, cameras, lr=DEFAULT_LR, max_optim_iter=200, converged_threshold=1e-4, levels=3,
                 poll_every=10, device="cuda", log_eps=None):
        from .pose import exp_se3
        self.device = torch.device(device)
        self.levels, self.max_iter, self.thr, self.poll = levels, int(max_optim_iter), float(converged_threshold), poll_every
        self.cameras = cameras
        self.packed = []
        for m in maps:
            if "packed" in m:
                self.packed.append({"packed": m["packed"], "n": int(m["n"])})
            else:
                t = lambda a: torch.as_tensor(np.asarray(a) if not torch.is_tensor(a) else a,
                                              dtype=torch.float32).to(self.device).contiguous()
                n = int(np.asarray(m["xyz"]).shape[0])
                pk = pack_map(t(m["xyz"]), t(m["opacity"]), t(m["sh"]), scales=t(m["scale"]), rotations=t(m["rot"]))
                self.packed.append({"packed": pk, "n": n})
        self.lr = lr
        self.trackers, self.ev = [], []
        for l in range(levels):
            sc = 0.5 ** l
            bufs, probs = [], []
            for (mi, W, H, fx, fy) in cameras:
                w, h = int(W * sc), int(H * sc)
                es = torch.zeros(w * h, dtype=torch.float32, device=self.device)
                eu = torch.zeros(w * h, dtype=torch.float32, device=self.device)
                bufs.append((es, eu))
                probs.append(Problem(mi, np.eye(3), np.zeros(3), np.zeros(3), np.zeros(3), 0.01, w, h, fx * sc,
                                     fy * sc, es, eu, lr=lr, log_eps=log_eps))
            self.ev.append(bufs)
            # capacity is fitted on the first frame
            self.trackers.append(BatchedTracker(self.packed, probs, key_capacity=1 << 20, device=self.device))
        self.order = self.trackers[0].order
        # event buffers in the trackers' (map-grouped) problem order
        self.ev = [[bufs[pi] for pi in self.order] for bufs in self.ev]
        self.num = len(cameras)
        self.state = self.trackers[0].state
        for tr in self.trackers[1:]:
            tr.state = self.state
        self.fitted = False
        self.iterations = 0

    def _set_unsigned(self, tr, flags):
        sz = C.sizeof(_lib.Pair)
        off = _lib.Pair.unsigned_mode.offset // 4
        tab = tr.frame.pair_table.view(torch.int32).view(tr.num, sz // 4)
        tab[:, off].copy_(torch.as_tensor(flags, dtype=torch.int32))

    def _host_states(self):
        return self.state.view(torch.uint8).cpu().numpy().copy()

    def _write_overlay(self, overlay_dir, pi, slot, fi):
        import os
        from . import io as gio
        fr = self.trackers[0].frame
        d = fr.pixels(2 * slot + 1)[0] - fr.pixels(2 * slot)[0]  # I_next - I_last (frame.py:86-94)
        n = d / torch.linalg.vector_norm(d)
        mi, W, H, fx, fy = self.cameras[pi]
        e = self.ev[0][slot][0].view(H, W)
        path = os.path.join(overlay_dir, "problem_%d" % pi)
        os.makedirs(path, exist_ok=True)
        gio.write_png(os.path.join(path, "frame_%d.png" % fi), gio.event_overlay(e, n))

    def track(self, init_states, windows, overlay_dir=None):
        """init_states: per problem (R, t, lin_vel, ang_vel) (world -> camera, FP64);
        windows: per frame, a list with one EventArray per problem (or a tuple
        (x, y, polarity, ts, camera_or_None)).  Returns per problem a list of
        (timestamp, R, t).  overlay_dir: if given, each frame's tracking image (the signed
        event frame over the last finest-level render difference, utils/tracker.py:267-270)
        is written to overlay_dir/problem_<i>/frame_<f>.png."""
        from .events import event_frames
        from .pose import exp_se3, matrix, so3_log
        n = self.num
        arr = (_lib.PoseState * n)()
        # problems are stored in map order (self.order)
        for slot, pi in enumerate(self.order):
            R, t, lv, av = init_states[pi]
            s = arr[slot]
            for k in range(9):
                s.R[k] = float(np.asarray(R).reshape(9)[k])
            for k in range(3):
                s.t[k], s.lin_vel[k], s.ang_vel[k] = float(t[k]), float(lv[k]), float(av[k])
            for k in range(4):
                s.lr[k], s.lr_scale[k] = float(self.lr[k]), 1.0
            s.last_view, s.next_view = 2 * slot, 2 * slot + 1
            s.control, s.max_iter, s.conv_thr = 1, self.max_iter, self.thr
        host = arr
        traj = [[] for _ in range(n)]
        last_dtau = [0.0] * n
        for fi, frame in enumerate(windows):
            init_pose = []
            for slot, pi in enumerate(self.order):
                w = frame[pi]
                ts = w.ts if hasattr(w, "ts") else w[3]
                dtau = float(ts[-1] - ts[0]) / 1e6 if len(ts) else 0.0
                s = host[slot]
                tau = (dtau + last_dtau[slot]) / 2
                u = np.concatenate([np.asarray(s.lin_vel[:]) * tau, np.asarray(s.ang_vel[:]) * tau])
                T = exp_se3(u) @ matrix(np.asarray(s.R[:]).reshape(3, 3), np.asarray(s.t[:]))
                # the frame's initial status is the predicted pose (tracker.py:133-139)
                init_pose.append((T[:3, :3].copy(), T[:3, 3].copy()))
                for k in range(9):
                    s.R[k] = float(T[:3, :3].reshape(9)[k])
                for k in range(3):
                    s.t[k] = float(T[k, 3])
                s.delta_tau = dtau
                for k in range(12):
                    s.m[k] = s.v[k] = 0.0
                for k in range(4):
                    s.step[k] = 0
                # event pyramid of this problem into every level's buffers
                x, y, pol = (w.x, w.y, w.polarity) if hasattr(w, "x") else w[:3]
                cam = None if hasattr(w, "x") else w[4]
                mi, W, H, fx, fy = self.cameras[pi]
                tt = lambda a: a if torch.is_tensor(a) else torch.from_numpy(np.ascontiguousarray(a)).to(self.device)
                sig, uns = event_frames(tt(x), tt(y), tt(pol), W, H, 9, self.levels, self.device, camera=cam)
                for l in range(self.levels):
                    self.ev[l][slot][0].copy_(sig[l].reshape(-1))
                    self.ev[l][slot][1].copy_(uns[l].reshape(-1))
            for lvl in range(self.levels - 1, -1, -1):
                tr = self.trackers[lvl]
                opt_vel = int(lvl != self.levels - 1)
                for slot in range(n):
                    s = host[slot]
                    s.frozen, s.level_iter, s.start_vel, s.hist_n, s.opt_vel = 0, 0, 0, 0, opt_vel
                    for k in range(4):
                        s.lr_scale[k] = 1.0
                self.state.copy_(torch.frombuffer(bytearray(bytes(host)), dtype=torch.uint8))
                self._set_unsigned(tr, [1 - opt_vel] * n)
                check(lib().gsevt_track_init_views(_ptr(tr.frame.view_table), _ptr(self.state), n, _stream()),
                      "gsevt_track_init_views")
                if not self.fitted:
                    tr.fit_capacity(margin=2.0)
                if tr.graph is None:
                    tr.graph = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(tr.graph):
                        tr.step()
                    # capture does not run the work: restore the level's starting state
                    self.state.copy_(torch.frombuffer(bytearray(bytes(host)), dtype=torch.uint8))
                    self._set_unsigned(tr, [1 - opt_vel] * n)
                    check(lib().gsevt_track_init_views(_ptr(tr.frame.view_table), _ptr(self.state), n, _stream()),
                          "gsevt_track_init_views")
                limit = 2 * self.max_iter + 2
                done_iters = 0
                while done_iters < limit:
                    for _ in range(self.poll):
                        tr.graph.replay()
                    done_iters += self.poll
                    st = tr.states_raw()
                    if all(int(x) for x in st["frozen"]):
                        break
                self.iterations += done_iters
                st_b = self._host_states()
                host = (_lib.PoseState * n).from_buffer_copy(st_b.tobytes())
                stat, _ = tr.frame.status()
                bad = stat & (_lib.STATUS_KEY_OVERFLOW | _lib.STATUS_SORT_TIMEOUT | _lib.STATUS_LAYOUT)
                if bad:
                    raise RuntimeError("tracking at pyramid level %d: %s" % (lvl, _lib.status_names(bad)))
            self.fitted = True
            for slot, pi in enumerate(self.order):
                s = host[slot]
                w = frame[pi]
                ts = w.ts if hasattr(w, "ts") else w[3]
                dtau = float(ts[-1] - ts[0]) / 1e6 if len(ts) else 0.0
                if fi >= 5:
                    R0, t0 = init_pose[slot]
                    R1 = np.asarray(s.R[:]).reshape(3, 3)
                    t1 = np.asarray(s.t[:])
                    D = matrix(R1, t1) @ np.linalg.inv(matrix(R0, t0))
                    tau = (dtau + last_dtau[slot]) / 2
                    lv = D[:3, 3] / tau
                    av = so3_log(D[:3, :3]) / tau
                    for k in range(3):
                        s.lin_vel[k] = 0.5 * lv[k] + 0.5 * s.lin_vel[k]
                        s.ang_vel[k] = 0.5 * av[k] + 0.5 * s.ang_vel[k]
                last_dtau[slot] = dtau
                stamp = (ts[0] + (ts[-1] - ts[0]) / 2) / 1e6 if len(ts) else 0.0
                traj[pi].append((stamp, np.asarray(s.R[:]).reshape(3, 3).copy(), np.asarray(s.t[:]).copy()))
                if overlay_dir is not None:
                    self._write_overlay(overlay_dir, pi, slot, fi)
        self.state.copy_(torch.frombuffer(bytearray(bytes(host)), dtype=torch.uint8))
        # Adam iterations each problem ran (a frozen problem does not count)
        self.problem_iterations = [0] * n
        for slot, pi in enumerate(self.order):
            self.problem_iterations[pi] = int(host[slot].iter)
        return traj
