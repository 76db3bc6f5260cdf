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
                 event_unsigned=None, lr=DEFAULT_LR, opt_vel=True, unsigned=False):
        self.map_index = map_index
        self.R, self.t = np.asarray(R, np.float64), np.asarray(t, np.float64)
        self.lin_vel, self.ang_vel = np.asarray(lin_vel, np.float64), np.asarray(ang_vel, np.float64)
        self.delta_tau = float(delta_tau)
        self.width, self.height, self.fx, self.fy = int(width), int(height), float(fx), float(fy)
        self.event_signed = event_signed.reshape(-1).contiguous().float()
        self.event_unsigned = None if event_unsigned is None else event_unsigned.reshape(-1).contiguous().float()
        self.lr, self.opt_vel, self.unsigned = lr, bool(opt_vel), bool(unsigned)


def _field(name):
    return getattr(_lib.PoseState, name).offset


class BatchedTracker:
    def __init__(self, maps, problems, key_capacity=None, device="cuda"):
        """maps: list of dicts with xyz, opacity, sh, scale, rot (numpy or tensors) or
        already-packed tensors under "packed" with "n"."""
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
            ev = p.event_unsigned if (p.unsigned and p.event_unsigned is not None) else p.event_signed
            pairs.append({"last": 2 * i, "next": 2 * i + 1, "event": ev, "unsigned": p.unsigned, "pose": i})
        self.frame = GSFrame(specs, views, channels=1, pairs=pairs, key_capacity=key_capacity or (1 << 20),
                             device=self.device)
        self.num = len(self.problems)
        self.loss = torch.zeros(self.num, dtype=torch.float64, device=self.device)
        self._init_states()
        self.graph = None
        if key_capacity is None:
            self.fit_capacity()

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
