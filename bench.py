"""Tracking-iteration benchmark (one JSON line on rank 0).

Metric: tracking iterations per second at 500k Gaussians, 640x480 — one iteration is
the (t, t + dtau) render pair forward, the normalised intensity-change loss against
the event frame, the adjoint to the 6-DoF pose twist and 6-DoF velocity, the Adam step
and the pose / velocity update (utils/tracker.py:176-222).

  value      batched adjoint path (gsevt_track_step_batched, one CUDA graph per
             iteration), inputs resident in HBM, CUDA events per iteration, L2 flushed
             between iterations (outside the timed events)
  e2e        the same iteration through the public API with the step's inputs (event
             frame and pose state) copied from pinned host memory and the result (loss
             and pose state) read back, every step, inside the timed region
  plain      the plain per-view drop-in path (reference-structured tracker over the
             drop-in GaussianRasterizer, torch glue and torch Adam), timed beside it
  roofline   dominant stage of the iteration against the measured HBM bandwidth
  iteration_roofline  canonical compulsory bytes of a whole iteration (attribute reads,
             projected records, pairs, pixels; counts from the reference's 3-sigma
             binning) times iterations/s, against the same peak
  cpu_baseline  the CPU oracle (C + OpenMP) running the same iteration on the host
             cores, on a bounded sample

--impl reference times the reference's CPU implementation of the path: the reference
rasterizer's native source is absent from its tree, so this is the oracle restatement
(oracle/, kind "port") on all host cores.

Multi-GPU: tracking problems are independent; under torchrun every rank runs its own
replica (no collective on the data path), value = sum over ranks, time = max over ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "gs-evt_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np

WORKLOADS = {
    # name: (gaussians, seed, width, height, focal, events, hypotheses)
    "adjoint-500k-640x480": (500_000, 2, 640, 480, 600.0, 1_000_000, 1),
    "plain-300k-640x480": (300_000, 1, 640, 480, 600.0, 1_000_000, 1),
    "hypotheses-64x2-500k": (500_000, 3, 640, 480, 600.0, 1_000_000, 64),
}
METRIC = "tracking iters/sec at 500k Gaussians 640x480 (fwd+pose bwd); batched vs plain"
HBM_FALLBACK = 6800.0


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK, "fallback"


class ClockSampler:
    """SM clock and clock-event reasons sampled DURING the timed region (read-only).

    A thread polls NVML through ctypes (libnvidia-ml.so.1, which ships with the driver)
    every 2 ms, so that even a region of a few tens of milliseconds gets many samples;
    without NVML it falls back to `nvidia-smi --query-gpu ... -lms 200`."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason* bits (nvml.h)
    REASONS = ((0x8, "hw_slowdown"), (0x40, "hw_thermal_slowdown"), (0x20, "sw_thermal_slowdown"),
               (0x4, "sw_power_cap"), (0x80, "hw_power_brake_slowdown"))

    def __init__(self, gpu_index=0, uuid=None):
        self.gpu_index, self.uuid = gpu_index, uuid
        self.proc = None
        self.thread = None
        self.samples = []
        self.stop_flag = threading.Event()

    def _nvml(self):
        import ctypes as C
        nv = C.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            return None
        h = C.c_void_p()
        ok = False
        if self.uuid:
            ok = nv.nvmlDeviceGetHandleByUUID(self.uuid.encode(), C.byref(h)) == 0
        if not ok:
            ok = nv.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.gpu_index), C.byref(h)) == 0
        return (nv, h) if ok else None

    def start(self):
        try:
            handle = self._nvml()
        except Exception:
            handle = None
        if handle is not None:
            import ctypes as C
            nv, h = handle
            mx = C.c_uint(0)
            nv.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx))
            self.max_mhz = float(mx.value)

            def run():
                clk, rs = C.c_uint(0), C.c_ulonglong(0)
                while not self.stop_flag.is_set():
                    if nv.nvmlDeviceGetClockInfo(h, 1, C.byref(clk)) == 0 and \
                            nv.nvmlDeviceGetCurrentClocksEventReasons(h, C.byref(rs)) == 0:
                        self.samples.append((float(clk.value), int(rs.value)))
                    time.sleep(0.002)

            self.thread = threading.Thread(target=run, daemon=True)
            self.thread.start()
            return
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu_index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.thread is not None:
            self.stop_flag.set()
            self.thread.join()
            if not self.samples:
                return None
            reasons = sorted({nm for _, r in self.samples for bit, nm in self.REASONS if r & bit})
            return {"sm_mhz": statistics.median(c for c, _ in self.samples), "sm_max_mhz": self.max_mhz,
                    "reasons": reasons, "samples": len(self.samples), "source": "nvml, 2 ms"}
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi, 200 ms"}


def gpu_uuid(dev):
    """NVML-style UUID string of a torch device (None when torch does not expose it)."""
    import torch
    try:
        u = str(torch.cuda.get_device_properties(dev).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u
    except Exception:
        return None


def build_problem(name, device, seed_offset=0):
    import torch
    from gsevt import synthetic
    from gsevt import pose as gpose
    from gsevt.engine import GSFrame, MapSpec, ViewSpec, pack_map
    from gsevt.events import event_frames
    n, seed, W, H, f, n_events, hyp = WORKLOADS[name]
    sc = synthetic.Scenario(n, seed + seed_offset, W, H, f, n_events)
    m = sc.map
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
    rot = t(m["rot"])
    packed = pack_map(t(m["xyz"]), t(m["opacity"]), t(m["sh"]), scales=t(m["scale"]), rotations=rot)
    # events from grey log-intensity renders at the ground-truth pair poses
    Tl, Tn = sc.gt_pair()
    cam = sc.camera
    views = [ViewSpec(W, H, 0, R=T[:3, :3], t=T[:3, 3], P=cam.proj, campos=gpose.campos(T[:3, :3], T[:3, 3]),
                      tanfovx=cam.tanfovx, tanfovy=cam.tanfovy) for T in (Tl, Tn)]
    fr = GSFrame([MapSpec(n, packed=packed)], views, channels=1, device=device)
    fr.render(exact_keys=True)
    I_last = fr.pixels(0)[0].cpu().numpy()
    I_next = fr.pixels(1)[0].cpu().numpy()
    del fr
    ex, ey, ep, ts = synthetic.synth_events(I_last, I_next, n_events, seed + 77, delta_tau=sc.delta_tau)
    sig, uns = event_frames(t(ex), t(ey), t(ep), W, H, 9, 1, device)
    return dict(scenario=sc, map=m, packed=packed, n=n, W=W, H=H, f=f, E=sig[0].reshape(-1).contiguous(),
                E_unsigned=uns[0].reshape(-1).contiguous(), events=(ex, ey, ep, ts), hypotheses=hyp)


def make_tracker(prob, device, hypotheses=None, tuning="table"):
    from gsevt import synthetic
    from gsevt.batched import BatchedTracker, Problem
    sc = prob["scenario"]
    hyp = hypotheses or prob["hypotheses"]
    if hyp == 1:
        poses = [(sc.init_R, sc.init_t)]
    else:
        poses = synthetic.hypotheses(sc.gt_R, sc.gt_t, hyp, sc.seed + 5)
    # each problem reads its own copy of the event frame
    own = (lambda t: t.clone()) if hyp > 1 else (lambda t: t)
    probs = [Problem(0, R, t, sc.init_lin, sc.init_ang, sc.delta_tau, prob["W"], prob["H"], prob["f"], prob["f"],
                     own(prob["E"]), own(prob["E_unsigned"]), opt_vel=True) for R, t in poses]
    return BatchedTracker([{"packed": prob["packed"], "n": prob["n"]}], probs, device=device, tuning=tuning)


def time_graph(bt, steps, warmup, flush):
    import torch
    bt.capture(warmup=max(1, warmup))
    for _ in range(warmup):
        bt.graph.replay()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        bt.graph.replay()
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    return sum(times) / len(times)


def run_hypotheses(dev, flush, steps=10, warmup=3):
    """64 pose hypotheses (0-20 cm / 0-10 degrees from ground truth) of one 500k map at
    640x480, 128 views per launch, each hypothesis with its own event frame; iteration time
    and the best hypothesis' error after the timed iterations."""
    from gsevt import pose as gpose
    prob = build_problem("hypotheses-64x2-500k", dev)
    bt = make_tracker(prob, dev, hypotheses=64)
    ms = time_graph(bt, steps, warmup, flush)
    st = bt.states()
    sc = prob["scenario"]
    err_t = [float(np.linalg.norm(st["t"][i] - sc.gt_t)) for i in range(bt.num)]
    err_r = [gpose.rotation_error_deg(st["R"][i], sc.gt_R) for i in range(bt.num)]
    best = int(np.argmin(np.asarray(err_t) + np.radians(err_r)))
    return {"workload": "hypotheses-64x2-500k", "problems": bt.num, "views": 2 * bt.num, "ms_per_iter": ms,
            "problem_iters_per_s": 1000.0 / ms * bt.num, "keys": int(bt.num_keys),
            "iterations_run": int(st["iter"][0]), "best_hypothesis_error_mm": 1000.0 * err_t[best],
            "best_hypothesis_error_deg": err_r[best],
            "l2": "flushed (256 MB write) between timed iterations",
            "tuning": dict(bt.frame.tuning(), source=bt.tuning_source)}


def make_sequences_tracker(dev, count=16, tuning="table"):
    """16 concurrent sequences, each with its own map (log-uniform 50k-1.5M Gaussians,
    seeds 10-25) and resolution (346x260, 640x480, 1280x720 in turn), event windows of
    log-uniform 10k-2M events, all views in one launch per stage.  Returns (tracker,
    total Gaussians, resolutions)."""
    import torch
    from gsevt import synthetic
    from gsevt import pose as gpose
    from gsevt.batched import BatchedTracker, Problem
    from gsevt.engine import GSFrame, MapSpec, ViewSpec, pack_map
    from gsevt.events import event_frames
    rng = np.random.default_rng(10)
    res = [(346, 260), (640, 480), (1280, 720)]
    maps, probs, total = [], [], 0
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(5e4), np.log(1.5e6))))
        W, H = res[i % 3]
        f = 600.0 * W / 640.0
        ne = int(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
        sc = synthetic.Scenario(n, 10 + i, W, H, f, ne)
        m = sc.map
        pk = pack_map(t(m["xyz"]), t(m["opacity"]), t(m["sh"]), scales=t(m["scale"]), rotations=t(m["rot"]))
        cam = sc.camera
        views = [ViewSpec(W, H, 0, R=T[:3, :3], t=T[:3, 3], P=cam.proj, campos=gpose.campos(T[:3, :3], T[:3, 3]),
                          tanfovx=cam.tanfovx, tanfovy=cam.tanfovy) for T in sc.gt_pair()]
        fr = GSFrame([MapSpec(n, packed=pk)], views, channels=1, device=dev)
        fr.render(exact_keys=True)
        a, b = fr.pixels(0)[0].cpu().numpy(), fr.pixels(1)[0].cpu().numpy()
        del fr
        ex, ey, ep, ts = synthetic.synth_events(a, b, ne, 77 + i, delta_tau=sc.delta_tau)
        sig, uns = event_frames(t(ex), t(ey), t(ep), W, H, 9, 1, dev)
        maps.append({"packed": pk, "n": n})
        probs.append(Problem(i, sc.init_R, sc.init_t, sc.init_lin, sc.init_ang, sc.delta_tau, W, H, f, f,
                             sig[0].reshape(-1).contiguous(), uns[0].reshape(-1).contiguous(), opt_vel=True))
        total += n
    return BatchedTracker(maps, probs, device=dev, tuning=tuning), total, res


def run_sequences(dev, flush, steps=10, warmup=3, count=16):
    """The 16 uneven sequences of make_sequences_tracker: time of one iteration of all."""
    bt, total, res = make_sequences_tracker(dev, count)
    ms = time_graph(bt, steps, warmup, flush)
    return {"workload": "sequences-16-uneven", "problems": count, "views": 2 * count, "gaussians_total": total,
            "ms_per_iter": ms, "problem_iters_per_s": 1000.0 / ms * count, "keys": int(bt.num_keys),
            "resolutions": ["%dx%d" % r for r in res], "l2": "flushed (256 MB write) between timed iterations",
            "tuning": dict(bt.frame.tuning(), source=bt.tuning_source)}


def run_sequence_compare(dev, which, frames=200, repeats=3, window_s=0.025):
    """Long-sequence check of the tracker against the reference-structured loop: sequence i
    of the 16-sequence workload (its map size, event count, resolution and trajectory; the
    events are drawn again from a generator seeded 1000 + i) is tracked over `frames`
    windows `repeats` times by BatchedSequenceTracker (alone in its launch) and once by the
    plain per-view Tracker (torch Adam over the drop-in rasterizer, utils/tracker.py's
    loop).  Reports each run's RMS and final drift and the first window whose error
    exceeds 10 mm (not timed against anything; the plain loop takes minutes)."""
    import torch
    from gsevt import synthetic
    from gsevt import pose as gpose
    from gsevt.batched import BatchedSequenceTracker, DEFAULT_LR
    from gsevt.camera import Camera
    from gsevt.engine import GSFrame, MapSpec, ViewSpec, pack_map
    from gsevt.events import EventArray
    from gsevt.renderer import GaussianMap
    from gsevt.tracker import Tracker
    rng = np.random.default_rng(10)
    res = [(346, 260), (640, 480), (1280, 720)]
    params = []
    for i in range(16):
        n = int(np.exp(rng.uniform(np.log(5e4), np.log(1.5e6))))
        ne = int(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
        params.append((n, ne))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    us = int(round(window_s * 1e6))
    out = []
    for i in which:
        n, ne = params[i]
        W, H = res[i % 3]
        f = 600.0 * W / 640.0
        m = synthetic.make_map(n, 10 + i)
        pk = pack_map(t(m["xyz"]), t(m["opacity"]), t(m["sh"]), scales=t(m["scale"]), rotations=t(m["rot"]))
        tr = synthetic.SinusoidTrajectory(10 + i)
        cam = synthetic.PinholeCamera(W, H, f)
        R0, t0 = tr.pose(0.0)
        views = [ViewSpec(W, H, 0, R=R0, t=t0, P=cam.proj, campos=gpose.campos(R0, t0), tanfovx=cam.tanfovx,
                          tanfovy=cam.tanfovy) for _ in range(2)]
        fr = GSFrame([MapSpec(n, packed=pk)], views, channels=1, device=dev)
        gen = torch.Generator(device=dev)
        gen.manual_seed(1000 + i)
        wins = []
        for k in range(frames):
            for j, tau in enumerate((k * window_s, (k + 1) * window_s)):
                fr.set_view_pose(j, *tr.pose(tau))
            fr.render(exact_keys=True)
            x, y, pol = synthetic.synth_events_device(fr.pixels(0)[0], fr.pixels(1)[0], ne, gen)
            wins.append((x.cpu().numpy(), y.cpu().numpy(), pol.cpu().numpy(),
                         np.array([k * us, (k + 1) * us], np.int64)))
        del fr
        R, tt = tr.pose(0.5 * window_s)
        lv, av = tr.velocity(0.5 * window_s)

        def drift(traj):
            et = []
            for k, (_, Rk, tk) in enumerate(traj):
                Rg, tg = tr.pose((k + 0.5) * window_s)
                et.append(float(np.linalg.norm(gpose.campos(Rk, tk) - gpose.campos(Rg, tg))))
            return {"rms_drift_mm": 1e3 * float(np.sqrt(np.mean(np.square(et)))), "final_error_mm": 1e3 * et[-1],
                    "first_window_over_10mm": next((k for k, e in enumerate(et) if e > 0.01), None)}
        row = {"sequence": i, "resolution": "%dx%d" % (W, H), "gaussians": n, "events_per_window": ne, "batched": []}
        for _ in range(repeats):
            seq = BatchedSequenceTracker([{"packed": pk, "n": n}], [(0, W, H, f, f)], device=dev)
            traj = seq.track([(R, tt, lv, av)], [[(w[0], w[1], w[2], w[3], None)] for w in wins])
            row["batched"].append(dict(drift(traj[0]), adam_iterations=int(seq.iterations)))
        cfg = {"Event": {"img_width": W, "img_height": H, "gaussian_kernel_size": 9,
                         "intrinsic": {"data": [f, 0, W / 2, 0, f, H / 2, 0, 0, 1]},
                         "distortion_factors": [0, 0, 0, 0, 0]},
               "Optimizer": {"cam_rot_delta": DEFAULT_LR[0], "cam_trans_delta": DEFAULT_LR[1],
                             "cam_w_delta": DEFAULT_LR[2], "cam_v_delta": DEFAULT_LR[3],
                             "converged_threshold": 1e-4, "max_optim_iter": 200}}
        c = Camera(torch.tensor(R, dtype=torch.float32), torch.tensor(tt, dtype=torch.float32),
                   torch.tensor(av, dtype=torch.float32), torch.tensor(lv, dtype=torch.float32),
                   cam.fovx, cam.fovy, W, H, delta_tau=window_s, device=dev)
        c.fx, c.fy = cam.fx, cam.fy
        ev = [EventArray(w[0], w[1], w[2], np.linspace(w[3][0], w[3][1], len(w[0])).astype(np.int64))
              for w in wins]
        trk = Tracker(cfg, ev, c, GaussianMap.from_synthetic(m, device=dev), None, torch.zeros(3, device=dev), dev)
        row["plain"] = dict(drift(trk.tracking()), adam_iterations=int(trk.iterations))
        out.append(row)
        print(json.dumps(row), flush=True)
    return {"mode": "sequence-compare", "frames": frames, "window_s": window_s, "sequences": out,
            "trajectory": "T(tau) = exp(sin(2 pi 0.2 tau) [0.5 m u, 20 deg k]), u, k unit axes per sequence"}


def run_sequence_tracking(dev, frames=10, count=16, window_s=0.025):
    """16 concurrent sequences tracked frame by frame along their own smooth trajectories:
    maps of 50k-1.5M Gaussians (log-uniform, seeds 10-25), sensors 346x260 / 640x480 /
    1280x720 in turn, event windows of 10k-2M events (log-uniform), ground-truth motion
    T(tau) = exp(sin(2 pi 0.2 tau) [0.5 m u, 20 deg k]) (synthetic.SinusoidTrajectory),
    `frames` consecutive windows of `window_s` each.  The events of every window are drawn
    on the device from grey renders at the window's two end poses (not timed).  Timed:
    BatchedSequenceTracker.track over all frames (per frame: constant-velocity prediction,
    event pyramid, three pyramid levels of coarse / fine Adam stages with slope
    convergence, all sequences in lockstep, weighted velocity after five frames).
    Reports tracked frames/s over all sequences and the RMS drift against the trajectory
    at the window centres."""
    import torch
    from gsevt import synthetic
    from gsevt import pose as gpose
    from gsevt.batched import BatchedSequenceTracker
    from gsevt.engine import GSFrame, MapSpec, ViewSpec, pack_map
    rng = np.random.default_rng(10)
    res = [(346, 260), (640, 480), (1280, 720)]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(77)
    maps, cams, trajs, counts = [], [], [], []
    windows = [[None] * count for _ in range(frames)]
    us = int(round(window_s * 1e6))
    total = 0
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(5e4), np.log(1.5e6))))
        W, H = res[i % 3]
        f = 600.0 * W / 640.0
        ne = int(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
        m = synthetic.make_map(n, 10 + i)
        pk = pack_map(t(m["xyz"]), t(m["opacity"]), t(m["sh"]), scales=t(m["scale"]), rotations=t(m["rot"]))
        maps.append({"packed": pk, "n": n})
        cams.append((i, W, H, f, f))
        tr = synthetic.SinusoidTrajectory(10 + i)
        trajs.append(tr)
        counts.append(ne)
        total += n
        cam = synthetic.PinholeCamera(W, H, f)
        R0, t0 = tr.pose(0.0)
        views = [ViewSpec(W, H, 0, R=R0, t=t0, P=cam.proj, campos=gpose.campos(R0, t0), tanfovx=cam.tanfovx,
                          tanfovy=cam.tanfovy) for _ in range(2)]
        fr = GSFrame([MapSpec(n, packed=pk)], views, channels=1, device=dev)
        for k in range(frames):
            for j, tau in enumerate((k * window_s, (k + 1) * window_s)):
                fr.set_view_pose(j, *tr.pose(tau))
            fr.render(exact_keys=True)
            x, y, p = synthetic.synth_events_device(fr.pixels(0)[0], fr.pixels(1)[0], ne, gen)
            windows[k][i] = (x, y, p, np.array([k * us, (k + 1) * us], np.int64), None)
        del fr
    init = []
    for tr in trajs:
        R, tt = tr.pose(0.5 * window_s)
        lv, av = tr.velocity(0.5 * window_s)
        init.append((R, tt, lv, av))
    seq = BatchedSequenceTracker(maps, cams, device=dev)
    torch.cuda.synchronize()
    t_start = time.perf_counter()
    traj = seq.track(init, windows)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_start
    drift_t, drift_r, final_t = [], [], []
    for i, tr in enumerate(trajs):
        et, er = [], []
        for k, (stamp, R, tt) in enumerate(traj[i]):
            Rg, tg = tr.pose((k + 0.5) * window_s)
            # camera centres (world frame) and relative rotation
            et.append(float(np.linalg.norm(gpose.campos(R, tt) - gpose.campos(Rg, tg))))
            er.append(gpose.rotation_error_deg(R, Rg))
        drift_t.append(float(np.sqrt(np.mean(np.square(et)))))
        drift_r.append(float(np.sqrt(np.mean(np.square(er)))))
        final_t.append(et[-1])
    return {"workload": "sequences-16-uneven-tracking", "sequences": count, "frames": frames,
            "window_s": window_s, "gaussians_total": total, "events_per_window": counts,
            "resolutions": ["%dx%d" % r for r in res], "wall_s": wall,
            "tracked_frames_per_s": count * frames / wall, "adam_iterations": int(seq.iterations),
            "problem_iterations": int(sum(seq.problem_iterations)),
            "rms_drift_mm": [1e3 * v for v in drift_t], "rms_drift_deg": drift_r,
            "mean_rms_drift_mm": 1e3 * float(np.mean(drift_t)), "mean_rms_drift_deg": float(np.mean(drift_r)),
            "final_error_mm": [1e3 * v for v in final_t],
            "trajectory": "T(tau) = exp(sin(2 pi 0.2 tau) [0.5 m u, 20 deg k]), u, k unit axes per sequence"}


def graph_kernel_count(bt):
    """Kernel launches in one batched iteration, counted as the kernel nodes of a CUDA graph
    capture of it (captured, not run; driver cuGraphGetNodes / cuGraphNodeGetType), or None
    when this torch cannot keep the captured graph."""
    import ctypes as C
    import torch
    try:
        g = torch.cuda.CUDAGraph(keep_graph=True)
    except TypeError:
        return None
    try:
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.graph(g, stream=s):
            bt.step()
        raw = C.c_void_p(g.raw_cuda_graph())
        cu = C.CDLL("libcuda.so.1")
        n = C.c_size_t(0)
        if cu.cuGraphGetNodes(raw, None, C.byref(n)) != 0:
            return None
        nodes = (C.c_void_p * n.value)()
        if cu.cuGraphGetNodes(raw, nodes, C.byref(n)) != 0:
            return None
        kernels = 0
        for i in range(n.value):
            t = C.c_int(-1)
            if cu.cuGraphNodeGetType(C.c_void_p(nodes[i]), C.byref(t)) != 0:
                return None
            kernels += int(t.value == 0)  # CU_GRAPH_NODE_TYPE_KERNEL
        return kernels
    except Exception:
        return None
    finally:
        torch.cuda.synchronize()


def tune_workloads(names, iters=20, out=None):
    """Autotune the launch choices of each named workload on this GPU (gsevt.tuner) and
    write the table; prints one JSON line per workload."""
    import torch
    from gsevt import tuner
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    table = tuner.load_table(out or tuner.TABLE_PATH)
    for name in names:
        if name == "sequences-16-uneven":
            bt, _, _ = make_sequences_tracker(dev, tuning="defaults")
        else:
            bt = make_tracker(build_problem(name, dev), dev, tuning="defaults")
        best, ms, trials = tuner.tune(bt, iters=iters, flush=flush)
        tuner.record(table, bt.frame.L, best, ms, trials, workload=name,
                     device=torch.cuda.get_device_name(dev))
        tuner.save_table(table, out or tuner.TABLE_PATH)
        print(json.dumps({"mode": "tune", "workload": name, "key": tuner.shape_key(bt.frame.L), "choice": best,
                          "ms_per_iter": ms, "trials": [{"choice": c, "ms": t} for c, t in trials]}))
        del bt
        torch.cuda.empty_cache()


def stage_times(bt, reps=5):
    """CUDA-event time of each stage of one iteration (no graph), median over reps."""
    import ctypes as C
    import torch
    from gsevt._lib import lib, check
    from gsevt.engine import _ptr, _stream
    fr = bt.frame
    names = ["preprocess_fwd", "bin_and_sort", "blend_fwd", "loss", "blend_bwd", "preprocess_bwd", "finalize"]
    acc = {k: [] for k in names}
    for _ in range(reps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
        ev[0].record()
        fr.preprocess(); ev[1].record()
        fr.bin_and_sort(0); ev[2].record()
        fr.blend(); ev[3].record()
        fr.loss(bt.loss); ev[4].record()
        fr.blend_backward(); ev[5].record()
        fr.preprocess_backward(None); ev[6].record()
        # finalize through the full step would redo the stages; time the step minus the rest
        ev[7].record()
        torch.cuda.synchronize()
        for i, k in enumerate(names[:-1]):
            acc[k].append(ev[i].elapsed_time(ev[i + 1]))
    return {k: statistics.median(v) for k, v in acc.items() if v}


def algorithmic_bytes(bt, prob):
    """Compulsory HBM bytes per launch of each stage (counts read from the device)."""
    import torch
    from gsevt import _lib
    fr = bt.frame
    st, K = fr.status()
    n = prob["n"]
    V = fr.L.num_views
    off = _lib.workspace_offsets(fr.L)["bin"]
    binv = fr.workspace[off:off + 16 * fr.L.num_vg].view(torch.int32).view(-1, 4)
    nvis = int((binv[:, 0] > 0).sum().item())
    P = fr.L.total_pixels
    passes = (fr.L.sort_bits - 32 + 7) // 8  # tile-sort passes over the pairs
    maps = len(fr.maps)
    return {
        # attributes once per map (232 B), per (view, Gaussian) 16 B bin record, 32 B blend
        # record; compaction + 4 depth-sort passes over the visible slots (8 B each way)
        "preprocess_fwd": 232 * n * maps + 16 * n * V + 32 * nvis + 16 * nvis * 5,
        # duplication: bin 16 B per visible slot, 8 B per pair written; each tile-sort pass
        # reads and writes 8 B per pair; histogram 4 B per pair; ranges 8 B per pair
        "bin_and_sort": 16 * nvis + 8 * K + 16 * K * passes + 4 * K + 8 * K,
        # per key: 4 B value + 32 B record gather; per pixel 8 B written
        "blend_fwd": 36 * K + 8 * P,
        "loss": 12 * P,
        # gather as forward, per pixel 12 B read, per visible slot 32 B gradient accumulation
        "blend_bwd": 36 * K + 12 * P + 32 * nvis,
        "preprocess_bwd": 232 * n * maps + 16 * n * V + 32 * nvis,
        "counts": {"keys": K, "visible_slots": nvis, "pixels": P, "views": V, "tile_sort_passes": passes,
                   "depth_sort_passes": 4},
    }


def iteration_bytes(prob, device):
    """Canonical compulsory bytes of one tracking iteration (the same formula for the plain
    and the batched path): 236 N M + 236 U + sum over views of (8 N + 88 N_v + 108 K_v +
    24 P_v) + 20 P per pair, with N_v, K_v and U from the reference's 3-sigma binning of
    the two views at the starting pose (a frame without render pairs bins that way)."""
    import torch
    from gsevt import _lib
    from gsevt import pose as gpose
    from gsevt.engine import GSFrame, MapSpec, ViewSpec
    sc = prob["scenario"]
    cam = sc.camera
    views = []
    for T in gpose.pair_poses(sc.init_R, sc.init_t, sc.init_lin, sc.init_ang, sc.delta_tau):
        R, t = T[:3, :3], T[:3, 3]
        views.append(ViewSpec(prob["W"], prob["H"], 0, R=R, t=t, P=cam.proj, campos=gpose.campos(R, t),
                              tanfovx=cam.tanfovx, tanfovy=cam.tanfovy))
    n = prob["n"]
    fr = GSFrame([MapSpec(n, packed=prob["packed"])], views, channels=1, device=device)
    fr.render(exact_keys=True)
    off = _lib.workspace_offsets(fr.L)["bin"]
    touched = fr.workspace[off:off + 16 * fr.L.num_vg].view(torch.int32).view(-1, 4)[:, 0].view(len(views), n)
    vis = touched > 0
    nv = int(vis.sum().item())
    u = int(vis.any(dim=0).sum().item())
    K = int(fr.num_keys)
    P = fr.L.total_pixels
    b = 236 * n + 236 * u + 8 * n * len(views) + 88 * nv + 108 * K + 24 * P + 20 * (P // 2)
    return {"bytes_per_iter": b, "gaussians": n, "visible_any_view": u, "visible_slots": nv, "keys_3sigma": K,
            "pixels": P}


def time_batched(bt, steps, warmup, flush):
    import torch
    bt.capture(warmup=max(1, warmup))
    for _ in range(warmup):
        bt.graph.replay()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush.zero_()  # write a buffer larger than L2 between timed iterations
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        bt.graph.replay()
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    return times


def time_e2e(bt, prob, steps, warmup):
    """Public-API iteration with host buffers: per step, H2D of the event frame from pinned
    memory, the iteration, and D2H of the pose states (pose, velocity, loss and gradient of
    every problem: the step's result).  The pose state itself stays on the device from
    step to step, as in tracking."""
    import torch
    E_host = prob["E"].cpu().pin_memory()
    S_out = torch.empty_like(bt.state, device="cpu").pin_memory()
    ev_dev = bt.problems[0].event_signed
    h2d = E_host.numel() * E_host.element_size()
    d2h = S_out.numel() * S_out.element_size()

    def one():
        ev_dev.copy_(E_host, non_blocking=True)
        bt.graph.replay()
        S_out.copy_(bt.state, non_blocking=True)

    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        one()
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / steps
    return ms, h2d, d2h


def time_plain(prob, device, iters=8, warmup=3):
    """The plain per-view drop-in path: reference-structured iteration (RenderFrame with two
    rasterizer calls, torch grey / normalisation / loss, autograd, torch Adam, update_vwRT)."""
    import torch
    from gsevt.camera import Camera
    from gsevt.renderer import GaussianMap
    from gsevt.tracker import make_optimizer, plain_iteration
    sc = prob["scenario"]
    cam = sc.camera
    c = Camera(torch.tensor(sc.init_R, dtype=torch.float32), torch.tensor(sc.init_t, dtype=torch.float32),
               torch.tensor(sc.init_ang, dtype=torch.float32), torch.tensor(sc.init_lin, dtype=torch.float32),
               cam.fovx, cam.fovy, cam.width, cam.height, delta_tau=sc.delta_tau, device=device)
    c.fx, c.fy = cam.fx, cam.fy
    gm = GaussianMap.from_synthetic(prob["map"], device=device)
    lrs = {"cam_rot_delta": 0.004, "cam_trans_delta": 0.004, "cam_w_delta": 0.002, "cam_v_delta": 0.002}
    opt = make_optimizer(c, lrs)
    bg = torch.zeros(3, device=device)
    E = prob["E"].view(1, prob["H"], prob["W"])
    for _ in range(warmup):
        plain_iteration(c, gm, bg, opt, 0, True, E, None)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(iters):
        plain_iteration(c, gm, bg, opt, 0, True, E, None)
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) * 1000.0 / iters


def cpu_iteration(prob, poses=None):
    """One tracking iteration of the pair on the host with the oracle (FP32 forward of both
    views, FP64 loss and adjoint along the frozen contributor lists, exact chain)."""
    from oracle import oracle
    from oracle import pose as opose
    sc = prob["scenario"]
    m = prob["map"]
    W, H = prob["W"], prob["H"]
    cam = sc.camera
    cov = oracle.cov3d(m["scale"], m["rot"])
    E = prob["E_np"]
    Tl, Tn = opose.pair_poses(sc.init_R, sc.init_t, sc.init_lin, sc.init_ang, sc.delta_tau)
    recs = []
    for T in (Tl, Tn):
        v = opose.view_vector(T[:3, :3], T[:3, 3], W, H, prob["f"], prob["f"], np.float64)
        r = oracle.rasterize_view(m["xyz"], cov, m["sh"], m["opacity"], v.astype(np.float32), W, H, [0.0], nch=1,
                                  record=True)
        recs.append((r, v))
    L, gn, gl = oracle.loss(recs[0][0]["image"][0], recs[1][0]["image"][0], E, False, grads=True)
    gx = []
    for (r, v), g in zip(recs, (gl, gn)):
        x, _ = oracle.frozen_backward(r, m["xyz"], m["opacity"], v, W, H, [0.0], 1, g.reshape(1, H, W),
                                      sh=m["sh"], cov_pre=cov)
        gx.append(x)
    return opose.chain_pose_gradient(gx[0], gx[1], sc.init_lin, sc.init_ang, sc.delta_tau), L


def cpu_baseline(prob, budget_s=30.0):
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    prob["E_np"] = prob["E"].cpu().numpy()
    t0 = time.perf_counter()
    cpu_iteration(prob)
    dt = time.perf_counter() - t0
    iters = 1
    while time.perf_counter() - t0 + dt < budget_s and iters < 3:
        cpu_iteration(prob)
        iters += 1
    total = time.perf_counter() - t0
    return {"value": iters / total, "unit": "iters/s", "cores": int(os.environ["OMP_NUM_THREADS"]),
            "kind": "port",
            "sample": "%d full tracking iteration(s) of the 640x480 pair at %d Gaussians (oracle: FP32 forward, "
                      "FP64 adjoint), %.1f s" % (iters, prob["n"], total)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch
    name = args.workload
    os.environ["OMP_NUM_THREADS"] = str(os.cpu_count())
    # the reference arm never touches the GPU: build the same seeded problem on the host
    from gsevt import synthetic
    from oracle import oracle
    from oracle import pose as opose
    n, seed, W, H, f, n_events, hyp = WORKLOADS[name]
    sc = synthetic.Scenario(n, seed, W, H, f, n_events)
    m = sc.map
    cov = oracle.cov3d(m["scale"], m["rot"])
    imgs = []
    for T in sc.gt_pair():
        v = opose.view_vector(T[:3, :3], T[:3, 3], W, H, f, f, np.float32)
        imgs.append(oracle.rasterize_view(m["xyz"], cov, m["sh"], m["opacity"], v, W, H, [0.0], nch=1)["image"][0])
    ex, ey, ep, ts = synthetic.synth_events(imgs[0], imgs[1], n_events, seed + 77, delta_tau=sc.delta_tau)
    E, _, _ = oracle.event_frame(W, H, ex, ey, ep, 9)
    prob = dict(scenario=sc, map=m, n=n, W=W, H=H, f=f, E_np=E)
    budget = 150.0
    t_start = time.perf_counter()
    for _ in range(min(args.warmup, 1)):
        cpu_iteration(prob)
    done, t0 = 0, time.perf_counter()
    per = None
    while done < args.steps:
        cpu_iteration(prob)
        done += 1
        per = (time.perf_counter() - t0) / done
        if time.perf_counter() - t_start + per > budget:
            break
    total = time.perf_counter() - t0
    val = done / total
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "iters/s", "n_gpus": args.gpus,
            "steps": done, "warmup": min(args.warmup, 1), "ms_per_step": 1000.0 * total / done,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": name, "gaussians": n, "width": W, "height": H,
                                             "events": n_events},
            "cpu_baseline": {"value": val, "unit": "iters/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "%d full iteration(s) of the %s pair on the oracle restatement "
                                       "(the reference rasterizer's native source is absent)" % (done, name)},
            "e2e": {"value": val, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_profile(args):
    import torch
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    prob = build_problem(args.workload, dev)
    bt = make_tracker(prob, dev)
    torch.cuda.synchronize()
    for _ in range(args.warmup + args.steps):
        bt.step()
    torch.cuda.synchronize()
    st, k = bt.check_status()
    print(json.dumps({"mode": "profile", "workload": args.workload, "iterations": args.warmup + args.steps,
                      "keys": k, "status": st}))


def run_profile_plain(args):
    """The plain per-view drop-in path for a launch list: warmup + steps iterations of the
    reference-structured loop (two rasterizer calls, torch grey / loss / autograd / Adam),
    with each iteration's wall time and GPU time (CUDA events around it) printed, so that
    the host share of an iteration can be read beside the kernel times."""
    import torch
    from gsevt.camera import Camera
    from gsevt.renderer import GaussianMap
    from gsevt.tracker import make_optimizer, plain_iteration
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    prob = build_problem(args.workload, dev)
    sc, cam = prob["scenario"], prob["scenario"].camera
    c = Camera(torch.tensor(sc.init_R, dtype=torch.float32), torch.tensor(sc.init_t, dtype=torch.float32),
               torch.tensor(sc.init_ang, dtype=torch.float32), torch.tensor(sc.init_lin, dtype=torch.float32),
               cam.fovx, cam.fovy, cam.width, cam.height, delta_tau=sc.delta_tau, device=dev)
    c.fx, c.fy = cam.fx, cam.fy
    gm = GaussianMap.from_synthetic(prob["map"], device=dev)
    opt = make_optimizer(c, {"cam_rot_delta": 0.004, "cam_trans_delta": 0.004, "cam_w_delta": 0.002,
                             "cam_v_delta": 0.002})
    bg = torch.zeros(3, device=dev)
    E = prob["E"].view(1, prob["H"], prob["W"])
    rows = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        a.record()
        plain_iteration(c, gm, bg, opt, 0, True, E, None)
        b.record()
        torch.cuda.synchronize()
        rows.append({"iteration": i, "wall_ms": 1e3 * (time.perf_counter() - t0), "event_ms": a.elapsed_time(b)})
    print(json.dumps({"mode": "profile-plain", "workload": args.workload, "iterations": rows}))


def max_over_ranks(x, device):
    """Largest value of the float x over the ranks of the default process group (x when
    there is none): the job's time is its slowest replica's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(per_rank_iters_per_s, world):
    """Whole-job throughput of `world` independent replicas (weak scaling)."""
    return per_rank_iters_per_s * world


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gsevt", choices=["gsevt", "reference"])
    ap.add_argument("--workload", default="adjoint-500k-640x480", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the 64-hypothesis and 16-sequence workloads reported beside the headline")
    ap.add_argument("--sequence-frames", type=int, default=10,
                    help="frames each of the 16 sequences tracks in the sequence-tracking workload")
    ap.add_argument("--compare-sequences", default="9,15",
                    help="with --mode sequence-compare: indices of the 16 sequences to track with both loops")
    ap.add_argument("--tune-workload", action="append", default=None,
                    help="with --mode tune: workloads to tune (default: the headline, the 64 hypotheses and "
                         "the 16 sequences)")
    ap.add_argument("--mode", default="bench",
                    choices=["bench", "profile", "profile-plain", "sequence-tracking", "sequence-compare", "tune"],
                    help="profile: build the workload, then run warmup + steps un-graphed iterations "
                         "(for ncu launch lists; prints no timings)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "profile":
        return run_profile(args)
    if args.mode == "profile-plain":
        return run_profile_plain(args)
    if args.mode == "tune":
        return tune_workloads(args.tune_workload or ["adjoint-500k-640x480", "hypotheses-64x2-500k",
                                                     "sequences-16-uneven"])
    if args.mode == "sequence-compare":
        import torch
        torch.cuda.set_device(0)
        which = [int(x) for x in args.compare_sequences.split(",") if x.strip()]
        print(json.dumps(run_sequence_compare(torch.device("cuda", 0), which, frames=args.sequence_frames)))
        return
    if args.mode == "sequence-tracking":
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(run_sequence_tracking(torch.device("cuda", 0), frames=args.sequence_frames)))
        return

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    warmup = max(3, args.warmup)
    prob = build_problem(args.workload, dev, seed_offset=rank)
    bt = make_tracker(prob, dev)
    hbm, peak_kind = measured_peaks()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # per-stage times and algorithmic bytes (one un-graphed iteration's stages)
    stages = stage_times(bt)
    algo = algorithmic_bytes(bt, prob)
    top = max(stages, key=lambda k: stages[k])

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local, gpu_uuid(dev))
    clocks.start()
    times = time_batched(bt, args.steps, warmup, flush)
    clk = clocks.stop()
    ms = max_over_ranks(sum(times) / len(times), dev)
    iters_per_s = 1000.0 / ms * bt.num
    value = replica_value(iters_per_s, world)
    e2e_ms, h2d, d2h = time_e2e(bt, prob, max(10, args.steps // 2), 3)
    e2e_ms = max_over_ranks(e2e_ms, dev)
    plain_ms = None if args.no_plain else time_plain(prob, dev)
    st, K = bt.check_status()

    # CUDA-event timing of the dominant stage (its own launch stream), bytes / time
    top_ms = stages[top]
    achieved = algo[top] / (top_ms * 1e-3) / 1e9
    # DRAM traffic needs an ncu capture, which is never taken inside a timed run: null here
    # (the per-launch traffic of the captured build is in the profiles/ summaries)
    traffic = None
    # kernels per iteration of the batched step: preprocess, visible scan and compaction
    # (inside the cooperative sort when it runs), then either one cooperative launch
    # (visible-slot capacity within 8192 keys per SM and at most 256 super-tiles) that
    # sorts by depth and builds the super-tile lists, or the depth sort (cooperative, or a
    # histogram and 4 onesweep passes), sorted sums, paired scan, coarse duplication and
    # the super-tile sort (histogram, passes, + a range kernel when there are two); then
    # tile filter, blend fwd, loss, blend bwd, twist adjoint, finalize
    L = bt.frame.L
    nsup = L.super_tiles if L.super_tiles > 0 else L.total_tiles // 4 + L.num_views + 1
    super_passes = (max(1, int(nsup - 1).bit_length()) + 7) // 8
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    coop_keys = min(sms, 160) * 8192
    coop = L.num_vg <= coop_keys
    compact_launches = 0 if coop and L.num_scan_blocks * 256 <= coop_keys else 2
    if coop and super_passes == 1:
        launches_per_iter = 8 + compact_launches
    else:
        launches_per_iter = 11 + compact_launches + (1 if coop else 5) + super_passes + (1 if super_passes > 1 else 0)
    # the kernel nodes of a captured iteration, counted in the graph itself when torch can
    # keep it (the estimate above otherwise)
    counted = graph_kernel_count(bt)
    launches_source = "estimate from the launch sequence"
    if counted is not None:
        launches_per_iter, launches_source = counted, "kernel nodes of the captured iteration graph"
    it_bytes = iteration_bytes(prob, dev)
    it_gbs = it_bytes["bytes_per_iter"] * (1000.0 / ms) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "gaussians": prob["n"], "width": prob["W"], "height": prob["H"],
                   "events": WORKLOADS[args.workload][5], "hypotheses": bt.num, "views_per_launch": 2 * bt.num,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed (256 MB write) between timed iterations", "path": "batched adjoint, CUDA graph",
                   "tuning": dict(bt.frame.tuning(), source=bt.tuning_source)},
        "e2e": {"value": 1000.0 / e2e_ms * bt.num * world, "unit": "iters/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "plain": None if plain_ms is None else {"value": 1000.0 / plain_ms, "unit": "iters/s", "ms_per_step": plain_ms,
                                                "batched_over_plain": (1000.0 / ms) / (1000.0 / plain_ms)},
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes": algo[top], "stage_ms": stages,
                     "stage_path": "stages run one at a time through the frame API: bin_and_sort is the full "
                                   "tile sort and preprocess_bwd the uncached twist adjoint; the graphed step "
                                   "bins through super-tiles and runs the cached adjoint (its per-kernel times "
                                   "are in the ncu launch list)"},
        "iteration_roofline": dict(it_bytes, achieved=it_gbs, peak=hbm, unit="GB/s", frac=it_gbs / hbm,
                                   note="canonical compulsory bytes of a whole iteration times the "
                                        "batched iterations/s of one GPU, against that GPU's HBM peak"),
        "counts": algo["counts"], "status": st,
        "gpu_launches": launches_per_iter * args.steps,
        "gpu_launches_per_iteration": {"value": launches_per_iter, "source": launches_source},
        "clocks": clk,
    }
    if not args.no_secondary:
        del bt
        torch.cuda.empty_cache()
        line["secondary"] = [run_hypotheses(dev, flush), run_sequences(dev, flush),
                             run_sequence_tracking(dev, frames=args.sequence_frames)]
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(prob)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
