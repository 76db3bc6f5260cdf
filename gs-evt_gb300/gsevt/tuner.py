"""Autotuner of the launch choices of a batched tracking frame (gsevt_tuning).

The choices are independent of the results (every combination renders the same images
and losses bit for bit; gradients differ only by FP32 atomic order), so the tuner only
measures speed: for a BatchedTracker it times one graph-captured Adam iteration under each
candidate with CUDA events (median over `iters` replays, a buffer larger than L2 written
between them) and keeps the fastest.  The search is a coordinate descent from the library
defaults over

    blend_staging    1 (cp.async per thread) | 2 (TMA tile::gather4 issued by one warp) |
                     3 (TMA tile::gather4 issued by every warp)
    depth_sort_kpt   4 | 8 | 12   keys per thread of the onesweep depth sort
    pair_sort_kpt    4 | 8 | 12   keys per thread of the onesweep (super-)tile sorts
    coop_sort        0 (one cooperative launch when the sort fits) | 1 (never)
    blend_schedule   0 (one block per tile) | 1 (resident blocks, one longest-first tile queue)
    adjoint_pixels   2 (two pixels per lane of the tracker adjoint) | 1 (one pixel per lane)
    forward_pixels   2 (two pixels per lane of the grey forward blend) | 1 (one pixel per lane)

(14 timings per pass, two passes).  Choices that a frame cannot use (the cooperative sort
of a frame above 8192 slots per SM, the onesweep passes of a sort that runs cooperatively)
time alike and the defaults are kept for them.

The table maps a workload shape (views, maps, slots, pixels) to its choice; BatchedTracker
loads it read-only (`tuning="table"`, the default) and falls back to the defaults for an
unknown shape.  `python -m gsevt.tuner --workload ...` (or `bench.py --mode tune`) measures
on the current GPU and writes the table.
"""
import json
import os
import statistics

import torch

TABLE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_table.json")
DEFAULTS = {"blend_staging": 1, "depth_sort_kpt": 12, "pair_sort_kpt": 12, "coop_sort": 0, "blend_schedule": 0,
            "adjoint_pixels": 2, "forward_pixels": 2}
SPACE = {"blend_staging": (1, 2, 3), "blend_schedule": (0, 1), "adjoint_pixels": (2, 1), "forward_pixels": (2, 1),
         "depth_sort_kpt": (4, 8, 12), "pair_sort_kpt": (4, 8, 12), "coop_sort": (0, 1)}


def shape_key(layout):
    """Table key of a frame layout: views, maps, (view, Gaussian) slots and pixels."""
    return "v%d-m%d-g%d-p%d" % (layout.num_views, layout.num_maps, layout.num_vg, layout.total_pixels)


def load_table(path=TABLE_PATH):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def lookup(layout, table=None):
    """The tuned choice for this layout's shape, or None."""
    table = load_table() if table is None else table
    e = table.get(shape_key(layout))
    if not e:
        return None
    return {k: int(e["choice"][k]) for k in DEFAULTS if k in e.get("choice", {})}


def time_choice(bt, choice, iters=20, warmup=3, flush=None):
    """Median CUDA-event time (ms) of one graph-captured iteration of `bt` under `choice`.
    The pose state is restored afterwards, so tuning does not advance the tracker."""
    saved = bt.state.clone()
    bt.frame.set_tuning(**choice)
    bt.capture(warmup=1)
    for _ in range(warmup):
        bt.graph.replay()
    torch.cuda.synchronize()
    times = []
    for _ in range(iters):
        if flush is not None:
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        bt.graph.replay()
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    st, _ = bt.frame.status()
    bt.state.copy_(saved)
    bt.graph = None
    if st:
        raise RuntimeError("tuning run reported device status %#x" % st)
    return statistics.median(times)


def tune(bt, space=SPACE, iters=20, passes=2, flush=None, log=None):
    """Coordinate descent over `space` from the defaults; returns (best choice, best ms,
    every timing as a list of (choice, ms))."""
    best = dict(DEFAULTS)
    # the first timing of a tracker also pays for its first capture and the clock ramp:
    # the defaults are timed twice and the faster time is the baseline
    first = time_choice(bt, best, iters, flush=flush)
    best_ms = min(first, time_choice(bt, best, iters, flush=flush))
    trials = [(dict(best), best_ms)]
    for _ in range(passes):
        changed = False
        for knob, values in space.items():
            for v in values:
                if v == best[knob]:
                    continue
                cand = dict(best, **{knob: v})
                ms = time_choice(bt, cand, iters, flush=flush)
                trials.append((dict(cand), ms))
                if log:
                    log("%s -> %.4f ms" % (cand, ms))
                # keep a change only when it is clearly faster than the run-to-run spread
                if ms < best_ms * 0.99:
                    best, best_ms, changed = cand, ms, True
        if not changed:
            break
    bt.frame.set_tuning(**best)
    return best, best_ms, trials


def record(table, layout, choice, ms, trials, workload=None, device=None):
    table[shape_key(layout)] = {"choice": choice, "ms_per_iter": ms, "workload": workload, "device": device,
                                "default_ms": next((t for c, t in trials if c == DEFAULTS), None),
                                "trials": [{"choice": c, "ms": t} for c, t in trials]}
    return table


def save_table(table, path=TABLE_PATH):
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


if __name__ == "__main__":
    import argparse
    import sys
    here = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, here)
    import bench
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", action="append", default=None)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--out", default=TABLE_PATH)
    args = ap.parse_args()
    bench.tune_workloads(args.workload or ["adjoint-500k-640x480"], args.iters, args.out)
