"""The project's launch-shape autotuner.

Every tunable kernel (or_kernel_id_t) runs one warp per event -- or, for the
dynamically scheduled YZ and global-tracking kernels, per work unit -- and
takes 1, 2, 4, 8 or 16 of them per CTA (CTAs of 32 to 512 threads; XZ at most
8 for its shared memory).  The choice changes timing only, never results
(tests/test_autotune_gpu.py runs the whole chain with every shape and
compares bit for bit), so the tuner only measures: each stage in the chain's
order, on a sample batch of the target workload, every candidate timed with
CUDA events on the stage's own input state (restored from a device copy
before each run), the fastest kept and applied before the next stage is
tuned on its output.

    cfg = autotune.tune(rc, hits, candidates=(1, 2, 4, 8, 16))
    autotune.apply(rc, cfg)          # or_set_launch per kernel
    autotune.save(cfg, "tuned.json"); autotune.apply(rc, autotune.load("tuned.json"))
"""
import json

import numpy as np

from . import _lib, pipeline

STAGES = ("event_reduce", "xz", "yz", "back_clean", "global", "select")


def _torch():
    import torch
    return torch


def set_launch(rc, kernel, warps):
    _lib.check(rc.lib.or_set_launch(rc.ctx, _lib.KERNELS[kernel], int(warps)), "or_set_launch")


def get_launch(rc, kernel):
    return int(rc.lib.or_get_launch(rc.ctx, _lib.KERNELS[kernel]))


def apply(rc, cfg):
    for k, w in cfg["best"].items():
        set_launch(rc, k, w)


def save(cfg, path):
    with open(path, "w") as f:
        json.dump(cfg, f, indent=1)


def load(path):
    with open(path) as f:
        return json.load(f)


def _hits(b):
    return [b.nhits_cham, b.hits_cham, b.nhits_hodo, b.hits_hodo, b.nhits_prop, b.hits_prop]


def _tracks(b):
    return [b.ntracks, b.tracks, b.toomany, b.ntracklets]


def tune(rc, hits, candidates=(1, 2, 4, 8, 16), repeats=3, device=0):
    """Tune every stage on the events of `hits` (a layout.HostHits of the
    target workload, as packed).  Leaves the best shapes applied to `rc` and
    returns {"best": {kernel: warps}, "ms": {kernel: {warps: ms}}, "events": n}."""
    torch = _torch()
    b = pipeline.DeviceBatch(hits.n, device)
    b.upload_hits(hits)
    b.toomany.zero_()
    b.ntracklets.zero_()
    snap_h = [t.clone() for t in _hits(b)]
    snap_t = [t.clone() for t in _tracks(b)]
    calls = {"event_reduce": rc.event_reduce, "xz": rc.xz_tracking, "yz": rc.yz_tracking,
             "back_clean": rc.back_track_cleaning, "global": rc.global_tracking, "select": rc.selection}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    result = {"best": {}, "ms": {}, "events": hits.n, "candidates": list(candidates)}

    def restore():
        for d, s in zip(_hits(b), snap_h):
            d.copy_(s)
        for d, s in zip(_tracks(b), snap_t):
            d.copy_(s)

    for stage in STAGES:
        times = {}
        for w in candidates:
            if stage == "xz" and w > 8:
                continue
            set_launch(rc, stage, w)
            best = float("inf")
            for _ in range(repeats):
                restore()
                ev0.record()
                calls[stage](b)
                ev1.record()
                rc.sync()
                best = min(best, ev0.elapsed_time(ev1))
            times[w] = best
        w_best = min(times, key=times.get)
        set_launch(rc, stage, w_best)
        result["best"][stage] = w_best
        result["ms"][stage] = {str(k): v for k, v in times.items()}
        # the stage's output with the chosen shape is the next stage's input
        restore()
        calls[stage](b)
        rc.sync()
        snap_h = [t.clone() for t in _hits(b)]
        snap_t = [t.clone() for t in _tracks(b)]
    del snap_h, snap_t, b
    return result
