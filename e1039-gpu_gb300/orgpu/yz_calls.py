"""The YZ stage on its own, for profiling its kernels: on the seeded uneven
batch, after the device packer, the event reducer and XZ, one plain call
(or_yz), one with every combination-scorer row pruned and one at a keep
threshold (or_yz_scored), each from the same XZ tracklets, then the device
times of the three (CUDA events).

    python -m orgpu.yz_calls --events 100000 [--t-keep 0.02] [--plain-only] [--lib path/to/liborgpu.so]

Under ncu, `--metrics gpu__time_duration.sum` gives every launch of the
three calls in order (the profiles of the YZ kernels are made this way).
"""
import argparse
import json

import numpy as np

from . import GEOMETRY_E906, _lib, learned, pipeline
from . import synth as S


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--events", type=int, default=100000)
    ap.add_argument("--seed", type=int, default=906002)
    ap.add_argument("--t-keep", type=float, default=0.02)
    ap.add_argument("--plain-only", action="store_true")
    ap.add_argument("--lib", default=None, help="a build of the library (default: the package's)")
    args = ap.parse_args()
    import torch
    lib = _lib.load(args.lib) if args.lib else None
    plane, wp = _lib.geometry_load(GEOMETRY_E906)
    geo = S.Geometry(plane, wp)
    rec, off, _ = S.generate(geo, S.config_uneven(args.events, args.seed))
    rec, off = S.cap_records(rec, off)
    n = len(off) - 1
    rc = pipeline.Reconstruction(plane, 0, lib=lib)
    b = pipeline.DeviceBatch(n)
    d_rec = torch.from_numpy(rec.view(np.uint8)).cuda()
    d_off = torch.from_numpy(off).cuda()
    d_wp = torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda()
    rc.pack(b, d_rec, d_off, d_wp)
    b.ntracklets.zero_()
    rc.event_reduce(b)
    rc.xz_tracking(b)
    rc.sync()
    xz = (b.ntracks.clone(), b.tracks.clone())
    calls = [("plain", lambda: rc.yz_tracking(b))]
    if not args.plain_only:
        cs = learned.ComboScorer(rc)
        model = learned.DeviceModel(learned.ScorerParams.load(learned.MODEL_COMBO_E906))
        rows = learned.OuterRows(n)
        calls += [("all_rows_pruned", lambda: cs.yz(b, rows, model, 2.0, 1.5)),
                  ("t_keep", lambda: cs.yz(b, rows, model, args.t_keep, args.t_keep))]
    out = {"events": n}
    for name, fn in calls:
        b.ntracks.copy_(xz[0])
        b.tracks.copy_(xz[1])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        rc.sync()
        out[name + "_ms"] = e0.elapsed_time(e1)
    print(json.dumps(out))
    rc.close()


if __name__ == "__main__":
    main()
