"""Train the learned tracklet scorer on the GPU and pick its keep threshold.

Training data: seeded synthetic E906 events labelled by the plain method on
the GPU (a tracklet is positive when it ends as a global track, stationID 6).
The default set is the learned-scorer configuration: 200,000 events with one
dimuon and Poisson(150) noise hits; --uneven adds events of the uneven batch
(0-3 muons, log-normal noise) under other seeds than the benchmark's.

The network is trained by the library's own kernels (or_mlp_gradient +
or_mlp_adam; mini-batch 8,192, Adam, lr 1e-3), the keep threshold is the
highest score threshold that keeps the target share of the positive
tracklets of a held-out tenth, and the result is evaluated end to end: the
plain and the learned path on the same held-out events, recall = share of
the plain run's global tracks the learned run reproduces bit for bit.

    python -m orgpu.scorer_train --events 200000 --uneven 100000 \
        --out e1039-gpu_gb300/data/scorer_e906.npz
"""
import argparse
import json
import time

import numpy as np

from . import GEOMETRY_E906, _lib, learned, pipeline
from . import layout as L
from . import synth as S


def _torch():
    import torch
    return torch


def device_events(rc, geo, rec, off, device=0):
    """A DeviceBatch holding the packed events (device packer)."""
    torch = _torch()
    n = len(off) - 1
    b = pipeline.DeviceBatch(n, device)
    d_rec = torch.from_numpy(rec.view(np.uint8)).cuda(device)
    d_off = torch.from_numpy(off).cuda(device)
    d_wp = torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda(device)
    rc.pack(b, d_rec, d_off, d_wp)
    return b, (d_rec, d_off, d_wp)


def collect(rc, lrn, geo, cfg, chunk=25000):
    """(features [rows, 16], labels [rows]) of cfg's events, labelled by the
    plain method."""
    feats, labs = [], []
    rec_all, off_all, _ = S.generate(geo, cfg)
    rec_all, off_all = S.cap_records(rec_all, off_all)
    n = len(off_all) - 1
    for a in range(0, n, chunk):
        z = min(n, a + chunk)
        rec = rec_all[off_all[a]:off_all[z]]
        off = (off_all[a:z + 1] - off_all[a]).astype(off_all.dtype)
        b, keep_alive = device_events(rc, geo, rec, off)
        r = learned.TrackletRows(b.n)
        lrn.plain_with_rows(b, r)
        rc.sync()
        nr = r.n_rows()
        feats.append(r.features[:nr * L.NFEAT].cpu().numpy().reshape(nr, L.NFEAT))
        labs.append(r.labels[:nr].cpu().numpy())
        del b, r, keep_alive
    return np.concatenate(feats), np.concatenate(labs)


def threshold_for_recall(scores, labels, target):
    """Highest t such that the share of positives with score >= t is at
    least `target`."""
    pos = np.sort(scores[labels == 1])
    if len(pos) == 0:
        return 0.0
    k = int(np.floor((1.0 - target) * len(pos)))
    return float(np.nextafter(pos[k], -np.inf)) if k > 0 else float(np.nextafter(pos[0], -np.inf))


def score_rows(lrn, sp, feats):
    torch = _torch()
    model = learned.DeviceModel(sp)
    fx = torch.from_numpy(np.ascontiguousarray(feats, np.float32).reshape(-1)).cuda()
    out = torch.zeros(len(feats), dtype=torch.float32, device="cuda")
    lrn.score(model, fx, len(feats), out)
    lrn.rc.sync()
    return out.cpu().numpy()


def evaluate(rc, lrn, geo, cfg, sp, steps=2):
    """Plain vs learned on cfg's events: recall, extra tracks, kept share and
    the device time of each path (ms per batch, median of `steps`)."""
    torch = _torch()
    rec, off, _ = S.generate(geo, cfg)
    rec, off = S.cap_records(rec, off)
    b0, keep0 = device_events(rc, geo, rec, off)
    n = b0.n
    hits = [t.clone() for t in (b0.nhits_cham, b0.hits_cham, b0.nhits_hodo, b0.hits_hodo, b0.nhits_prop,
                                b0.hits_prop)]
    bp = pipeline.DeviceBatch(n)
    bl = pipeline.DeviceBatch(n)
    r = learned.TrackletRows(n)
    model = learned.DeviceModel(sp)

    def reset(b):
        for dst, src in zip((b.nhits_cham, b.hits_cham, b.nhits_hodo, b.hits_hodo, b.nhits_prop, b.hits_prop), hits):
            dst.copy_(src)

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_plain, t_learned = [], []
    for _ in range(steps):
        reset(bp)
        ev0.record()
        rc.run_batch(bp)
        ev1.record()
        rc.sync()
        t_plain.append(ev0.elapsed_time(ev1))
        reset(bl)
        ev0.record()
        lrn.run_batch(bl, r, model, sp.t_keep, sp.t_unc)
        ev1.record()
        rc.sync()
        t_learned.append(ev0.elapsed_time(ev1))
    n_ref, n_match, n_new = lrn.agreement(bp, bl)
    nr = r.n_rows()
    kept = float(r.keep[:nr].float().mean().item()) if nr else 1.0
    del keep0
    return {"events": n, "plain_tracks": n_ref, "reproduced": n_match, "learned_tracks": n_new,
            "recall": n_match / n_ref if n_ref else 1.0, "rows": nr, "kept_share": kept,
            "plain_ms": float(np.median(t_plain)), "learned_ms": float(np.median(t_learned)),
            "speedup": float(np.median(t_plain) / np.median(t_learned))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--events", type=int, default=200000)
    ap.add_argument("--uneven", type=int, default=0)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--pos-weight", type=float, default=4.0)
    ap.add_argument("--target", type=float, default=0.999, help="share of positive tracklets kept")
    ap.add_argument("--band", type=float, default=0.0, help="uncertain band below t_keep (events re-run plain)")
    ap.add_argument("--eval-events", type=int, default=20000)
    ap.add_argument("--seed", type=int, default=906003)
    ap.add_argument("--out", default=learned.MODEL_E906)
    ap.add_argument("--report", default=None)
    args = ap.parse_args()
    torch = _torch()

    plane, wp = _lib.geometry_load(GEOMETRY_E906)
    geo = S.Geometry(plane, wp)
    rc = pipeline.Reconstruction(plane, 0)
    lrn = learned.Learned(rc)
    t0 = time.time()
    X, y = collect(rc, lrn, geo, S.config_small(args.events, args.seed))
    if args.uneven:
        Xu, yu = collect(rc, lrn, geo, S.config_uneven(args.uneven, args.seed + 7))
        X, y = np.concatenate([X, Xu]), np.concatenate([y, yu])
    t_collect = time.time() - t0
    rng = np.random.default_rng(args.seed)
    perm = rng.permutation(len(y))
    nval = len(y) // 10
    val, trn = perm[:nval], perm[nval:]
    mean = X[trn].mean(0).astype(np.float32)
    std = X[trn].std(0).astype(np.float32)
    inv_std = np.where(std > 1e-6, 1.0 / np.maximum(std, 1e-6), 1.0).astype(np.float32)
    sp = learned.ScorerParams.init(mean, inv_std, seed=args.seed)
    Xt = torch.from_numpy(np.ascontiguousarray(X[trn]).reshape(-1)).cuda()
    yt = torch.from_numpy(np.ascontiguousarray(y[trn])).cuda()
    tr = learned.Trainer(lrn, sp, Xt, yt, batch=args.batch, lr=args.lr, pos_weight=args.pos_weight)
    t1 = time.time()
    losses = [tr.epoch(rng) for _ in range(args.epochs)]
    rc.sync()
    t_train = time.time() - t1
    sp = tr.result()
    s_val = score_rows(lrn, sp, X[val])
    sp.t_keep = threshold_for_recall(s_val, y[val], args.target)
    sp.t_unc = max(0.0, sp.t_keep - args.band)
    pruned = float(np.mean(s_val < sp.t_unc))
    ev = {"small": evaluate(rc, lrn, geo, S.config_small(args.eval_events, args.seed + 100), sp),
          "uneven": evaluate(rc, lrn, geo, S.config_uneven(args.eval_events, args.seed + 200), sp),
          "high_occupancy": evaluate(rc, lrn, geo, S.config_high_occupancy(args.eval_events, args.seed + 300), sp)}
    sp.meta = {"train_events_small": args.events, "train_events_uneven": args.uneven, "rows": int(len(y)),
               "positive_share": float(y.mean()), "epochs": args.epochs, "batch": args.batch, "lr": args.lr,
               "pos_weight": args.pos_weight, "target_tracklet_recall": args.target,
               "val_pruned_share": pruned, "collect_s": round(t_collect, 1), "train_s": round(t_train, 2),
               "loss_first": losses[0], "loss_last": losses[-1], "eval": ev}
    sp.save(args.out)
    print(json.dumps(sp.meta, indent=1))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(sp.meta, f, indent=1)


if __name__ == "__main__":
    main()
