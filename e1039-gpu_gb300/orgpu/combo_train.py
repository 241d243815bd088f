"""Train the combination scorer on the GPU and pick its thresholds.

The candidates are the station-3 (u3, v3) outer iterations of the YZ loop
u3 x v3 x u2 x v2 (reconstruction_kernels.cuh:1320-1461) of every tracklet the
YZ stage queues: or_yz_scored writes one row of 16 features per live outer
iteration.  A row is positive when its outer iteration holds its tracklet's
best combination and the tracklet ends as a global track (or_outer_labels,
after back-track cleaning and global tracking of the plain run).

Training set: the learned-scorer configuration -- 200,000 events with one
dimuon and Poisson(150) noise -- labelled by the plain method on the GPU,
plus --uneven events of the uneven batch under other seeds than the
benchmark's.  The network (16-64-64-1, BF16, the library's forward, backward
and Adam kernels; mini-batch 8,192, lr 1e-3) is trained on nine tenths of the
rows.  The keep threshold is then chosen end to end on held-out events: for
each candidate threshold the plain and the pruned path run on the same
events, and the kept threshold is the highest whose dimuon recall -- the
share of the plain run's dimuons, tracks bit for bit, that the pruned run
reproduces -- reaches --target on the one-dimuon events and on the uneven
ones.  t_unc sets the uncertain band below it: an event where a tracklet's
rows all fall below t_keep but the best reaches t_unc runs plain.

    python -m orgpu.combo_train --events 200000 --uneven 100000 \\
        --out e1039-gpu_gb300/data/combo_scorer_e906.npz
"""
import argparse
import json
import time

import numpy as np

from . import GEOMETRY_E906, _lib, learned, pipeline
from . import layout as L
from . import synth as S
from .scorer_train import device_events


def _torch():
    import torch
    return torch


def collect(rc, cs, geo, cfg, chunk=20000):
    """(features [rows, 16] float32, labels [rows] uint8) on the device for
    cfg's events, labelled by the plain method; and the rows that did not fit."""
    torch = _torch()
    feats, labs = [], []
    rec_all, off_all, _ = S.generate(geo, cfg)
    rec_all, off_all = S.cap_records(rec_all, off_all)
    n = len(off_all) - 1
    lost = 0
    for a in range(0, n, chunk):
        z = min(n, a + chunk)
        rec = rec_all[off_all[a]:off_all[z]]
        off = (off_all[a:z + 1] - off_all[a]).astype(off_all.dtype)
        b, keep_alive = device_events(rc, geo, rec, off)
        orows = learned.OuterRows(b.n)
        cs.plain_with_rows(b, orows)
        rc.sync()
        total = int(orows.rows.item())
        nr = min(total, orows.max_rows)
        lost += total - nr
        feats.append(orows.features[:nr * L.NFEAT].view(nr, L.NFEAT).clone())
        labs.append(orows.labels[:nr].clone())
        del b, orows, keep_alive
        torch.cuda.empty_cache()
    return torch.cat(feats), torch.cat(labs), lost


def evaluate(rc, cs, geo, cfg, sp, thresholds, band, steps=2):
    """Plain vs pruned on cfg's events for each keep threshold: track and
    dimuon recall, extra tracks, uncertain events, the device time of each
    path (ms per batch, median of `steps`) and the share of rows kept."""
    torch = _torch()
    rec, off, _ = S.generate(geo, cfg)
    rec, off = S.cap_records(rec, off)
    b0, keep0 = device_events(rc, geo, rec, off)
    n = b0.n
    hits = [t.clone() for t in (b0.nhits_cham, b0.hits_cham, b0.nhits_hodo, b0.hits_hodo, b0.nhits_prop,
                                b0.hits_prop)]
    bp = pipeline.DeviceBatch(n)
    bl = pipeline.DeviceBatch(n)
    orows = learned.OuterRows(n)
    model = learned.DeviceModel(sp)
    tracklets = learned.Learned(rc)

    def reset(b):
        for dst, src in zip((b.nhits_cham, b.hits_cham, b.nhits_hodo, b.hits_hodo, b.nhits_prop, b.hits_prop), hits):
            dst.copy_(src)

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, b):
        ts = []
        for _ in range(steps):
            reset(b)
            ev0.record()
            fn(b)
            ev1.record()
            rc.sync()
            ts.append(ev0.elapsed_time(ev1))
        return float(np.median(ts))

    t_plain = timed(rc.run_batch, bp)
    out = []
    for t_keep in thresholds:
        t_unc = max(0.0, t_keep - band)
        t_pruned = timed(lambda b: cs.run_batch(b, orows, model, t_keep, t_unc), bl)
        n_ref, n_match, n_new = tracklets.agreement(bp, bl)
        nr = orows.n_rows()
        kept = float((orows.scores[:nr] >= t_keep).float().mean().item()) if nr else 1.0
        unc = int(orows.uncertain[:n].sum().item())
        d_ref, d_rep, d_new, dt_ref, dt_rep = learned.dimuon_agreement(rc, bp, bl)
        out.append({"t_keep": t_keep, "t_unc": t_unc, "events": n, "plain_tracks": n_ref, "reproduced": n_match,
                    "pruned_tracks": n_new, "recall": n_match / n_ref if n_ref else 1.0,
                    "plain_dimuons": d_ref, "dimuons_reproduced": d_rep, "pruned_dimuons": d_new,
                    "dimuon_recall": d_rep / d_ref if d_ref else 1.0, "rows": nr, "rows_kept": kept,
                    "uncertain_events": unc, "plain_ms": t_plain, "pruned_ms": t_pruned,
                    "speedup": t_plain / t_pruned})
    del keep0
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--events", type=int, default=200000)
    ap.add_argument("--uneven", type=int, default=100000)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--pos-weight", type=float, default=20.0)
    ap.add_argument("--target", type=float, default=0.995, help="dimuon recall the keep threshold must reach")
    ap.add_argument("--band", type=float, default=0.002, help="uncertain band below t_keep (events run plain)")
    ap.add_argument("--eval-events", type=int, default=20000)
    ap.add_argument("--seed", type=int, default=906013)
    ap.add_argument("--out", default=learned.MODEL_COMBO_E906)
    ap.add_argument("--report", default=None)
    args = ap.parse_args()
    torch = _torch()

    plane, wp = _lib.geometry_load(GEOMETRY_E906)
    geo = S.Geometry(plane, wp)
    rc = pipeline.Reconstruction(plane, 0)
    cs = learned.ComboScorer(rc)
    t0 = time.time()
    X, y, lost = collect(rc, cs, geo, S.config_small(args.events, args.seed))
    if args.uneven:
        Xu, yu, lu = collect(rc, cs, geo, S.config_uneven(args.uneven, args.seed + 7))
        X, y, lost = torch.cat([X, Xu]), torch.cat([y, yu]), lost + lu
    t_collect = time.time() - t0
    n = int(y.numel())
    rng = np.random.default_rng(args.seed)
    perm = torch.from_numpy(rng.permutation(n).astype(np.int64)).to(X.device)
    trn = perm[n // 10:]
    sample = X[trn[:min(len(trn), 2_000_000)]].double()
    mean = sample.mean(0).float().cpu().numpy()
    std = sample.std(0).float().cpu().numpy()
    inv_std = np.where(std > 1e-6, 1.0 / np.maximum(std, 1e-6), 1.0).astype(np.float32)
    sp = learned.ScorerParams.init(mean, inv_std, seed=args.seed)
    Xt = X[trn].contiguous().view(-1)
    yt = y[trn].contiguous()
    del X
    tr = learned.Trainer(learned.Learned(rc), sp, Xt, yt, batch=args.batch, lr=args.lr, pos_weight=args.pos_weight)
    t1 = time.time()
    losses = [tr.epoch(rng) for _ in range(args.epochs)]
    rc.sync()
    t_train = time.time() - t1
    sp = tr.result()
    del Xt, yt, tr
    torch.cuda.empty_cache()
    # thresholds, end to end on held-out events
    grid = [0.002, 0.005, 0.01, 0.02, 0.03, 0.05, 0.08, 0.12, 0.2]
    ev_small = evaluate(rc, cs, geo, S.config_small(args.eval_events, args.seed + 100), sp, grid, args.band)
    ev_uneven = evaluate(rc, cs, geo, S.config_uneven(args.eval_events, args.seed + 200), sp, grid, args.band)
    ok = [k for k in range(len(grid)) if ev_small[k]["dimuon_recall"] >= args.target and
          ev_uneven[k]["dimuon_recall"] >= args.target]
    k = max(ok) if ok else 0
    sp.t_keep = grid[k]
    sp.t_unc = max(0.0, grid[k] - args.band)
    sp.meta = {"candidates": "live (u3, v3) outer iterations of the queued YZ tracklets", "rows": n,
               "rows_not_stored": lost, "positive_share": float(y.float().mean().item()),
               "train_events_small": args.events, "train_events_uneven": args.uneven, "epochs": args.epochs,
               "batch": args.batch, "lr": args.lr, "pos_weight": args.pos_weight, "target_dimuon_recall": args.target,
               "band": args.band, "collect_s": round(t_collect, 1), "train_s": round(t_train, 2),
               "loss_first": losses[0], "loss_last": losses[-1], "chosen": k,
               "eval_small": ev_small, "eval_uneven": ev_uneven}
    sp.save(args.out)
    print(json.dumps({key: v for key, v in sp.meta.items() if not key.startswith("eval")}, indent=1))
    for name, ev in (("small", ev_small), ("uneven", ev_uneven)):
        for r in ev:
            print(name, json.dumps({key: (round(v, 4) if isinstance(v, float) else v) for key, v in r.items()}))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(sp.meta, f, indent=1)


if __name__ == "__main__":
    main()
