"""The plain-GPU baseline: the reference's own kernels and this library's,
stage by stage, on the same events of the same GB300, with CUDA events on the
launching stream; and, on the way, a parity check of every stage at full batch
size, compared on the device.

Runs on a machine with a GPU and the reference images built by
oracle/ref/build_ref.py (device code compiled from the reference sources,
unchanged).  For each configuration:

  1. generate the events (orgpu/synth.py), keep those inside the reference's
     array bounds (raw chamber hits per plane <= 120, windowed hits and pairs
     <= 100 -- the oracle's domain counters decide, as for the golden
     fixtures);
  2. run this library's chain (ER, XZ, YZ, cleaning, global, selection) on
     chunks of at most 10,000 events -- the reference's struct capacity
     (EstnEvtMax, reconstruction_constants.h:20) -- each stage timed;
  3. give every reference kernel the library's state before that stage
     (device-to-device copies into the reference structs), launch it as the
     reference host does (online_reconstruction.cu:776-933: one block per
     event, 8 threads for the event reducer, 32 for the others), time it and
     compare its output with the library's on the device.

The reference XZ kernel is not run (barriers in divergent code, K:684-807);
the YZ kernels of both sides start from the library's XZ tracklets, and chain
totals are given with and without XZ.  Both reference images are timed:
fmad1 is the reference as its Makefile builds it (nvcc's default
-fmad=true), fmad0 the build the library is bit-exact with.

Output: <out>/ref_timing.json.  Usage:
    python tests/golden/ref_timing.py --out <output directory>
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for p in (REPO, os.path.join(REPO, "e1039-gpu_gb300"), HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

import golden_io as G  # noqa: E402
from oracle import pyoracle as O  # noqa: E402
from orgpu import GEOMETRY_E906, layout as L, synth as S  # noqa: E402

MAX_CHAM_RAW = 120
MAX_WINDOW = 100
CHUNK = L.REF_EVTMAX

STAGES = ["event_reduce", "xz", "yz", "back_clean", "global", "select"]
REF_KEYS = {"event_reduce": ["er"], "yz": ["yz"], "back_clean": ["clean", "clean_x"], "global": ["global"],
            "select": ["prop", "gclean", "gclean_x"]}


def configs(n_uneven):
    return [("small", S.config_small(1000, 906001)),
            ("uneven", S.config_uneven(n_uneven, 906002)),
            ("high_occupancy", S.config_high_occupancy(10000, 906004))]


def in_domain(plane, hits0):
    n = hits0.n
    h2, t2, st2 = hits0.copy(), L.HostTracks(n), O.OracleState(n)
    O.run_all(plane, h2, t2, st2, counted=True)
    c = st2.counts.reshape(n, O.NCOUNTS)
    raw = hits0.nhits_cham.reshape(n, L.NCHAM).max(axis=1)
    return (raw <= MAX_CHAM_RAW) & (c[:, 6] <= MAX_WINDOW) & (c[:, 7] <= MAX_WINDOW)


def hits_mismatch(torch, rk, b, n):
    """Events whose reduced hit lists differ (counts, or any valid field bit)."""
    bad = torch.zeros(n, dtype=torch.bool, device=b.toomany.device)
    for cn, hn, npl, cap in (("nhits_cham", "hits_cham", L.NCHAM, L.MAXHITS_CHAM),
                             ("nhits_hodo", "hits_hodo", L.NHODO, L.MAXHITS_HODO),
                             ("nhits_prop", "hits_prop", L.NPROP, L.MAXHITS_PROP)):
        rc = rk.view(cn, n).view(n, npl)
        oc = getattr(b, cn).view(n, npl)
        bad |= (rc != oc).any(1)
        w = L.NHITSPARAM * cap
        valid = torch.arange(w, device=oc.device)[None, None, :] < (L.NHITSPARAM * oc.clamp(0, cap))[..., None]
        rh = rk.view(hn, n).view(torch.int32).view(n, npl, w)
        oh = getattr(b, hn).view(torch.int32).view(n, npl, w)
        bad |= ((rh != oh) & valid).any(2).any(1)
    return bad


def tracks_mismatch(torch, rk, b, n, toomany):
    """(events with a different slot count or a different discrete field,
    events with any differing bit, max relative difference of a fit field)."""
    ok = toomany == 0
    rn = rk.view("ntracks", n).view(n, L.NSLOTS)
    on = b.ntracks.view(n, L.NSLOTS)
    count_bad = (rn != on).any(1) & ok
    rt = rk.view("tracks", n).view(n, L.NSLOTS, L.SLOTCAP, L.NTRKPARAM)
    ot = b.tracks.view(n, L.NSLOTS, L.SLOTCAP, L.NTRKPARAM)
    k = torch.arange(L.SLOTCAP, device=on.device)
    valid = (k[None, None, :] < on.clamp(0, L.SLOTCAP)[..., None].long()) & ok[:, None, None]
    diff = (rt.view(torch.int32) != ot.view(torch.int32)) & valid[..., None]
    disc = torch.from_numpy(G.DISCRETE_FIELDS).to(on.device)
    disc_bad = diff[..., disc].flatten(1).any(1) | count_bad
    any_bad = diff.flatten(1).any(1) | count_bad
    fit = torch.tensor(G.FIT_FIELDS, device=on.device)
    a, c = rt[..., fit].double(), ot[..., fit].double()
    rel = ((a - c).abs() / c.abs().clamp_min(1e-30))
    rel = torch.where(valid[..., None] & (a != c), rel, torch.zeros_like(rel))
    return int(disc_bad.sum()), int(any_bad.sum()), float(rel.max()) if rel.numel() else 0.0, any_bad


def run_config(torch, plane, geo, rc, images, name, cfg, dump=None, dump_image="fmad0", dump_max=0):
    from orgpu import pipeline
    t0 = time.time()
    rec, off, _ = S.generate(geo, cfg)
    rec, off = S.cap_records(rec, off)
    n_all = len(off) - 1
    keep = np.nonzero(in_domain(plane, S.pack(rec, off, geo.wire_pos_f32())))[0]
    rec, off = G.select_events(rec, off, keep)
    n = len(keep)
    ours = {s: 0.0 for s in STAGES}
    refs = {v: {s: 0.0 for s in REF_KEYS} for v in images}
    par = {v: {"er_events": 0, "er_flag_events": 0, **{s: [0, 0, 0.0] for s in ("yz", "back_clean", "global",
                                                                                 "select")}} for v in images}
    accepted = 0
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for c0 in range(0, n, CHUNK):
        c1 = min(n, c0 + CHUNK)
        m = c1 - c0
        r_c, o_c = G.select_events(rec, off, np.arange(c0, c1))
        hits0 = S.pack(r_c, o_c, geo.wire_pos_f32())
        b = pipeline.DeviceBatch(m)
        calls = {"event_reduce": rc.event_reduce, "xz": rc.xz_tracking, "yz": rc.yz_tracking,
                 "back_clean": rc.back_track_cleaning, "global": rc.global_tracking, "select": rc.selection}
        # warm-up of the library's chain, then the timed chain; the state
        # after every stage is kept on the device for the reference's input
        for rep in range(2):
            b.upload_hits(hits0)
            b.toomany.zero_()
            b.ntracklets.zero_()
            snaps = {}
            for s in STAGES:
                ev[0].record()
                calls[s](b)
                ev[1].record()
                rc.sync()
                if rep == 1:
                    ours[s] += ev[0].elapsed_time(ev[1])
                snaps[s] = {"toomany": b.toomany.clone(), "ntracks": b.ntracks.clone(), "tracks": b.tracks.clone()}
                if s == "event_reduce":
                    hits_er = [t.clone() for t in (b.nhits_cham, b.hits_cham, b.nhits_hodo, b.hits_hodo,
                                                   b.nhits_prop, b.hits_prop)]
        accepted += int((snaps["xz"]["toomany"] == 0).sum())
        for v, rk in images.items():
            rk.set_plane(plane)
            # warm-up: every kernel once on one event (module loading); the
            # tracking kernels see no tracks there, so they read no hits
            rk.timing = None
            rk.put_hits(hits0)
            rk.put_flags(np.zeros(m, np.uint8))
            rk.event_reduce(1)
            rk.view("ntracks", 1).zero_()
            for fn in (rk.yz, rk.back_clean, rk.global_tracking, rk.selection):
                fn(1)
            rk.timing = {}
            # ER on the raw hits
            rk.put_hits(hits0)
            rk.put_flags(np.zeros(m, np.uint8))
            rk.event_reduce(m)
            par[v]["er_events"] += int(hits_mismatch(torch, rk, b_with(b, hits_er), m).sum())
            # the reference's flag also sums uninitialised rows (K:128-133):
            # compare it with the library's only where both are defined
            par[v]["er_flag_events"] += int((rk.view("flags", m) != snaps["event_reduce"]["toomany"]).sum())
            prev = {"yz": "xz", "back_clean": "yz", "global": "back_clean", "select": "global"}
            fns = {"yz": rk.yz, "back_clean": rk.back_clean, "global": rk.global_tracking, "select": rk.selection}
            for s in ("yz", "back_clean", "global", "select"):
                src = snaps[prev[s]]
                for dst, t in zip(("nhits_cham", "hits_cham", "nhits_hodo", "hits_hodo", "nhits_prop", "hits_prop"),
                                  hits_er):
                    rk.view(dst, m).copy_(t)
                rk.view("ntracks", m).copy_(src["ntracks"])
                rk.view("tracks", m).copy_(src["tracks"])
                rk.view("flags", m).copy_(src["toomany"])
                fns[s](m)
                want = b_tracks(b, snaps[s])
                d, a, r, bad = tracks_mismatch(torch, rk, want, m, snaps["xz"]["toomany"])
                if dump is not None and v == dump_image and a:
                    for ie in torch.nonzero(bad).flatten().tolist()[:max(0, dump_max - len(dump[s]))]:
                        dump[s].append({"event": c0 + ie, "records": r_c[o_c[ie]:o_c[ie + 1]].copy(),
                                        "ours_ntracks": want.ntracks.view(m, L.NSLOTS)[ie].cpu().numpy(),
                                        "ours_tracks": want.tracks.view(m, -1)[ie].cpu().numpy(),
                                        "ref_ntracks": rk.view("ntracks", m).view(m, L.NSLOTS)[ie].cpu().numpy(),
                                        "ref_tracks": rk.view("tracks", m).view(m, -1)[ie].cpu().numpy()})
                if s in ("yz", "global"):
                    # the reference again on the same inputs: events where its
                    # two runs disagree (its uninitialised per-thread scratch)
                    first = _View()
                    first.ntracks = rk.view("ntracks", m).clone()
                    first.tracks = rk.view("tracks", m).clone()
                    saved, rk.timing = rk.timing, None
                    rk.view("ntracks", m).copy_(src["ntracks"])
                    rk.view("tracks", m).copy_(src["tracks"])
                    fns[s](m)
                    rk.timing = saved
                    self_bad = tracks_mismatch(torch, rk, first, m, snaps["xz"]["toomany"])[1]
                    par[v]["self_" + s] = par[v].get("self_" + s, 0) + self_bad
                par[v][s][0] += d
                par[v][s][1] += a
                par[v][s][2] = max(par[v][s][2], r)
            for s, keys in REF_KEYS.items():
                refs[v][s] += sum(rk.timing.get(k, 0.0) for k in keys)
            rk.timing = None
        del b
        torch.cuda.empty_cache()
    out = {"generated": n_all, "in_domain": n, "accepted_after_xz": accepted, "seconds": round(time.time() - t0, 1),
           "library_ms": ours}
    for v in images:
        r = refs[v]
        chain = sum(r.values())
        lib_no_xz = sum(ours[s] for s in REF_KEYS)
        out[v] = {"reference_ms": r,
                  "reference_chain_ms_without_xz": chain,
                  "library_chain_ms_without_xz": lib_no_xz,
                  "library_chain_ms": sum(ours.values()),
                  "reference_events_per_s_without_xz": n / (chain / 1000.0) if chain else None,
                  "library_events_per_s": n / (sum(ours.values()) / 1000.0),
                  "speedup_per_stage": {s: (r[s] / ours[s] if ours[s] else None) for s in REF_KEYS},
                  "speedup_chain_without_xz": chain / lib_no_xz if lib_no_xz else None,
                  "reference_run_twice_differing_events": {st: par[v].get("self_" + st, 0) for st in ("yz", "global")},
                  "parity": {"er_hit_mismatch_events": par[v]["er_events"],
                             "er_flag_mismatch_events_raw": par[v]["er_flag_events"],
                             **{s: {"discrete_mismatch_events": par[v][s][0], "any_bit_mismatch_events": par[v][s][1],
                                    "max_rel_fit": par[v][s][2]} for s in ("yz", "back_clean", "global", "select")}}}
    return out


class _View:
    pass


def b_with(b, hits):
    """A DeviceBatch-like view with the given hit tensors."""
    v = _View()
    (v.nhits_cham, v.hits_cham, v.nhits_hodo, v.hits_hodo, v.nhits_prop, v.hits_prop) = hits
    v.toomany = b.toomany
    return v


def b_tracks(b, snap):
    v = _View()
    v.ntracks, v.tracks = snap["ntracks"], snap["tracks"]
    return v


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(REPO, "out", "ref_timing"))
    ap.add_argument("--uneven-events", type=int, default=100000)
    ap.add_argument("--images", default="fmad1,fmad0")
    ap.add_argument("--configs", default="small,uneven,high_occupancy")
    ap.add_argument("--dump", type=int, default=0, help="save up to this many differing events per stage (fmad0)")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    import torch
    from oracle.ref import refrun
    from orgpu import pipeline
    plane, wp = O.parse_geometry(GEOMETRY_E906)
    geo = S.Geometry(plane, wp)
    rc = pipeline.Reconstruction(plane, 0)
    images = {v: refrun.RefKernels(v) for v in args.images.split(",")}
    report = {"device": torch.cuda.get_device_name(0), "chunk_events": CHUNK, "configs": {}}
    for name, cfg in configs(args.uneven_events):
        if name not in args.configs.split(","):
            continue
        dump = {s: [] for s in ("yz", "back_clean", "global", "select")} if args.dump else None
        report["configs"][name] = run_config(torch, plane, geo, rc, images, name, cfg, dump, "fmad0", args.dump)
        if dump is not None and any(dump.values()):
            flat = {}
            for s, lst in dump.items():
                for i, d in enumerate(lst):
                    for k, x in d.items():
                        flat[f"{s}/{i}/{k}"] = np.asarray(x)
            np.savez_compressed(os.path.join(args.out, f"mismatch_{name}.npz"), **flat)
        print(name, json.dumps(report["configs"][name]), flush=True)
    for rk in images.values():
        rk.close()
    with open(os.path.join(args.out, "ref_timing.json"), "w") as f:
        json.dump(report, f, indent=1)


if __name__ == "__main__":
    main()
