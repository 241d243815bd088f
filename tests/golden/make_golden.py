"""Pin the CPU oracle against the reference's own kernels and write the golden
fixtures the CPU tests check the oracle with.

Runs on a machine with a GPU and the reference images built by
oracle/ref/build_ref.py (device code compiled from the reference sources).
For each image (fmad0: -fmad=false; fmad1: nvcc's default, as the reference
Makefile builds it) every stage the reference can run safely is fed the
oracle's state before that stage (injection), and its output is compared with
the oracle's:

  ER      gkernel_eR on the packed raw hits      -> reduced hit lists, flags
  XZ      xz_pin_kernel (oracle/ref/xz_pin.cuh) on the oracle's reduced hits:
          the XZ candidates computed by the reference's own helpers (hit
          pairing, x at y = 0, both fits, left/right resolution, hodoscope
          matches), compared as per-event multisets with the oracle's
          tracklets, since the reference's XZ kernel itself cannot be run
  YZ      gKernel_YZ_tracking on the oracle's XZ tracklets
  clean   gKernel_BackTrackCleaning + ..._crossthreads on the oracle's YZ output
  global  gKernel_Global_tracking on the oracle's cleaned tracks
  sel     gKernel_PropSegmentMatching + gKernel_GlobalTrackCleaning{,_crossthreads}
          on the oracle's global tracks
  vtx     gKernel_Vertexing on the oracle's selected tracks
  dim     gKernel_DimuonBuilding on the oracle's vertexed tracks
  hist    gKernel_fill_display_histograms on the oracle's tracks and dimuons,
          with seeded trigger words, one event per launch (its "+=" from
          concurrent blocks would lose counts)

The reference XZ kernel itself is not run (barriers in divergent code).
Events are first checked against the reference's array bounds with the oracle's
domain counters; events outside them are not given to the reference.

The library is also built a second time with nvcc's default multiply-add
contraction (build_lib.build(fmad=True), liborgpu_fmad1.so) and its stages,
fed the same oracle states, are compared with the fmad1 image: how close the
library comes to the reference as its Makefile builds it when compiled the
same way ("lib_fmad1" in the report).

Outputs (under --out):
  golden_report.json      per image and stage: events, matches, mismatches
  ref_e906.npz            fixture: the records of a few events per
                          configuration and the reference's output of every
                          stage for them, for both images

Usage: python tests/golden/make_golden.py --out <output directory>
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

# reference array bounds (reconstruction_kernels.cuh)
MAX_CHAM_RAW = 120     # hitarraycopy[600] holds 5 fields of 120 survivors (K:16)
MAX_WINDOW = 100       # hitidx / hitpairs arrays (K:890-903, K:1857-1867)

CONFIGS = [
    # name, config, events, fixture events
    ("small", S.config_small(1000, 906001), 1000, 16),
    ("uneven", S.config_uneven(2000, 906002), 2000, 8),
    ("high_occupancy", S.config_high_occupancy(500, 906004), 500, 8),
]


class Snap:
    """Oracle state after every stage, plus the per-event domain counters."""

    def __init__(self, plane, hits0, trig=None):
        n = hits0.n
        st = O.OracleState(n)
        self.hits0 = hits0
        self.hits_er = hits0.copy()
        O.event_reduce(self.hits_er, st)
        self.toomany_er = st.toomany.copy()
        t = L.HostTracks(n)
        O.xz(plane, self.hits_er, t, st)
        self.toomany_xz = st.toomany.copy()
        self.tracks_xz = t.copy()
        O.yz(plane, self.hits_er, t, st)
        self.tracks_yz = t.copy()
        O.back_clean(t, st)
        self.tracks_clean = t.copy()
        O.global_tracking(plane, self.hits_er, t, st)
        self.tracks_global = t
        ts = t.copy()
        O.prop_matching(plane, self.hits_er, ts, st)
        O.global_clean(ts, st)
        self.tracks_sel = ts
        tv = ts.copy()
        O.vertexing(plane, tv, st)
        self.tracks_vtx = tv
        self.dims = L.HostDimuons(n)
        O.dimuons(plane, tv, self.dims, st)
        self.trig = S.trigger_bits(n) if trig is None else np.asarray(trig, np.int32)
        self.hists = O.hist_table()
        O.fill_histograms(tv, self.dims, self.hists, self.trig, st)
        # domain counters from a counted run of the whole chain
        h2, t2, st2 = hits0.copy(), L.HostTracks(n), O.OracleState(n)
        O.run_all(plane, h2, t2, st2, counted=True)
        self.counts = st2.counts.reshape(n, O.NCOUNTS)


def in_domain(hits0, snap):
    n = hits0.n
    raw = hits0.nhits_cham.reshape(n, L.NCHAM).max(axis=1)
    # the reference's dimuon kernel stores a 17th dimuon past its event's 16
    # records (K:3059), beyond its buffer for the last event: keep events the
    # oracle gives fewer than 16
    return ((raw <= MAX_CHAM_RAW) & (snap.counts[:, 6] <= MAX_WINDOW) & (snap.counts[:, 7] <= MAX_WINDOW) &
            (snap.dims.ndimuons < L.DIMUON_MAX))


def recomputed_flags(h):
    """HasTooManyHits from the reduced counts: station sums over the planes
    of D0, D2, D3p, D3m against 210/120/90/90 (K:128-139 over the 8 real rows)."""
    c = h.nhits_cham.reshape(h.n, L.NCHAM).astype(np.int64)
    d0 = c[:, 0:6].sum(1)
    d2 = c[:, 12:18].sum(1)
    d3p = c[:, 18:24].sum(1)
    d3m = c[:, 24:30].sum(1)
    return ((d0 > 210) | (d2 > 120) | (d3p > 90) | (d3m > 90)).astype(np.uint8)


def run_reference(rk, plane, snap, n):
    """Reference outputs of every stage, each fed the oracle's previous state."""
    out = {}
    rk.set_plane(plane)
    # ER
    rk.put_hits(snap.hits0)
    rk.put_flags(np.zeros(n, np.uint8))
    t0 = time.time()
    rk.event_reduce(n)
    out["t_er"] = time.time() - t0
    out["hits_er"] = rk.get_hits(n)
    out["flags_er"] = rk.get_flags(n)
    # XZ candidates on the reference's helpers, from the oracle's reduced hits
    rk.put_hits(snap.hits_er)
    rk.put_flags(snap.toomany_er)
    out["xz"] = rk.xz_candidates(n)
    # YZ
    rk.put_hits(snap.hits_er)
    rk.put_tracks(snap.tracks_xz)
    rk.put_flags(snap.toomany_xz)
    t0 = time.time()
    rk.yz(n)
    out["t_yz"] = time.time() - t0
    out["tracks_yz"] = rk.get_tracks(n)
    # cleaning
    rk.put_tracks(snap.tracks_yz)
    rk.back_clean(n)
    out["tracks_clean"] = rk.get_tracks(n)
    # global
    rk.put_tracks(snap.tracks_clean)
    t0 = time.time()
    rk.global_tracking(n)
    out["t_global"] = time.time() - t0
    out["tracks_global"] = rk.get_tracks(n)
    # post-global selection
    rk.put_tracks(snap.tracks_global)
    rk.selection(n)
    out["tracks_sel"] = rk.get_tracks(n)
    # vertexing, dimuons (M:939-968)
    rk.put_tracks(snap.tracks_sel)
    rk.vertexing(n)
    out["tracks_vtx"] = rk.get_tracks(n)
    rk.put_tracks(snap.tracks_vtx)
    rk.put_dimuons(L.HostDimuons(n))
    rk.dimuons(n)
    out["dims"] = rk.get_dimuons(n)
    # histograms (M:983) on the oracle's tracks and dimuons
    rk.put_dimuons(snap.dims)
    out["hists"] = rk.histograms(np.nonzero(snap.toomany_xz == 0)[0], O.hist_table(), snap.trig)
    return out


def compare(snap, ref, rtol):
    rep = {}
    er = G.compare_hits(G.compact_hits(ref["hits_er"]), G.compact_hits(snap.hits_er))
    rep["er_hits"] = {"events": snap.hits0.n, "mismatch": er[:20], "n_mismatch": len(er)}
    flags_ref = ref["flags_er"]
    flags_re = recomputed_flags(ref["hits_er"])
    rep["er_flags"] = {"accepted_by_oracle": int((snap.toomany_er == 0).sum()),
                       "recomputed_vs_oracle_mismatch": int((flags_re != snap.toomany_er).sum()),
                       "reference_raw_vs_oracle_mismatch": int((flags_ref != snap.toomany_er).sum())}
    rep["xz"] = compare_xz(snap, ref["xz"], rtol)
    for stage, want in (("yz", snap.tracks_yz), ("clean", snap.tracks_clean), ("global", snap.tracks_global),
                        ("sel", snap.tracks_sel)):
        a = G.compact_tracks(ref["tracks_" + stage], snap.toomany_xz)
        b = G.compact_tracks(want, snap.toomany_xz)
        r = G.compare_tracks(a, b, rtol)
        for k in ("count_mismatch", "discrete_mismatch", "value_mismatch"):
            r["n_" + k] = len(r[k])
            r[k] = r[k][:20]
        rep[stage] = r
    r = G.compare_tracks(G.compact_tracks(ref["tracks_vtx"], snap.toomany_xz),
                         G.compact_tracks(snap.tracks_vtx, snap.toomany_xz), rtol)
    for k in ("count_mismatch", "discrete_mismatch", "value_mismatch"):
        r["n_" + k] = len(r[k])
        r[k] = r[k][:20]
    rep["vtx"] = r
    r = G.compare_dimuons(G.compact_dimuons(ref["dims"], snap.toomany_xz),
                          G.compact_dimuons(snap.dims, snap.toomany_xz), rtol, phi_ulps=4)
    for k in ("count_mismatch", "value_mismatch"):
        r["n_" + k] = len(r[k])
        r[k] = r[k][:20]
    rep["dim"] = r
    rep["hist"] = {"differing_tables": G.compare_hists(ref["hists"], snap.hists, phi_slack=2),
                   "counts": float(snap.hists.values_array().sum())}
    rep["seconds"] = {k: ref[k] for k in ("t_er", "t_yz", "t_global")}
    return rep


def run_library(rc, snap, n):
    """The library's stages on a context `rc`, each fed the oracle's state
    before that stage (as the reference kernels are)."""
    import torch
    from orgpu import pipeline
    b = pipeline.DeviceBatch(n)
    out = {}

    def flags(f):
        b.toomany.copy_(torch.from_numpy(np.ascontiguousarray(f, np.uint8)))

    b.upload_hits(snap.hits0)
    flags(np.zeros(n, np.uint8))
    rc.event_reduce(b)
    rc.sync()
    out["hits_er"] = b.download_hits()
    for stage, hits_in, tracks_in, flags_in, call in (
            ("xz", snap.hits_er, None, snap.toomany_er, rc.xz_tracking),
            ("yz", snap.hits_er, snap.tracks_xz, snap.toomany_xz, rc.yz_tracking),
            ("clean", snap.hits_er, snap.tracks_yz, snap.toomany_xz, rc.back_track_cleaning),
            ("global", snap.hits_er, snap.tracks_clean, snap.toomany_xz, rc.global_tracking),
            ("sel", snap.hits_er, snap.tracks_global, snap.toomany_xz, rc.selection)):
        b.upload_hits(hits_in)
        if tracks_in is not None:
            b.upload_tracks(tracks_in)
        flags(flags_in)
        b.ntracklets.zero_()
        call(b)
        rc.sync()
        out["tracks_" + stage] = b.download_tracks()
        out["flags_" + stage] = b.toomany.cpu().numpy()
    return out


def compare_library(lib_out, ref, snap, rtol):
    """A library build's stage outputs against a reference image's, each
    stage on the same oracle input."""
    rep = {}
    er = G.compare_hits(G.compact_hits(ref["hits_er"]), G.compact_hits(lib_out["hits_er"]))
    rep["er_hits"] = {"n_mismatch": len(er)}
    acc = np.nonzero(snap.toomany_xz == 0)[0]
    pin = G.xz_from_pin(ref["xz"][0], ref["xz"][1], acc)
    lib_xz = G.xz_from_tracks(_take_tracks(lib_out["tracks_xz"], acc), None)
    r = G.compare_xz(lib_xz, pin, rtol)
    rep["xz"] = {k: r[k] for k in ("candidates", "n_set_mismatch", "n_value_mismatch", "max_rel_fit")}
    for stage in ("yz", "clean", "global", "sel"):
        r = G.compare_tracks(G.compact_tracks(lib_out["tracks_" + stage], snap.toomany_xz),
                             G.compact_tracks(ref["tracks_" + stage], snap.toomany_xz), rtol)
        rep[stage] = {"tracks": r.get("tracks"), "n_count_mismatch": len(r["count_mismatch"]),
                      "n_discrete_mismatch": len(r["discrete_mismatch"]),
                      "n_value_mismatch": len(r["value_mismatch"]), "max_rel_fit": r["max_rel_fit"]}
    return rep


def compare_xz(snap, pin, rtol):
    """The XZ candidates of the reference's helpers against the oracle's
    tracklets, on the events the oracle's XZ stage accepts; and, for the
    events it rejects, whether the reference threads see the same cause: a
    bin with more than 20 pairs (K:359-375) or more accepted candidates than
    the 512 tracklet slots (16 per thread, per station-3 half) hold
    (K:719-723, K:824-839)."""
    out, nout, st = pin
    acc = np.nonzero(snap.toomany_xz == 0)[0]
    a = G.xz_from_pin(out, nout, acc)
    b = G.xz_from_tracks(_take_tracks(snap.tracks_xz, acc), None)
    r = G.compare_xz(a, b, rtol)
    r["threads_out_full"] = int(((st & 4) != 0).sum())
    r["threads_out_of_domain"] = int(((st & 2) != 0).sum())
    rej = np.nonzero((snap.toomany_xz != 0) & (snap.toomany_er == 0))[0]
    over = ((st[rej] & 1) != 0).any(axis=1)
    par = np.stack([nout[rej][:, 0::2].sum(1), nout[rej][:, 1::2].sum(1)], 1) if len(rej) else np.zeros((0, 2))
    full = (par.sum(1) >= L.TRKMAX) | (par > L.NSLOTS // 2 * L.SLOTCAP).any(1)
    r["oracle_rejected"] = int(len(rej))
    r["rejected_same_cause"] = int((over | full).sum())
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(REPO, "out", "golden"))
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    from oracle.ref import refrun

    plane, wp = O.parse_geometry(GEOMETRY_E906)
    geo = S.Geometry(plane, wp)
    report = {"configs": {}}
    fixture = {}
    images = {v: refrun.RefKernels(v) for v in ("fmad0", "fmad1")}
    import build_lib
    from orgpu import _lib, pipeline
    rc_fmad1 = pipeline.Reconstruction(plane, 0, lib=_lib.load(build_lib.build(fmad=True)))
    for name, cfg, n_all, n_fix in CONFIGS:
        rec, off, _ = S.generate(geo, cfg)
        rec, off = S.cap_records(rec, off)
        hits_all = S.pack(rec, off, geo.wire_pos_f32())
        snap_all = Snap(plane, hits_all)
        keep = np.nonzero(in_domain(hits_all, snap_all))[0]
        rec_k, off_k = G.select_events(rec, off, keep)
        hits0 = S.pack(rec_k, off_k, geo.wire_pos_f32())
        snap = Snap(plane, hits0)
        n = hits0.n
        crep = {"generated": int(n_all), "in_domain": int(n),
                "max_yz_window": int(snap_all.counts[:, 6].max()),
                "max_global_window": int(snap_all.counts[:, 7].max()),
                "max_raw_chamber_hits": int(hits_all.nhits_cham.max()),
                "oracle_yz_tracks": int(sum(1 for e in range(n) for s_, k_, r in snap.tracks_yz.records(e)
                                           if r[L.TRK_STID] == 5 and not snap.toomany_xz[e])),
                "oracle_global_tracks": int(sum(1 for e in range(n) for s_, k_, r in snap.tracks_global.records(e)
                                               if r[L.TRK_STID] == 6 and not snap.toomany_xz[e]))}
        # fixture events: the first n_fix in-domain events the XZ stage accepted
        acc = np.nonzero(snap.toomany_xz == 0)[0]
        fix = np.concatenate([acc[:n_fix], np.nonzero(snap.toomany_xz)[0][:2]])
        fix = np.sort(fix)
        rec_f, off_f = G.select_events(rec_k, off_k, fix)
        fixture[f"{name}/records"] = rec_f.view(np.uint8).reshape(-1, L.HIT_RECORD_DTYPE.itemsize)
        fixture[f"{name}/offsets"] = off_f
        fixture[f"{name}/trigger_bits"] = snap.trig[fix]
        for v, rk in images.items():
            ref = run_reference(rk, plane, snap, n)
            crep[v] = compare(snap, ref, 0.0 if v == "fmad0" else 1e-5)
            if v == "fmad1":
                crep["lib_fmad1_vs_ref_fmad1"] = compare_library(run_library(rc_fmad1, snap, n), ref, snap, 1e-5)
            sub = _subset(ref, fix)
            for key, arr in sub.items():
                fixture[f"{name}/{v}/{key}"] = arr
            # histograms of the fixture events alone, the way the CPU test refills them
            rk.put_tracks(snap.tracks_vtx)
            rk.put_dimuons(snap.dims)
            rk.put_flags(snap.toomany_xz)
            hf = rk.histograms([e for e in fix if not snap.toomany_xz[e]], O.hist_table(), snap.trig)
            fixture[f"{name}/{v}/hist_values"] = hf.values_array()
        report["configs"][name] = crep
        print(name, json.dumps({k: crep[k] for k in ("generated", "in_domain")}), flush=True)
    for rk in images.values():
        rk.close()
    rc_fmad1.close()
    with open(os.path.join(args.out, "golden_report.json"), "w") as f:
        json.dump(report, f, indent=1)
    np.savez_compressed(os.path.join(args.out, "ref_e906.npz"), **fixture)
    print(json.dumps(_summary(report)))


def _subset(ref, idx):
    """Compact reference outputs of the events idx."""
    out = {}
    h = _take_hits(ref["hits_er"], idx)
    out["er_counts"], out["er_hits"] = G.compact_hits(h)
    out["er_flags"] = ref["flags_er"][idx]
    out["xz_count"], out["xz_records"] = G.xz_from_pin(ref["xz"][0], ref["xz"][1], idx)
    for stage in ("yz", "clean", "global", "sel", "vtx"):
        t = _take_tracks(ref["tracks_" + stage], idx)
        nt, w, r = G.compact_tracks(t)
        out[f"{stage}_ntracks"], out[f"{stage}_where"], out[f"{stage}_records"] = nt, w, r
    d = L.HostDimuons(len(idx))
    d.ndimuons[:] = ref["dims"].ndimuons[idx]
    d.dimuons[:] = ref["dims"].dimuons.reshape(ref["dims"].n, L.EVT_DIM_FLOATS)[idx].reshape(-1)
    out["dim_n"], out["dim_records"] = G.compact_dimuons(d)
    return out


def _take_hits(h, idx):
    o = L.HostHits(len(idx))
    for a_new, a_old, per in zip(o.arrays(), h.arrays(), (L.NCHAM, L.EVT_CHAM_FLOATS, L.NHODO, L.EVT_HODO_FLOATS,
                                                          L.NPROP, L.EVT_PROP_FLOATS)):
        a_new[:] = a_old.reshape(h.n, per)[idx].reshape(-1)
    return o


def _take_tracks(t, idx):
    o = L.HostTracks(len(idx))
    o.ntracks[:] = t.ntracks.reshape(t.n, L.NSLOTS)[idx].reshape(-1)
    o.tracks[:] = t.tracks.reshape(t.n, L.EVT_TRK_FLOATS)[idx].reshape(-1)
    return o


def _summary(report):
    s = {}
    for name, c in report["configs"].items():
        for v in ("fmad0", "fmad1"):
            r = c[v]
            s[f"{name}/{v}"] = {"er": r["er_hits"]["n_mismatch"],
                                "flags_recomputed": r["er_flags"]["recomputed_vs_oracle_mismatch"],
                                **{st: [r[st]["n_count_mismatch"], r[st]["n_discrete_mismatch"],
                                        r[st]["n_value_mismatch"], r[st]["max_rel_fit"]]
                                   for st in ("yz", "clean", "global", "sel", "vtx")},
                                "xz": [r["xz"]["n_set_mismatch"], r["xz"]["n_value_mismatch"], r["xz"]["max_rel_fit"],
                                       r["xz"]["oracle_rejected"] - r["xz"]["rejected_same_cause"]],
                                "dim": [r["dim"]["n_count_mismatch"], r["dim"]["n_value_mismatch"]],
                                "hist": r["hist"]["differing_tables"]}
    return s


if __name__ == "__main__":
    main()
