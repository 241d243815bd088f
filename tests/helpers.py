"""Shared test helpers: seeded events, oracle stage snapshots, bitwise
comparison of the reference-layout buffers over their valid regions."""
import numpy as np

from oracle import pyoracle as O
from orgpu import layout as L
from orgpu import synth as S


def make_events(plane, wp, cfg):
    geo = S.Geometry(plane, wp)
    rec, off, truth = S.generate(geo, cfg)
    rec, off = S.cap_records(rec, off)
    hits = S.pack(rec, off, geo.wire_pos_f32())
    return geo, rec, off, hits, truth


def mixed_events(plane, wp, n_small=160, n_uneven=160, seed=7):
    """Config-1 style events followed by uneven-occupancy ones, one batch."""
    geo = S.Geometry(plane, wp)
    r1, o1, _ = S.generate(geo, S.config_small(n_small, seed))
    r2, o2, _ = S.generate(geo, S.config_uneven(n_uneven, seed + 1))
    rec = np.concatenate([r1, r2])
    off = np.concatenate([o1, o2[1:] + o1[-1]])
    rec, off = S.cap_records(rec, off)
    return geo, rec, off, S.pack(rec, off, geo.wire_pos_f32())


class Snapshots:
    """Oracle state after every stage, each a separate copy."""

    def __init__(self, plane, hits0, n_threads=0):
        n = hits0.n
        self.hits0 = hits0
        self.state = O.OracleState(n)
        self.hits_er = hits0.copy()
        O.event_reduce(self.hits_er, self.state, n_threads)
        self.toomany_er = self.state.toomany.copy()
        t = L.HostTracks(n)
        O.xz(plane, self.hits_er, t, self.state, n_threads)
        self.toomany_xz = self.state.toomany.copy()
        self.ntracklets = self.state.ntracklets.copy()
        self.tracks_xz = t.copy()
        O.yz(plane, self.hits_er, t, self.state, n_threads)
        self.tracks_yz = t.copy()
        O.back_clean(t, self.state, n_threads)
        self.tracks_clean = t.copy()
        O.global_tracking(plane, self.hits_er, t, self.state, n_threads)
        self.tracks_global = t
        # post-global selection on a copy
        ts = t.copy()
        O.prop_matching(plane, self.hits_er, ts, self.state, n_threads)
        O.global_clean(ts, self.state, n_threads)
        self.tracks_sel = ts


def hit_mismatches(a, b, max_report=10):
    """Events/planes whose counts or valid hit data differ bitwise."""
    out = []
    for name, per, stride, cap in (("cham", L.NCHAM, L.EVT_CHAM_FLOATS, L.MAXHITS_CHAM),
                                   ("hodo", L.NHODO, L.EVT_HODO_FLOATS, L.MAXHITS_HODO),
                                   ("prop", L.NPROP, L.EVT_PROP_FLOATS, L.MAXHITS_PROP)):
        ca, cb = getattr(a, "nhits_" + name), getattr(b, "nhits_" + name)
        da, db = getattr(a, "hits_" + name), getattr(b, "hits_" + name)
        diff = np.nonzero(ca != cb)[0]
        for k in diff[:max_report]:
            out.append((name, int(k // per), int(k % per), "count", int(ca[k]), int(cb[k])))
        for e in range(a.n):
            for p in range(per):
                n = int(ca[e * per + p])
                if n != int(cb[e * per + p]):
                    continue
                base = e * stride + L.NHITSPARAM * cap * p
                x = da[base:base + L.NHITSPARAM * n].view(np.uint32)
                y = db[base:base + L.NHITSPARAM * n].view(np.uint32)
                if not np.array_equal(x, y):
                    out.append((name, e, p, "data"))
                    if len(out) >= max_report:
                        return out
    return out


def track_mismatches(a, b, toomany=None, max_report=10):
    """(event, slot, k, first differing field) of track records that differ
    bitwise; events flagged in `toomany` are skipped."""
    out = []
    na = a.ntracks.reshape(a.n, L.NSLOTS)
    nb = b.ntracks.reshape(b.n, L.NSLOTS)
    ta = a.tracks.reshape(a.n, L.NSLOTS, L.SLOTCAP, L.NTRKPARAM).view(np.uint32)
    tb = b.tracks.reshape(b.n, L.NSLOTS, L.SLOTCAP, L.NTRKPARAM).view(np.uint32)
    for e in range(a.n):
        if toomany is not None and toomany[e]:
            continue
        if not np.array_equal(na[e], nb[e]):
            out.append((e, -1, -1, "ntracks"))
        else:
            for s in range(L.NSLOTS):
                k = int(na[e, s])
                if k and not np.array_equal(ta[e, s, :k], tb[e, s, :k]):
                    bad = np.nonzero(ta[e, s, :k] != tb[e, s, :k])
                    out.append((e, s, int(bad[0][0]), int(bad[1][0])))
        if len(out) >= max_report:
            break
    return out


def count_tracks(t, stid):
    n = 0
    for e in range(t.n):
        for s, k, r in t.records(e):
            n += int(r[L.TRK_STID] == stid)
    return n


def output_rows_oracle(hits, tracks, dims, toomany, raw_hits=None, event_ids=None, min_stid=7.0):
    """The reference host's output loop (online_reconstruction.cu:1063-1222)
    restated on host buffers: the row tables or_output_rows writes."""
    ev, hr, tr, th, dr = [], [], [], [], []
    for e in range(hits.n):
        if toomany[e] or (raw_hits is not None and raw_hits[e] == 0):
            continue
        h0, t0, th0, d0 = len(hr), len(tr), len(th), len(dr)
        for det in range(1, L.NDET):
            n, data = hits.plane(e, det)
            for l in range(n):
                hr.append((det, data[0, l], data[1, l], data[2, l], data[4, l]))
        for s in range(L.NSLOTS):
            for k in range(min(int(tracks.ntracks[e * L.NSLOTS + s]), L.SLOTCAP)):
                base = e * L.EVT_TRK_FLOATS + (s * L.SLOTCAP + k) * L.NTRKPARAM
                T = tracks.tracks[base:base + L.NTRKPARAM]
                if T[L.TRK_STID] < min_stid:
                    continue
                tr.append([T[i] for i in L.OUT_TRACK_SRC])
                for l in range(max(0, min(int(T[L.TRK_NHITS]), 18))):
                    th.append([T[L.TRK_HIT_DETID + l], T[L.TRK_HIT_CHAN + l], T[L.TRK_HIT_POS + l],
                               T[L.TRK_HIT_DRIFT + l], T[L.TRK_HIT_SIGN + l], T[L.TRK_HIT_TDC + l],
                               T[L.TRK_HIT_RESID + l]])
        for D in dims.records(e):
            dr.append([np.float32(D[L.DIM_POS_P + f[1]] + D[L.DIM_NEG_P + f[1]]) if isinstance(f, tuple) else D[f]
                       for f in L.OUT_DIMUON_SRC])
        ev.append((e, e if event_ids is None else int(event_ids[e]), len(hr) - h0, len(tr) - t0, len(dr) - d0, h0, t0,
                   th0, d0))
    f32 = np.float32
    return {"events": np.array(ev, np.int64).reshape(-1, L.OUT_EV_FIELDS),
            "hits": np.array(hr, f32).reshape(-1, L.OUT_HIT_FIELDS),
            "tracks": np.array(tr, f32).reshape(-1, L.OUT_TRACK_FIELDS),
            "track_hits": np.array(th, f32).reshape(-1, L.OUT_TRACKHIT_FIELDS),
            "dimuons": np.array(dr, f32).reshape(-1, L.OUT_DIMUON_FIELDS)}


def device_mismatches(b, e0, hits, tracks, state):
    """Compare events e0 .. e0 + hits.n of DeviceBatch `b` (after or_run_batch)
    with the oracle's buffers of the same events (after run_all), on the
    device.  Returns a dict of mismatch counts: hit lists per (event, plane)
    over the occupied head of each slot, the HasTooManyHits flag, nTracklets,
    slot counts and track records (all 148 floats, bitwise) of events the
    oracle did not reject."""
    import torch
    dev = b.toomany.device
    n = hits.n
    e1 = e0 + n
    out = {}

    def up(a):
        return torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(dev)

    for name, per, cap in (("cham", L.NCHAM, L.MAXHITS_CHAM), ("hodo", L.NHODO, L.MAXHITS_HODO),
                           ("prop", L.NPROP, L.MAXHITS_PROP)):
        dc = getattr(b, "nhits_" + name)[e0 * per:e1 * per]
        oc = up(getattr(hits, "nhits_" + name))
        w = L.NHITSPARAM * cap
        dd = getattr(b, "hits_" + name)[e0 * per * w:e1 * per * w].view(torch.int32).view(-1, w)
        od = up(getattr(hits, "hits_" + name)).view(torch.int32).view(-1, w)
        head = torch.arange(w, device=dev)[None, :] < (L.NHITSPARAM * oc.long())[:, None]
        bad_data = ((dd != od) & head).any(dim=1)
        out["hit_count_" + name] = int((dc != oc).sum())
        out["hit_data_" + name] = int((bad_data & (dc == oc)).sum())
    flags = b.toomany[e0:e1].cpu().numpy()
    out["toomany"] = int((flags != state.toomany).sum())
    out["ntracklets"] = int((b.ntracklets[e0:e1].cpu().numpy() != state.ntracklets).sum())
    keep = torch.from_numpy(state.toomany == 0).to(dev)
    dn = b.ntracks[e0 * L.NSLOTS:e1 * L.NSLOTS].view(n, L.NSLOTS)
    on = torch.from_numpy(tracks.ntracks.view(np.int16)).to(dev).view(n, L.NSLOTS)
    out["slot_counts"] = int(((dn != on).any(dim=1) & keep).sum())
    rec = L.NSLOTS * L.SLOTCAP * L.NTRKPARAM
    dt = b.tracks[e0 * rec:e1 * rec].view(torch.int32).view(n, L.NSLOTS, L.SLOTCAP, L.NTRKPARAM)
    ot = up(tracks.tracks).view(torch.int32).view(n, L.NSLOTS, L.SLOTCAP, L.NTRKPARAM)
    valid = torch.arange(L.SLOTCAP, device=dev)[None, None, :] < on.long()[:, :, None]
    valid &= keep[:, None, None]
    out["track_records"] = int(((dt != ot).any(dim=3) & valid).sum())
    out["tracks_compared"] = int(valid.sum())
    out["global_tracks"] = int(((ot[..., L.TRK_STID] == int(np.float32(6).view(np.int32))) & valid).sum())
    return out


def oracle_chunk(plane, geo, rec, off, e0, e1, n_threads=0):
    """The oracle's run_all on events e0..e1 of a record batch."""
    r = rec[off[e0]:off[e1]]
    o = (off[e0:e1 + 1] - off[e0]).astype(off.dtype)
    h = S.pack(r, o, geo.wire_pos_f32())
    t = L.HostTracks(e1 - e0)
    st = O.OracleState(e1 - e0)
    O.run_all(plane, h, t, st, n_threads)
    return h, t, st
