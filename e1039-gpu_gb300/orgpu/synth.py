"""Seeded synthetic E906/E1039 events for the online-reconstruction path.

The reference reads ROOT files of raw events (OnlineReconstruction/
online_reconstruction.cu:246-642), which are not available here.  This module
generates events with the same record format (int16 detectorID / elementID,
float32 tdcTime / driftDistance, in-time flag; LoadInput.h:10-20) and packs
them into the reference hit layout (online_reconstruction.cu:589-636).

Track model.  A muon of charge q and momentum p leaves the target
(z = -300 cm) on a straight line, gets a transverse kick in FMag (z = 251.4)
and one in KMag (z = 1064.26), and is straight elsewhere; the KMag kick is the
one the reconstruction inverts (tx_st1 = tx + PT_KICK_KMAG*q/p,
reconstruction_helper.cuh:622-626), the FMag kick uses the same convention
with PT_KICK_FMAG = 2.909 * FMAGSTR.  y is straight from the target.  Wires
are the geometry's wire lines (p1 + (elem-1)*dp1, direction dp); the hit
element is the nearest wire, drift = |distance| + N(0, 0.04 cm) clipped to
half a cell, per-plane efficiency 0.95.  Hodoscope paddles and prop tubes are
hit the same way.  Noise hits are uniform over the (plane, element) pairs of
the 48 planes the path reads.  Hits are sorted by (det, elem, tdc) inside an
event, which the event reducer's declustering assumes.
"""
import dataclasses

import numpy as np

from . import layout as L

Z_TARGET, Z_FMAG_BEND, Z_KMAG_BEND = -300.0, 251.4, 1064.26
PT_KICK_KMAG = -0.3819216
PT_KICK_FMAG = 2.909 * -1.054

# tdc windows by plane type (chambers, hodoscopes, prop tubes)
_TDC_WIN = ((1000.0, 1200.0), (900.0, 1000.0), (1200.0, 1400.0))


@dataclasses.dataclass
class EventConfig:
    n_events: int
    seed: int
    track_weights: tuple = (0.0, 0.0, 1.0)   # P(n_tracks = 0, 1, 2, ...)
    noise: str = "poisson"                  # "poisson" | "lognormal"
    noise_mean: float = 150.0               # poisson mean, or lognormal median
    noise_sigma: float = 0.8                # lognormal sigma (natural-log units)
    noise_clip: int = 3000
    afterpulse_frac: float = 0.0
    p_range: tuple = (10.0, 100.0)
    efficiency: float = 0.95
    drift_sigma: float = 0.04
    out_of_time_frac: float = 0.02          # noise hits with flag 1

    @property
    def label(self):
        return f"n{self.n_events}_s{self.seed}"


def config_small(n_events=1000, seed=906001):
    """One opposite-sign dimuon + Poisson(150) noise per event."""
    return EventConfig(n_events, seed, (0.0, 0.0, 1.0), "poisson", 150.0)


def config_uneven(n_events=100000, seed=906002):
    """0-3 muons (0.2/0.3/0.4/0.1), log-normal noise (median 300, sigma 0.8,
    clipped at 3000)."""
    return EventConfig(n_events, seed, (0.2, 0.3, 0.4, 0.1), "lognormal", 300.0, 0.8, 3000)


def config_high_occupancy(n_events=500000, seed=906004):
    """Two muons, Poisson(1000) noise, 10% after-pulse duplicates."""
    return EventConfig(n_events, seed, (0.0, 0.0, 1.0), "poisson", 1000.0, afterpulse_frac=0.10)


class Geometry:
    """Plane arrays the generator needs, from an OrPlane and wire positions."""

    def __init__(self, plane, wire_pos):
        self.plane = plane
        self.wire_pos = np.asarray(wire_pos, np.float64).reshape(L.NDET, L.WIREPOS_STRIDE)
        g = {n: plane.arr(n) for n, _ in L._PLANE_FIELDS}
        self.g = g
        self.nelem = g["nelem"].astype(np.int64)
        self.planes = np.array(L.PATH_PLANES, np.int64)

    def wire_pos_f32(self):
        return self.wire_pos.astype(np.float32)


def _xy_at(par, z):
    xv, yv, tx0, tx1, tx23, ty, xf, xk = par
    z = np.asarray(z, np.float64)
    x = np.where(z < Z_FMAG_BEND, xv + tx0 * (z - Z_TARGET),
                 np.where(z < Z_KMAG_BEND, xf + tx1 * (z - Z_FMAG_BEND), xk + tx23 * (z - Z_KMAG_BEND)))
    y = yv + ty * (z - Z_TARGET)
    return x, y


# (z, |x| limit, |y| limit) the track must stay inside: D0, D2, D3, last prop
# tube plane -- a little inside the planes' x1..x2 / y1..y2 extents
_APERTURES = ((620.0, 48.0, 56.0), (1345.0, 112.0, 128.0), (1915.0, 155.0, 158.0), (2395.0, 178.0, 178.0))


def _sample_tracks(rng, n, q, p_range):
    """n accepted muon tracks of charge q (vectorised rejection sampling).
    Returns a (8, n) array of _track_line parameters and invp."""
    out = np.zeros((8, n))
    invp = np.zeros(n)
    todo = np.arange(n)
    for _ in range(200):
        if len(todo) == 0:
            break
        m = len(todo)
        p = rng.uniform(p_range[0], p_range[1], m)
        k = q[todo] / p
        xv, yv = rng.normal(0.0, 0.3, m), rng.normal(0.0, 0.3, m)
        tx23 = rng.uniform(-0.12, 0.12, m)
        ty = rng.uniform(-0.05, 0.05, m)
        tx1 = tx23 + PT_KICK_KMAG * k
        tx0 = tx1 + PT_KICK_FMAG * k
        xf = xv + tx0 * (Z_FMAG_BEND - Z_TARGET)
        xk = xf + tx1 * (Z_KMAG_BEND - Z_FMAG_BEND)
        par = np.stack([xv, yv, tx0, tx1, tx23, ty, xf, xk])
        x0 = xk - tx23 * Z_KMAG_BEND
        y0 = yv - ty * Z_TARGET
        ok = (np.abs(x0) < 140.0) & (np.abs(tx23) < 0.14) & (np.abs(y0) < 45.0) & (np.abs(ty) < 0.09)
        for z, xl, yl in _APERTURES:
            x, y = _xy_at(par, z)
            ok &= (np.abs(x) <= xl) & (np.abs(y) <= yl)
        out[:, todo[ok]] = par[:, ok]
        invp[todo[ok]] = 1.0 / p[ok]
        todo = todo[~ok]
    keep = np.ones(n, bool)
    keep[todo] = False
    return out, invp, keep


def _plane_hits(geo, par, rng, eff, dsig, d):
    """Hits of all tracks on plane d: (track index, element, drift)."""
    g = geo.g
    z = g["z"][d]
    x, y = _xy_at(par, z)
    nt = x.shape[0]
    ok = rng.random(nt) <= eff
    ok &= (g["x1"][d] <= x) & (x <= g["x2"][d]) & (g["y1"][d] <= y) & (y <= g["y2"][d])
    n = int(geo.nelem[d])
    half = 0.5 * g["cellwidth"][d]
    noise = rng.normal(0.0, dsig, nt)
    if d <= L.NCHAM:
        dpx, dpy = g["deltapx"][d], g["deltapy"][d]
        ln = np.hypot(dpx, dpy)
        d1 = ((x - g["p1x_w1"][d]) * dpy - (y - g["p1y_w1"][d]) * dpx) / ln
        pitch = (g["dp1x"][d] * dpy - g["dp1y"][d] * dpx) / ln
        j = np.rint(d1 / pitch).astype(np.int64) + 1
        ok &= (j >= 1) & (j <= n)
        dist = np.abs(d1 - (j - 1) * pitch)
        drift = np.clip(dist + noise, 0.0, half)
    else:
        u = x * g["costheta"][d] + y * g["sintheta"][d]
        wp = geo.wire_pos[d, 1:n + 1]
        order = np.argsort(wp)
        ws = wp[order]
        pos = np.clip(np.searchsorted(ws, u), 1, n - 1)
        left, right = ws[pos - 1], ws[pos]
        pick = np.where(np.abs(u - left) <= np.abs(u - right), pos - 1, pos)
        j = order[pick] + 1
        dist = np.abs(wp[j - 1] - u)
        if d <= L.NCHAM + L.NHODO:
            if abs(g["costheta"][d]) > 0.5:
                lo, hi, other = g["y1"][d], g["y2"][d], y
            else:
                lo, hi, other = g["x1"][d], g["x2"][d], x
            ok = (rng.random(nt) <= eff) & (lo <= other) & (other <= hi) & (dist <= half)
            drift = np.zeros(nt)
        else:
            ok &= dist <= half
            drift = np.clip(dist + noise, 0.0, half)
    idx = np.nonzero(ok)[0]
    return idx, j[idx], drift[idx]


def generate(geo, cfg):
    """Generate cfg.n_events events (vectorised over tracks and noise hits).

    Returns (records, offsets, truth): records is a HIT_RECORD_DTYPE array
    sorted by (event, det, elem, tdc); offsets[e]..offsets[e+1] index event
    e; truth holds per-muon arrays (event, charge, invp, x0, tx, y0, ty).
    """
    rng = np.random.default_rng(cfg.seed)
    g = geo.g
    n_ev = cfg.n_events
    weights = np.asarray(cfg.track_weights, np.float64)
    weights = weights / weights.sum()
    ntrk = rng.choice(len(weights), size=n_ev, p=weights)
    tev = np.repeat(np.arange(n_ev), ntrk)
    # alternate charges inside an event: +, -, +, ...
    first = np.r_[0, np.cumsum(ntrk)[:-1]]
    rank = np.arange(len(tev)) - np.repeat(first, ntrk)
    q = np.where(rank % 2 == 0, 1.0, -1.0)
    par, invp, keep = _sample_tracks(rng, len(tev), q, cfg.p_range)
    par, invp, tev, q = par[:, keep], invp[keep], tev[keep], q[keep]
    ptype = np.array([L.plane_type(int(d)) for d in range(L.NDET)])
    win = np.array(_TDC_WIN)

    dets, elems, drifts, evs, flags, tdcs = [], [], [], [], [], []
    for d in geo.planes:
        d = int(d)
        idx, j, dr = _plane_hits(geo, par, rng, cfg.efficiency, cfg.drift_sigma, d)
        half = 0.5 * g["cellwidth"][d]
        tlo, thi = win[ptype[d]]
        frac = dr / half if half > 0 else np.zeros_like(dr)
        tdc = thi - frac * (thi - tlo) + rng.normal(0.0, 1.0, len(dr))
        dets.append(np.full(len(idx), d)); elems.append(j); drifts.append(dr)
        evs.append(tev[idx]); flags.append(np.full(len(idx), 2)); tdcs.append(tdc)
    # noise, uniform over the (plane, element) pairs of the path's planes
    if cfg.noise == "poisson":
        nn = rng.poisson(cfg.noise_mean, n_ev)
    else:
        nn = np.rint(cfg.noise_mean * np.exp(rng.normal(0.0, cfg.noise_sigma, n_ev))).astype(np.int64)
        nn = np.minimum(nn, cfg.noise_clip)
    tot = int(nn.sum())
    planes = geo.planes
    cum_el = np.cumsum(geo.nelem[planes])
    flat = rng.integers(0, int(cum_el[-1]), tot)
    pidx = np.searchsorted(cum_el, flat, side="right")
    det = planes[pidx]
    dets.append(det)
    elems.append(flat - np.concatenate(([0], cum_el))[pidx] + 1)
    half = 0.5 * g["cellwidth"][det]
    drifts.append(np.where(ptype[det] == 1, 0.0, rng.uniform(0.0, 1.0, tot) * half))
    evs.append(np.repeat(np.arange(n_ev), nn))
    flags.append(np.where(rng.random(tot) < cfg.out_of_time_frac, 1, 2))
    tdcs.append(rng.uniform(win[ptype[det], 0], win[ptype[det], 1]))

    det = np.concatenate(dets).astype(np.int16)
    elem = np.concatenate(elems).astype(np.int16)
    drift = np.concatenate(drifts).astype(np.float32)
    ev = np.concatenate(evs).astype(np.int64)
    flag = np.concatenate(flags).astype(np.int32)
    tdc = np.concatenate(tdcs).astype(np.float32)
    if cfg.afterpulse_frac > 0 and len(det):
        pick = np.nonzero(rng.random(len(det)) < cfg.afterpulse_frac)[0]
        det = np.r_[det, det[pick]]
        elem = np.r_[elem, elem[pick]]
        drift = np.r_[drift, drift[pick]]
        ev = np.r_[ev, ev[pick]]
        flag = np.r_[flag, flag[pick]]
        tdc = np.r_[tdc, (tdc[pick] + rng.uniform(50.0, 200.0, len(pick))).astype(np.float32)]
    # (event, det, elem, tdc) order with one integer radix sort: all tdc lie in
    # [512, 4096), where the float bit pattern minus that of 512.0 is
    # monotonic and fits 25 bits
    assert len(tdc) == 0 or (tdc.min() >= 512.0 and tdc.max() < 4096.0)
    tkey = tdc.view(np.int32).astype(np.int64) - int(np.float32(512.0).view(np.int32))
    key = (ev << 39) | (det.astype(np.int64) << 33) | (elem.astype(np.int64) << 25) | tkey
    order = np.argsort(key, kind="stable")
    rec = np.zeros(len(order), L.HIT_RECORD_DTYPE)
    rec["det"], rec["elem"], rec["tdc"] = det[order], elem[order], tdc[order]
    rec["drift"], rec["flag"] = drift[order], flag[order]
    offsets = np.concatenate(([0], np.cumsum(np.bincount(ev, minlength=n_ev)))).astype(np.int64)
    xv, yv, tx0, tx1, tx23, ty, xf, xk = par
    truth = {"event": tev, "charge": q.astype(np.int64), "invp": invp, "x0": xk - tx23 * Z_KMAG_BEND,
             "tx": tx23, "y0": yv - ty * Z_TARGET, "ty": ty}
    return rec, offsets, truth


def generate_capped(job):
    """generate() + cap_records() for a process pool: job = (OrPlane bytes,
    wire positions, EventConfig); returns (records, offsets)."""
    plane_bytes, wire_pos, cfg = job
    plane = L.OrPlane.from_buffer_copy(plane_bytes)
    rec, off, _ = generate(Geometry(plane, wire_pos), cfg)
    return cap_records(rec, off)


def trigger_bits(n_events, seed=906010):
    """Per-event trigger words (int32): the reference reads them from the raw
    event (gEvent::TriggerBits, online_reconstruction.cu:346); here ten
    seeded independent bits, each set with probability 1/2."""
    return np.random.default_rng(seed).integers(0, 1 << 10, n_events).astype(np.int32)


def cap_records(records, offsets):
    """Drop hits beyond each plane's slot capacity (the reference host writes
    past the slot otherwise, online_reconstruction.cu:406-417)."""
    ev = np.repeat(np.arange(len(offsets) - 1), np.diff(offsets))
    key = ev * L.NDET + records["det"].astype(np.int64)
    first = np.r_[True, key[1:] != key[:-1]]
    start = np.maximum.accumulate(np.where(first, np.arange(len(key)), 0))
    rank = np.arange(len(key)) - start
    cap = np.select([records["det"] <= L.NCHAM, records["det"] <= L.NCHAM + L.NHODO],
                    [L.MAXHITS_CHAM, L.MAXHITS_HODO], L.MAXHITS_PROP)
    keep = rank < cap
    new_counts = np.bincount(ev[keep], minlength=len(offsets) - 1)
    return records[keep], np.concatenate(([0], np.cumsum(new_counts))).astype(np.int64)


def pack(records, offsets, wire_pos_f32, n_events=None):
    """Pack records into a layout.HostHits (numpy), like the device packer.

    pos = float32(wire_pos[det][elem]); flag is stored as a float."""
    n = len(offsets) - 1 if n_events is None else n_events
    h = L.HostHits(n)
    if len(records) == 0:
        return h
    ev = np.repeat(np.arange(len(offsets) - 1), np.diff(offsets)).astype(np.int64)
    det = records["det"].astype(np.int64)
    key = ev * L.NDET + det
    first = np.r_[True, key[1:] != key[:-1]]
    start = np.maximum.accumulate(np.where(first, np.arange(len(key)), 0))
    rank = np.arange(len(key)) - start
    cnt = np.bincount(key, minlength=n * L.NDET).reshape(n, L.NDET)
    wp = np.asarray(wire_pos_f32, np.float32).reshape(L.NDET, L.WIREPOS_STRIDE)
    fields = (records["elem"].astype(np.float32), wp[det, records["elem"].astype(np.int64)],
              records["tdc"].astype(np.float32), records["flag"].astype(np.float32),
              records["drift"].astype(np.float32))
    for t, (lo, hi, stride, cap, per, counts, data) in enumerate((
            (1, L.NCHAM, L.EVT_CHAM_FLOATS, L.MAXHITS_CHAM, L.NCHAM, h.nhits_cham, h.hits_cham),
            (L.NCHAM + 1, L.NCHAM + L.NHODO, L.EVT_HODO_FLOATS, L.MAXHITS_HODO, L.NHODO, h.nhits_hodo, h.hits_hodo),
            (L.NCHAM + L.NHODO + 1, L.NDET - 1, L.EVT_PROP_FLOATS, L.MAXHITS_PROP, L.NPROP, h.nhits_prop,
             h.hits_prop))):
        counts[:] = cnt[:, lo:hi + 1].reshape(-1).astype(np.uint32)
        sel = (det >= lo) & (det <= hi)
        if not sel.any():
            continue
        e_s, d_s, r_s = ev[sel], det[sel] - lo, rank[sel]
        n_s = cnt[e_s, det[sel]]
        base = e_s * stride + L.NHITSPARAM * cap * d_s + r_s
        for f in range(L.NHITSPARAM):
            data[base + f * n_s] = fields[f][sel]
    return h
