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


def _track_line(rng, q, invp):
    """Piecewise-straight x(z) and straight y(z); returns callables' params."""
    xv, yv = rng.normal(0.0, 0.3), rng.normal(0.0, 0.3)
    tx23 = rng.uniform(-0.12, 0.12)
    ty = rng.uniform(-0.05, 0.05)
    k = invp * q
    tx1 = tx23 + PT_KICK_KMAG * k
    tx0 = tx1 + PT_KICK_FMAG * k
    xf = xv + tx0 * (Z_FMAG_BEND - Z_TARGET)
    xk = xf + tx1 * (Z_KMAG_BEND - Z_FMAG_BEND)
    return (xv, yv, tx0, tx1, tx23, ty, xf, xk)


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


def _accepted(par):
    xv, yv, tx0, tx1, tx23, ty, xf, xk = par
    x0 = xk - tx23 * Z_KMAG_BEND
    y0 = yv - ty * Z_TARGET
    if not (abs(x0) < 140.0 and abs(tx23) < 0.14 and abs(y0) < 45.0 and abs(ty) < 0.09):
        return False
    for z, xl, yl in _APERTURES:
        x, y = _xy_at(par, z)
        if abs(float(x)) > xl or abs(float(y)) > yl:
            return False
    return True


def _signal_hits(geo, par, rng, eff, dsig):
    """Hits of one track on the 48 planes: list of (det, elem, drift)."""
    g = geo.g
    out = []
    for d in geo.planes:
        if rng.random() > eff:
            continue
        z = g["z"][d]
        x, y = _xy_at(par, z)
        x, y = float(x), float(y)
        n = int(geo.nelem[d])
        dpx, dpy = g["deltapx"][d], g["deltapy"][d]
        ln = np.hypot(dpx, dpy)
        # active area of the plane (x1..x2, y1..y2 columns of the geometry)
        if not (g["x1"][d] <= x <= g["x2"][d] and g["y1"][d] <= y <= g["y2"][d]):
            continue
        half = 0.5 * g["cellwidth"][d]
        if d <= L.NCHAM:
            # drift chambers: nearest wire line; signed distance to wire 1 and
            # the signed pitch
            d1 = ((x - g["p1x_w1"][d]) * dpy - (y - g["p1y_w1"][d]) * dpx) / ln
            pitch = (g["dp1x"][d] * dpy - g["dp1y"][d] * dpx) / ln
            j = int(np.rint(d1 / pitch)) + 1
            if j < 1 or j > n:
                continue
            dist = abs(d1 - (j - 1) * pitch)
        elif d > L.NCHAM + L.NHODO:
            # prop tubes: nearest tube by its packed position, which is what
            # the reconstruction compares against
            u = x * g["costheta"][d] + y * g["sintheta"][d]
            wp = geo.wire_pos[d, 1:n + 1]
            j = int(np.argmin(np.abs(wp - u))) + 1
            dist = abs(wp[j - 1] - u)
            if dist > half:
                continue
        if d <= L.NCHAM or d > L.NCHAM + L.NHODO:
            drift = min(max(dist + rng.normal(0.0, dsig), 0.0), half)
            out.append((int(d), j, float(drift)))
        else:
            # hodoscope paddle: measured coordinate along the plane's axis, and
            # the paddle row's extent on the other axis
            u = x * g["costheta"][d] + y * g["sintheta"][d]
            if abs(g["costheta"][d]) > 0.5:
                lo, hi, other = g["y1"][d], g["y2"][d], y
            else:
                lo, hi, other = g["x1"][d], g["x2"][d], x
            if not (lo <= other <= hi):
                continue
            wp = geo.wire_pos[d, 1:n + 1]
            j = int(np.argmin(np.abs(wp - u))) + 1
            if abs(wp[j - 1] - u) > 0.5 * g["cellwidth"][d]:
                continue
            out.append((int(d), j, 0.0))
    return out


def generate(geo, cfg):
    """Generate cfg.n_events events.

    Returns (records, offsets, truth): records is a HIT_RECORD_DTYPE array
    sorted by (event, det, elem, tdc); offsets[e]..offsets[e+1] index event
    e; truth is a dict of per-track arrays (event, charge, invp, x0, tx, y0,
    ty) of the generated muons.
    """
    rng = np.random.default_rng(cfg.seed)
    g = geo.g
    planes = geo.planes
    nel = geo.nelem[planes]
    cum_el = np.cumsum(nel)
    tot_el = int(cum_el[-1])
    weights = np.asarray(cfg.track_weights, np.float64)
    weights = weights / weights.sum()

    ev_chunks, off = [], [0]
    truth = {k: [] for k in ("event", "charge", "invp", "x0", "tx", "y0", "ty")}
    ptype = np.array([L.plane_type(int(d)) for d in range(L.NDET)])
    for e in range(cfg.n_events):
        ntrk = int(rng.choice(len(weights), p=weights))
        hits = []
        for t in range(ntrk):
            q = 1 if t % 2 == 0 else -1
            for _ in range(200):
                p = rng.uniform(*cfg.p_range)
                par = _track_line(rng, q, 1.0 / p)
                if _accepted(par):
                    break
            else:
                continue
            for d, j, dr in _signal_hits(geo, par, rng, cfg.efficiency, cfg.drift_sigma):
                half = 0.5 * g["cellwidth"][d]
                tlo, thi = _TDC_WIN[ptype[d]]
                frac = dr / half if half > 0 else 0.0
                tdc = thi - frac * (thi - tlo) + rng.normal(0.0, 1.0)
                hits.append((d, j, tdc, dr, 2))
            xv, yv, tx0, tx1, tx23, ty, xf, xk = par
            truth["event"].append(e)
            truth["charge"].append(q)
            truth["invp"].append(1.0 / p)
            truth["x0"].append(xk - tx23 * Z_KMAG_BEND)
            truth["tx"].append(tx23)
            truth["y0"].append(yv - ty * Z_TARGET)
            truth["ty"].append(ty)
        if cfg.noise == "poisson":
            nn = int(rng.poisson(cfg.noise_mean))
        else:
            nn = int(np.rint(cfg.noise_mean * np.exp(rng.normal(0.0, cfg.noise_sigma))))
            nn = min(nn, cfg.noise_clip)
        if nn > 0:
            flat = rng.integers(0, tot_el, nn)
            pidx = np.searchsorted(cum_el, flat, side="right")
            det = planes[pidx]
            elem = flat - np.concatenate(([0], cum_el))[pidx] + 1
            half = 0.5 * g["cellwidth"][det]
            drift = np.where(ptype[det] == 1, 0.0, rng.uniform(0.0, 1.0, nn) * half)
            win = np.array(_TDC_WIN)[ptype[det]]
            tdc = rng.uniform(win[:, 0], win[:, 1])
            flag = np.where(rng.random(nn) < cfg.out_of_time_frac, 1, 2)
            hits.extend(zip(det.tolist(), elem.tolist(), tdc.tolist(), drift.tolist(), flag.tolist()))
        if cfg.afterpulse_frac > 0 and hits:
            nap = int(rng.binomial(len(hits), cfg.afterpulse_frac))
            pick = rng.choice(len(hits), nap, replace=False)
            for i in pick:
                d, j, tdc, dr, fl = hits[i]
                hits.append((d, j, tdc + rng.uniform(50.0, 200.0), dr, fl))
        a = np.array(hits, dtype=[("det", "<i2"), ("elem", "<i2"), ("tdc", "<f4"), ("drift", "<f4"),
                                  ("flag", "<i4")]) if hits else np.zeros(0, L.HIT_RECORD_DTYPE)
        a = a.astype(L.HIT_RECORD_DTYPE)
        a = a[np.lexsort((a["tdc"], a["elem"], a["det"]))]
        ev_chunks.append(a)
        off.append(off[-1] + len(a))
    records = np.concatenate(ev_chunks) if ev_chunks else np.zeros(0, L.HIT_RECORD_DTYPE)
    truth = {k: np.asarray(v) for k, v in truth.items()}
    return records, np.asarray(off, np.int64), truth


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
