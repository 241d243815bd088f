"""Compact forms of the reference-layout buffers for golden fixtures, and the
comparisons the golden tests use.

Hit collections are stored as per-event counts [n, 54] (index = detector id)
plus the concatenated valid hit fields; track collections as slot counts
[n, 32] plus (event, slot, position) and the 148-float record of every valid
track.  Both are built from layout.HostHits / HostTracks and compare bit for
bit or, for fit parameters, within a relative tolerance.
"""
import numpy as np

from orgpu import layout as L

# track-record fields that are discrete (ids, counts, signs, charge) and must
# match exactly under any float rounding of the fits
DISCRETE_FIELDS = np.zeros(L.NTRKPARAM, bool)
DISCRETE_FIELDS[[L.TRK_STID, L.TRK_THREAD, L.TRK_NHITS, L.TRK_CHARGE]] = True
DISCRETE_FIELDS[L.TRK_HIT_DETID:L.TRK_HIT_DETID + 18] = True
DISCRETE_FIELDS[L.TRK_HIT_CHAN:L.TRK_HIT_CHAN + 18] = True
DISCRETE_FIELDS[L.TRK_HIT_SIGN:L.TRK_HIT_SIGN + 18] = True
# fit parameters the 1e-5 relative tolerance is stated for
FIT_FIELDS = [L.TRK_CHI2, L.TRK_TX, L.TRK_TY, L.TRK_X0, L.TRK_Y0, L.TRK_INVP, L.TRK_ERR_TX, L.TRK_ERR_TY,
              L.TRK_ERR_X0, L.TRK_ERR_Y0, L.TRK_ERR_INVP]


def compact_hits(h):
    """(counts int32 [n, 55], hits float32 [m]) -- hits in event, detector
    order, each plane's 5*count floats as stored (SoA)."""
    counts = np.zeros((h.n, L.NDET), np.int32)
    parts = []
    for e in range(h.n):
        for det in range(1, L.NDET):
            n, data = h.plane(e, det)
            counts[e, det] = n
            if n:
                parts.append(data.reshape(-1))
    flat = np.concatenate(parts) if parts else np.zeros(0, np.float32)
    return counts, flat.astype(np.float32)


def compact_tracks(t, toomany=None):
    """(ntracks uint16 [n, 32], where int32 [m, 3], records float32 [m, 148]).
    Events flagged in `toomany` are stored with no tracks."""
    nt = t.ntracks.reshape(t.n, L.NSLOTS).copy()
    if toomany is not None:
        nt[np.asarray(toomany, bool)] = 0
    where, recs = [], []
    for e in range(t.n):
        for s in range(L.NSLOTS):
            for k in range(int(nt[e, s])):
                base = e * L.EVT_TRK_FLOATS + (s * L.SLOTCAP + k) * L.NTRKPARAM
                where.append((e, s, k))
                recs.append(t.tracks[base:base + L.NTRKPARAM])
    w = np.array(where, np.int32).reshape(-1, 3)
    r = np.array(recs, np.float32).reshape(-1, L.NTRKPARAM)
    return nt, w, r


def compare_hits(a, b):
    """Bitwise: list of (event, detector) whose counts or hit data differ."""
    ca, fa = a
    cb, fb = b
    out = []
    if ca.shape != cb.shape:
        return [("shape", ca.shape, cb.shape)]
    oa = np.concatenate([[0], np.cumsum(5 * ca.reshape(-1))])
    ob = np.concatenate([[0], np.cumsum(5 * cb.reshape(-1))])
    for i in range(ca.size):
        if ca.flat[i] != cb.flat[i]:
            out.append((i // L.NDET, i % L.NDET, "count"))
        elif not np.array_equal(fa[oa[i]:oa[i + 1]].view(np.uint32), fb[ob[i]:ob[i + 1]].view(np.uint32)):
            out.append((i // L.NDET, i % L.NDET, "data"))
    return out


RESID_FIELDS = np.zeros(L.NTRKPARAM, bool)
RESID_FIELDS[L.TRK_HIT_RESID:L.TRK_HIT_RESID + 18] = True


def compare_tracks(a, b, rtol=0.0, resid_atol=None):
    """Compare compact track sets.  rtol == 0: every field bit for bit.
    rtol > 0: discrete fields exactly, the rest within rtol relative to
    max(|a|, |b|) (absolute 1e-6 near zero); hit residuals, which are
    differences of nearly equal numbers, within resid_atol (cm) when given.
    Returns a dict with the events whose slot counts differ, the records
    with a discrete difference, the records outside the tolerance, and the
    largest relative difference seen on the fit parameters."""
    nta, wa, ra = a
    ntb, wb, rb = b
    res = {"events": int(nta.shape[0]), "tracks": int(wa.shape[0]), "count_mismatch": [], "discrete_mismatch": [],
           "value_mismatch": [], "max_rel_fit": 0.0}
    bad_events = np.nonzero((nta != ntb).any(axis=1))[0]
    res["count_mismatch"] = [int(e) for e in bad_events]
    if bad_events.size:
        keep_a = ~np.isin(wa[:, 0], bad_events)
        keep_b = ~np.isin(wb[:, 0], bad_events)
        wa, ra, wb, rb = wa[keep_a], ra[keep_a], wb[keep_b], rb[keep_b]
    assert np.array_equal(wa, wb)
    if rtol == 0.0:
        diff = (ra.view(np.uint32) != rb.view(np.uint32)).any(axis=1)
        res["value_mismatch"] = [tuple(int(x) for x in wa[i]) for i in np.nonzero(diff)[0]]
        return res
    disc = (ra[:, DISCRETE_FIELDS] != rb[:, DISCRETE_FIELDS]).any(axis=1)
    res["discrete_mismatch"] = [tuple(int(x) for x in wa[i]) for i in np.nonzero(disc)[0]]
    ok = ~disc
    scale = np.maximum(np.abs(ra), np.abs(rb))
    err = np.abs(ra.astype(np.float64) - rb.astype(np.float64))
    tol = np.maximum(rtol * scale, 1e-6)
    if resid_atol is not None:
        tol[:, RESID_FIELDS] = resid_atol
    both_nan = np.isnan(ra) & np.isnan(rb)
    out = ((err > tol) & ~both_nan & ~DISCRETE_FIELDS[None, :]).any(axis=1) & ok
    res["value_mismatch"] = [tuple(int(x) for x in wa[i]) for i in np.nonzero(out)[0]]
    if ok.any():
        rel = err[ok][:, FIT_FIELDS] / np.maximum(scale[ok][:, FIT_FIELDS], 1e-30)
        rel[~np.isfinite(rel)] = 0.0
        res["max_rel_fit"] = float(rel.max()) if rel.size else 0.0
    return res


def compact_dimuons(d, toomany=None):
    """(ndimuons uint16 [n], records float32 [m, 36]) with the fields the
    reference never computes set to 0."""
    nd = d.ndimuons[:d.n].astype(np.uint16).copy()
    if toomany is not None:
        nd[np.asarray(toomany, bool)] = 0
    nd = np.minimum(nd, L.DIMUON_MAX)
    recs = [d.dimuons[e * L.EVT_DIM_FLOATS:e * L.EVT_DIM_FLOATS + int(nd[e]) * L.NDIMUONPARAM]
            for e in range(d.n)]
    r = (np.concatenate(recs) if recs else np.zeros(0, np.float32)).reshape(-1, L.NDIMUONPARAM).copy()
    r[:, list(L.DIM_UNSET_FIELDS)] = 0.0
    return nd, r


def compare_dimuons(a, b, rtol=0.0, phi_ulps=0):
    """Events whose dimuon counts differ, and records that differ: every
    field bit for bit (rtol == 0) or within rtol relative (1e-6 absolute
    near zero); phi within phi_ulps units in the last place (atan2f differs
    by a few ulps between the C library and CUDA)."""
    nda, ra = a
    ndb, rb = b
    res = {"events": int(nda.shape[0]), "dimuons": int(ra.shape[0]), "count_mismatch": [], "value_mismatch": []}
    res["count_mismatch"] = [int(e) for e in np.nonzero(nda != ndb)[0]]
    if res["count_mismatch"] or ra.shape != rb.shape:
        return res
    fields = np.ones(L.NDIMUONPARAM, bool)
    if phi_ulps:
        fields[L.DIM_PHI] = False
        ua, ub = ra[:, L.DIM_PHI].view(np.int32).astype(np.int64), rb[:, L.DIM_PHI].view(np.int32).astype(np.int64)
        phi_bad = np.abs(ua - ub) > phi_ulps
    else:
        phi_bad = np.zeros(len(ra), bool)
    if rtol == 0.0:
        bad = (ra[:, fields].view(np.uint32) != rb[:, fields].view(np.uint32)).any(axis=1) | phi_bad
    else:
        err = np.abs(ra.astype(np.float64) - rb.astype(np.float64))[:, fields]
        tol = np.maximum(rtol * np.maximum(np.abs(ra), np.abs(rb))[:, fields], 1e-6)
        both_nan = (np.isnan(ra) & np.isnan(rb))[:, fields]
        bad = ((err > tol) & ~both_nan).any(axis=1) | phi_bad
    res["value_mismatch"] = [int(i) for i in np.nonzero(bad)[0]]
    return res


def compare_hists(a, b, phi_slack=0):
    """Histogram counts [trigger, variable, bin]: every table equal, except
    that the dimuon phi table (variable 11) may move up to phi_slack counts
    between neighbouring bins (a last-place difference in phi at a bin edge).
    Returns the (trigger, variable) tables that differ."""
    va, vb = a.values_array(), b.values_array()
    out = []
    for t in range(L.HIST_NTRIGGERS):
        for k in range(L.HIST_NVARS):
            x, y = va[t, k], vb[t, k]
            if k == 11 and phi_slack:
                if x.sum() != y.sum() or np.abs(x - y).sum() > 2 * phi_slack:
                    out.append((t, k))
            elif not np.array_equal(x, y):
                out.append((t, k))
    return out


def select_events(rec, off, idx):
    """Records and offsets of the events `idx` (in that order)."""
    idx = np.asarray(idx, np.int64)
    parts = [rec[off[e]:off[e + 1]] for e in idx]
    lens = np.array([len(p) for p in parts], np.int64)
    new_off = np.concatenate([[0], np.cumsum(lens)]).astype(off.dtype)
    return (np.concatenate(parts) if parts else rec[:0]), new_off


# ---------------------------------------------------------------------------
# XZ candidates (oracle/ref/xz_pin.cuh): 32 floats per accepted candidate,
# [binId, thread, nhits, x0, tx, err_x0, err_tx, 0, then per hit n < 4:
# det, elem, x, drift, sign, tdc]
XZ_REC = 32
XZ_FIT = [3, 4, 5, 6]  # x0, tx, err_x0, err_tx


def xz_from_tracks(t, toomany):
    """The tracklets of an XZ output (HostTracks) as candidate records:
    (counts int32 [n], records float32 [m, 32]) in (event, slot, position)
    order; events flagged in `toomany` hold none."""
    cnt = np.zeros(t.n, np.int32)
    recs = []
    for e in range(t.n):
        if toomany is not None and toomany[e]:
            continue
        for s, k, r in t.records(e):
            v = np.zeros(XZ_REC, np.float32)
            nh = int(r[L.TRK_NHITS])
            v[:7] = [r[L.TRK_STID], r[L.TRK_THREAD], r[L.TRK_NHITS], r[L.TRK_X0], r[L.TRK_TX], r[L.TRK_ERR_X0],
                     r[L.TRK_ERR_TX]]
            for n in range(min(nh, 4)):
                v[8 + 6 * n:14 + 6 * n] = [r[L.TRK_HIT_DETID + n], r[L.TRK_HIT_CHAN + n], r[L.TRK_HIT_POS + n],
                                           r[L.TRK_HIT_DRIFT + n], r[L.TRK_HIT_SIGN + n], r[L.TRK_HIT_TDC + n]]
            recs.append(v)
            cnt[e] += 1
    return cnt, np.array(recs, np.float32).reshape(-1, XZ_REC)


def xz_from_pin(out, nout, events=None):
    """Candidate records of xz_pin_kernel's output (records [n, 32, cap, 32],
    counts [n, 32]) for the given events, in (event, thread, order) order."""
    n = out.shape[0]
    ev = range(n) if events is None else events
    cnt = np.zeros(len(ev), np.int32)
    recs = []
    for i, e in enumerate(ev):
        for t in range(32):
            k = int(nout[e, t])
            if k:
                recs.append(out[e, t, :k])
                cnt[i] += k
    return cnt, (np.concatenate(recs) if recs else np.zeros((0, XZ_REC), np.float32)).astype(np.float32)


def compare_xz(a, b, rtol=0.0):
    """Per event, the multiset of candidates of a (counts, records) against
    b's: candidates are matched on (binId, thread, hit ids, signs); fit fields
    and hit floats bit for bit (rtol 0) or within rtol.  Returns a dict:
    events, candidates, events whose candidate sets differ, candidates with a
    fit difference, the largest relative fit difference."""
    (ca, ra), (cb, rb) = a, b
    oa = np.concatenate([[0], np.cumsum(ca)])
    ob = np.concatenate([[0], np.cumsum(cb)])
    disc = [0, 1, 2] + [8 + 6 * n + f for n in range(4) for f in (0, 1, 4)]
    set_mismatch, value_mismatch, max_rel = [], [], 0.0
    for e in range(len(ca)):
        A, B = ra[oa[e]:oa[e + 1]], rb[ob[e]:ob[e + 1]]
        ka = sorted(range(len(A)), key=lambda i: tuple(A[i, disc]))
        kb = sorted(range(len(B)), key=lambda i: tuple(B[i, disc]))
        if len(A) != len(B) or any(not np.array_equal(A[i, disc], B[j, disc]) for i, j in zip(ka, kb)):
            set_mismatch.append(e)
            continue
        for i, j in zip(ka, kb):
            x, y = A[i], B[j]
            if rtol == 0.0:
                if not np.array_equal(x.view(np.uint32), y.view(np.uint32)):
                    value_mismatch.append((e, int(x[0])))
            else:
                d = np.abs(x.astype(np.float64) - y) / np.maximum(np.abs(y.astype(np.float64)), 1e-30)
                d[(x == y)] = 0.0
                m = float(d[XZ_FIT].max())
                max_rel = max(max_rel, m)
                if m > rtol:
                    value_mismatch.append((e, int(x[0])))
    return {"events": int(len(ca)), "candidates": int(ca.sum()), "set_mismatch": set_mismatch[:20],
            "n_set_mismatch": len(set_mismatch), "value_mismatch": value_mismatch[:20],
            "n_value_mismatch": len(value_mismatch), "max_rel_fit": max_rel}
