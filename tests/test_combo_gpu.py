"""The combination scorer (or_yz_scored): pruning of the station-3 (u3, v3)
outer iterations of queued YZ tracklets, checked by the properties that make
the plain method its arbiter, with a seeded untrained network (the properties
hold for any scores):

  - rows only (no model): the YZ output equals or_yz's bit for bit, and the
    labels mark at most one row per tracklet;
  - nothing pruned (t_keep = 0, every sigmoid score is above it): equal to
    or_yz bit for bit;
  - every row below t_keep with the uncertain band covering it: every event
    with rows runs plain, equal to or_yz;
  - a real cut: no tracklet gains an extension the plain method did not
    give it, a pruned result is never better than the plain one (its chi2 is
    the minimum over a subset of the combinations), and where it reaches the
    plain chi2 the record is the plain record bit for bit -- the kept
    combinations see the scratch state of the plain run;
  - everything pruned: the queued tracklets lose their extension, the other
    tracklets keep theirs bit for bit.
"""
import numpy as np
import pytest

from helpers import mixed_events

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def runs(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import layout as L, learned, pipeline
    plane, wp = geometry
    _, _, _, hits = mixed_events(plane, wp, 150, 350, seed=61)
    rc = pipeline.Reconstruction(plane, 0)
    cs = learned.ComboScorer(rc)
    b = pipeline.DeviceBatch(hits.n, 0)
    b.upload_hits(hits)
    rc.event_reduce(b)
    rc.xz_tracking(b)
    rc.sync()
    xz = (b.ntracks.clone(), b.tracks.clone())
    rc.yz_tracking(b)
    rc.sync()
    plain = (b.ntracks.clone(), b.tracks.clone())
    sp = learned.ScorerParams.init(np.zeros(L.NFEAT, np.float32), np.ones(L.NFEAT, np.float32), seed=3)
    model = learned.DeviceModel(sp)
    orows = learned.OuterRows(hits.n)

    def scored(m, t_keep, t_unc):
        b.ntracks.copy_(xz[0])
        b.tracks.copy_(xz[1])
        cs.yz(b, orows, m, t_keep, t_unc)
        rc.sync()
        return b.ntracks.clone(), b.tracks.clone()

    yield rc, cs, b, orows, model, plain, scored, hits
    rc.close()


def _recs(state, n):
    from orgpu import layout as L
    nt, tr = state
    return nt.view(n, L.NSLOTS), tr.view(n, L.NSLOTS, L.SLOTCAP, L.NTRKPARAM)


def _equal(a, b, n, toomany):
    import torch
    from orgpu import layout as L
    na, ta = _recs(a, n)
    nb, tb = _recs(b, n)
    keep = (toomany == 0)
    assert torch.equal(na[keep], nb[keep])
    valid = torch.arange(L.SLOTCAP, device=na.device)[None, None, :] < na.long()[:, :, None]
    valid &= keep[:, None, None]
    return int(((ta.view(torch.int32) != tb.view(torch.int32)).any(dim=3) & valid).sum()) == 0


def test_rows_only_and_nothing_pruned_equal_plain(runs):
    rc, cs, b, orows, model, plain, scored, hits = runs
    got = scored(None, 0.5, 0.5)
    assert _equal(got, plain, hits.n, b.toomany)
    nr = orows.n_rows()
    assert nr > 1000
    g = orows.outer[:nr]
    assert bool((g >= 0).all()) and bool((g < 100 * 100).all())
    got = scored(model, 0.0, 0.0)
    assert _equal(got, plain, hits.n, b.toomany)
    assert int(orows.uncertain[:hits.n].sum()) == 0
    s = orows.scores[:nr]
    assert bool(((s > 0) & (s < 1)).all())


def test_uncertain_band_runs_plain(runs):
    rc, cs, b, orows, model, plain, scored, hits = runs
    got = scored(model, 2.0, 0.0)  # every row below t_keep, every tracklet's best in the band
    assert _equal(got, plain, hits.n, b.toomany)
    assert int(orows.uncertain[:hits.n].sum()) > 0


def test_pruned_results_never_beat_plain(runs):
    import torch
    from orgpu import layout as L
    rc, cs, b, orows, model, plain, scored, hits = runs
    n = hits.n
    scored(model, 0.0, 0.0)
    nr = orows.n_rows()
    t = float(torch.quantile(orows.scores[:nr].float(), 0.6).item())  # prune about 60 % of the rows
    got = scored(model, t, t)  # an empty uncertain band
    na, ta = _recs(plain, n)
    nb, tb = _recs(got, n)
    keep = (b.toomany == 0)
    assert torch.equal(na[keep], nb[keep])  # slot counts: the XZ tracklets
    valid = (torch.arange(L.SLOTCAP, device=na.device)[None, None, :] < na.long()[:, :, None]) & keep[:, None, None]
    ext_p = (ta[..., L.TRK_STID] == 5) & valid
    ext_g = (tb[..., L.TRK_STID] == 5) & valid
    assert not bool((ext_g & ~ext_p).any())  # no new extension
    both = ext_p & ext_g
    cp, cg = ta[..., L.TRK_CHI2][both], tb[..., L.TRK_CHI2][both]
    assert bool((cg >= cp).all())
    same = (cg == cp)
    ra = ta[both][same].view(torch.int32)
    rb = tb[both][same].view(torch.int32)
    assert torch.equal(ra, rb)
    lost = int((ext_p & ~ext_g).sum()) + int((~same).sum())
    assert lost > 0  # the cut did prune something


def test_everything_pruned_drops_queued_tracklets_only(runs):
    import torch
    from orgpu import layout as L
    rc, cs, b, orows, model, plain, scored, hits = runs
    n = hits.n
    got = scored(model, 2.0, 1.5)  # all rows below t_keep, none in the band
    assert int(orows.uncertain[:n].sum()) == 0
    na, ta = _recs(plain, n)
    nb, tb = _recs(got, n)
    keep = (b.toomany == 0)
    valid = (torch.arange(L.SLOTCAP, device=na.device)[None, None, :] < na.long()[:, :, None]) & keep[:, None, None]
    ext_p = (ta[..., L.TRK_STID] == 5) & valid
    ext_g = (tb[..., L.TRK_STID] == 5) & valid
    assert not bool((ext_g & ~ext_p).any())
    assert int(ext_g.sum()) < int(ext_p.sum())
    # the tracklets still extended (the ones evaluated in the planning pass)
    # carry the plain record bit for bit
    assert torch.equal(ta[ext_g].view(torch.int32), tb[ext_g].view(torch.int32))


def test_kept_list_equals_range_walk(runs):
    """The first-cut kernel walks the kept iterations as a list with the
    pruned ones' scratch writes folded in; with no survivor pool every unit
    runs on the combined kernel, and with a pool of one entry on the survivor
    kernel's combined fallback, both of which walk the unit's whole range and
    jump over the pruned iterations.  All give the same records bit for bit
    at any cut."""
    import torch
    rc, cs, b, orows, model, plain, scored, hits = runs
    scored(model, 0.0, 0.0)
    nr = orows.n_rows()
    for q in (0.3, 0.6, 0.9):
        t = float(torch.quantile(orows.scores[:nr].float(), q).item())
        listed = scored(model, t, t)
        for limit in (0, 1):  # no pool: the combined kernel; one entry: the survivor kernel's fallback
            rc.set_yz_pool_limit(limit)
            try:
                walked = scored(model, t, t)
            finally:
                rc.set_yz_pool_limit(-1)
            assert _equal(listed, walked, hits.n, b.toomany)
