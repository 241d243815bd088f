"""GPU parity of the stages after the selection -- vertexing, dimuon building
and the monitoring histograms -- against the CPU oracle on the same seeded
events.

Each stage is fed the oracle's output of the stage before it (injection):
  - vertexed tracks: every field bit for bit;
  - dimuons: counts and every field bit for bit, except phi, which comes
    from atan2f (CUDA's and the C library's may differ in the last places);
  - histograms: every count equal, the phi table up to a count moved between
    neighbouring bins by such a last-place difference.
"""
import numpy as np
import pytest

from helpers import Snapshots, mixed_events, track_mismatches

pytestmark = pytest.mark.gpu

PHI_ULPS = 4


@pytest.fixture(scope="module")
def setup(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import pyoracle as O
    from orgpu import layout as L, pipeline, synth as S
    plane, wp = geometry
    geo, rec, off, hits0 = mixed_events(plane, wp, 600, 600, seed=23)
    snap = Snapshots(plane, hits0)
    n = hits0.n
    st = O.OracleState(n)
    st.toomany[:] = snap.toomany_xz
    tv = snap.tracks_sel.copy()
    O.vertexing(plane, tv, st)
    dims = L.HostDimuons(n)
    O.dimuons(plane, tv, dims, st)
    trig = S.trigger_bits(n, seed=77)
    hists = O.hist_table()
    O.fill_histograms(tv, dims, hists, trig, st)
    rc = pipeline.Reconstruction(plane, 0)
    return dict(plane=plane, snap=snap, n=n, tv=tv, dims=dims, trig=trig, hists=hists, rc=rc)


def _batch(s, tracks):
    import torch
    from orgpu import pipeline
    b = pipeline.DeviceBatch(s["n"])
    b.upload_hits(s["snap"].hits_er)
    b.upload_tracks(tracks)
    b.toomany.copy_(torch.from_numpy(s["snap"].toomany_xz))
    return b


def _dims(s):
    import torch
    from orgpu import pipeline
    d = pipeline.DeviceDimuons(s["n"])
    d.ndimuons.copy_(torch.from_numpy(s["dims"].ndimuons.view(np.int16)))
    d.dimuons.copy_(torch.from_numpy(s["dims"].dimuons))
    return d


def test_vertexing_bit_exact(setup):
    s = setup
    b = _batch(s, s["snap"].tracks_sel)
    s["rc"].vertexing(b)
    s["rc"].sync()
    got = b.download_tracks()
    assert track_mismatches(got, s["tv"], s["snap"].toomany_xz) == []
    n7 = sum(1 for e in range(s["n"]) for _, _, r in got.records(e) if r[0] == 7 and not s["snap"].toomany_xz[e])
    assert n7 > 100


def test_dimuons(setup):
    import golden_io as G
    from orgpu import pipeline
    s = setup
    b = _batch(s, s["tv"])
    d = pipeline.DeviceDimuons(s["n"])
    s["rc"].dimuons(b, d)
    s["rc"].sync()
    got = d.download()
    r = G.compare_dimuons(G.compact_dimuons(got, s["snap"].toomany_xz),
                          G.compact_dimuons(s["dims"], s["snap"].toomany_xz), 0.0, phi_ulps=PHI_ULPS)
    assert r["count_mismatch"] == [] and r["value_mismatch"] == [], r
    assert r["dimuons"] > 20


def test_histograms(setup):
    import torch
    import golden_io as G
    from orgpu import pipeline
    s = setup
    b = _batch(s, s["tv"])
    d = _dims(s)
    h = pipeline.DeviceHists()
    tb = torch.from_numpy(s["trig"]).cuda()
    s["rc"].fill_histograms(b, d, h, tb)
    s["rc"].sync()
    got = h.download()
    assert G.compare_hists(got, s["hists"], phi_slack=2) == []
    assert got.values_array().sum() > 1000
    # a second fill adds the same counts again
    s["rc"].fill_histograms(b, d, h, tb)
    s["rc"].sync()
    np.testing.assert_array_equal(h.download().values_array(), 2 * got.values_array())
    h.zero_counts()
    assert h.download().values_array().sum() == 0


def test_run_physics_equals_the_three_calls(setup):
    import torch
    from orgpu import pipeline
    s = setup
    b = _batch(s, s["snap"].tracks_sel)
    d = pipeline.DeviceDimuons(s["n"])
    h = pipeline.DeviceHists()
    tb = torch.from_numpy(s["trig"]).cuda()
    s["rc"].run_physics(b, d, h, tb)
    s["rc"].sync()
    b2 = _batch(s, s["snap"].tracks_sel)
    d2 = pipeline.DeviceDimuons(s["n"])
    h2 = pipeline.DeviceHists()
    s["rc"].vertexing(b2)
    s["rc"].dimuons(b2, d2)
    s["rc"].fill_histograms(b2, d2, h2, tb)
    s["rc"].sync()
    assert torch.equal(b.tracks, b2.tracks) and torch.equal(d.dimuons, d2.dimuons)
    assert torch.equal(d.ndimuons, d2.ndimuons) and torch.equal(h.buf, h2.buf)


def test_flagged_events_untouched(setup):
    import torch
    from orgpu import pipeline
    s = setup
    b = _batch(s, s["snap"].tracks_sel)
    b.toomany.fill_(1)
    before = b.tracks.clone()
    d = pipeline.DeviceDimuons(s["n"])
    d.ndimuons.fill_(-1)
    s["rc"].vertexing(b)
    s["rc"].dimuons(b, d)
    s["rc"].sync()
    assert torch.equal(before, b.tracks)
    assert bool((d.ndimuons == -1).all())


@pytest.mark.parametrize("min_stid", [7.0, 5.0])
def test_output_rows(setup, min_stid):
    """The reference's output tree fields as row tables, event order, bit for
    bit against the restated host loop; events without raw hits skipped."""
    import torch
    from helpers import output_rows_oracle
    s = setup
    n = s["n"]
    b = _batch(s, s["tv"])
    d = _dims(s)
    raw = np.full(n, 5, np.int32)
    raw[::7] = 0
    ids = np.arange(n, dtype=np.int32) * 3 + 1000
    got = s["rc"].output_rows(b, d, torch.from_numpy(raw).cuda(), torch.from_numpy(ids).cuda(), min_stid)
    want = output_rows_oracle(s["snap"].hits_er, s["tv"], s["dims"], s["snap"].toomany_xz, raw, ids, min_stid)
    for k in ("events", "hits", "tracks", "track_hits", "dimuons"):
        assert got[k].shape == want[k].shape, k
        if k == "events":
            np.testing.assert_array_equal(got[k], want[k])
        else:
            assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), k
    assert len(got["tracks"]) > 50 and len(got["dimuons"]) > 10


def test_output_rows_capacity(setup):
    import torch
    from orgpu import _lib
    s = setup
    b = _batch(s, s["tv"])
    d = _dims(s)
    with pytest.raises(_lib.OrError):
        s["rc"].output_rows(b, d, caps=(10, 10, 10, 10, 10))
