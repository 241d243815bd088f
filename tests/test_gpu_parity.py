"""GPU parity: every stage of the sm_103a path against the CPU oracle on the
same seeded events, bit for bit (hit lists, track records, flags).

Each stage is checked by injection: the GPU stage gets the oracle's output of
the previous stage, so a mismatch points at one kernel.  The end-to-end test
runs the whole chain through one C-ABI call.
"""
import numpy as np
import pytest

from helpers import Snapshots, count_tracks, hit_mismatches, mixed_events, track_mismatches

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import pipeline
    plane, wp = geometry
    geo, rec, off, hits0 = mixed_events(plane, wp, 200, 200, seed=11)
    snap = Snapshots(plane, hits0)
    rc = pipeline.Reconstruction(plane, 0)
    return plane, geo, rec, off, hits0, snap, rc


def _batch(rc, n, pipeline_mod):
    return pipeline_mod.DeviceBatch(n, rc.device)


def test_event_reducer(setup):
    import torch
    from orgpu import pipeline
    plane, geo, rec, off, hits0, snap, rc = setup
    b = _batch(rc, hits0.n, pipeline)
    b.upload_hits(hits0)
    rc.event_reduce(b)
    rc.sync()
    assert hit_mismatches(b.download_hits(), snap.hits_er) == []
    np.testing.assert_array_equal(b.toomany.cpu().numpy(), snap.toomany_er)


def test_xz(setup):
    import torch
    from orgpu import pipeline
    plane, geo, rec, off, hits0, snap, rc = setup
    b = _batch(rc, hits0.n, pipeline)
    b.upload_hits(snap.hits_er)
    b.toomany.copy_(torch.from_numpy(snap.toomany_er))
    rc.xz_tracking(b)
    rc.sync()
    np.testing.assert_array_equal(b.toomany.cpu().numpy(), snap.toomany_xz)
    ok = snap.toomany_er == 0
    np.testing.assert_array_equal(b.ntracklets.cpu().numpy()[ok], snap.ntracklets[ok])
    assert track_mismatches(b.download_tracks(), snap.tracks_xz, snap.toomany_xz) == []
    assert int(snap.ntracklets.sum()) > 0


def test_yz(setup):
    import torch
    from orgpu import pipeline
    plane, geo, rec, off, hits0, snap, rc = setup
    b = _batch(rc, hits0.n, pipeline)
    b.upload_hits(snap.hits_er)
    b.toomany.copy_(torch.from_numpy(snap.toomany_xz))
    b.upload_tracks(snap.tracks_xz)
    rc.yz_tracking(b)
    rc.sync()
    assert track_mismatches(b.download_tracks(), snap.tracks_yz, snap.toomany_xz) == []
    assert count_tracks(snap.tracks_yz, 5) > 0


@pytest.mark.parametrize("limit", [0, 300, 5000])
def test_yz_survivor_pool_fallback(setup, limit):
    """The YZ path with the survivor pool limited, bit-exact with the oracle:
    limit 0 leaves no pool (the combined kernel runs every unit); 300 and
    5,000: units whose survivors do not fit run whole in the survivor kernel's
    combined fallback."""
    import torch
    from orgpu import pipeline
    plane, geo, rec, off, hits0, snap, rc = setup
    b = _batch(rc, hits0.n, pipeline)
    b.upload_hits(snap.hits_er)
    b.toomany.copy_(torch.from_numpy(snap.toomany_xz))
    b.upload_tracks(snap.tracks_xz)
    rc.set_yz_pool_limit(limit)
    try:
        rc.yz_tracking(b)
        rc.sync()
    finally:
        rc.set_yz_pool_limit(-1)
    assert track_mismatches(b.download_tracks(), snap.tracks_yz, snap.toomany_xz) == []


def test_back_clean(setup):
    import torch
    from orgpu import pipeline
    plane, geo, rec, off, hits0, snap, rc = setup
    b = _batch(rc, hits0.n, pipeline)
    b.toomany.copy_(torch.from_numpy(snap.toomany_xz))
    b.upload_hits(snap.hits_er)
    b.upload_tracks(snap.tracks_yz)
    rc.back_track_cleaning(b)
    rc.sync()
    assert track_mismatches(b.download_tracks(), snap.tracks_clean, snap.toomany_xz) == []


def test_global(setup):
    import torch
    from orgpu import pipeline
    plane, geo, rec, off, hits0, snap, rc = setup
    b = _batch(rc, hits0.n, pipeline)
    b.upload_hits(snap.hits_er)
    b.toomany.copy_(torch.from_numpy(snap.toomany_xz))
    b.upload_tracks(snap.tracks_clean)
    rc.global_tracking(b)
    rc.sync()
    assert track_mismatches(b.download_tracks(), snap.tracks_global, snap.toomany_xz) == []
    assert count_tracks(snap.tracks_global, 6) > 0


def test_post_global_selection(setup):
    import torch
    from orgpu import pipeline
    plane, geo, rec, off, hits0, snap, rc = setup
    b = _batch(rc, hits0.n, pipeline)
    b.upload_hits(snap.hits_er)
    b.toomany.copy_(torch.from_numpy(snap.toomany_xz))
    b.upload_tracks(snap.tracks_global)
    rc.prop_segment_matching(b)
    rc.global_track_cleaning(b)
    rc.sync()
    assert track_mismatches(b.download_tracks(), snap.tracks_sel, snap.toomany_xz) == []
    # the fused launch gives the same
    b.upload_tracks(snap.tracks_global)
    rc.selection(b)
    rc.sync()
    assert track_mismatches(b.download_tracks(), snap.tracks_sel, snap.toomany_xz) == []
    n6_before, n6_after = count_tracks(snap.tracks_global, 6), count_tracks(snap.tracks_sel, 6)
    assert 0 < n6_after < n6_before


def test_end_to_end(setup):
    from orgpu import pipeline
    plane, geo, rec, off, hits0, snap, rc = setup
    b = _batch(rc, hits0.n, pipeline)
    b.upload_hits(hits0)
    rc.run_batch(b)
    rc.sync()
    np.testing.assert_array_equal(b.toomany.cpu().numpy(), snap.state.toomany)
    np.testing.assert_array_equal(b.ntracklets.cpu().numpy(), snap.state.ntracklets)
    assert hit_mismatches(b.download_hits(), snap.hits_er) == []
    assert track_mismatches(b.download_tracks(), snap.tracks_global, snap.state.toomany) == []


def test_device_packer(setup):
    import torch
    from orgpu import pipeline
    plane, geo, rec, off, hits0, snap, rc = setup
    b = _batch(rc, hits0.n, pipeline)
    d_rec = torch.from_numpy(rec.view(np.uint8)).cuda()
    d_off = torch.from_numpy(off).cuda()
    d_wp = torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda()
    rc.pack(b, d_rec, d_off, d_wp)
    rc.sync()
    assert hit_mismatches(b.download_hits(), hits0) == []


def test_collect_tracks(setup):
    """The dense track output holds exactly the oracle's global tracks."""
    import torch
    from orgpu import layout as L, pipeline
    plane, geo, rec, off, hits0, snap, rc = setup
    b = _batch(rc, hits0.n, pipeline)
    b.upload_hits(snap.hits_er)
    b.toomany.copy_(torch.from_numpy(snap.state.toomany))
    b.upload_tracks(snap.tracks_global)
    out = torch.zeros(4096 * L.COLLECT_STRIDE, dtype=torch.float32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc.collect(b, out, cnt, 6.0)
    rc.sync()
    k = int(cnt.item())
    rows = out[:k * L.COLLECT_STRIDE].cpu().numpy().reshape(k, L.COLLECT_STRIDE)
    got = sorted((int(r[0]), int(r[1]), r[2:].tobytes()) for r in rows)
    want = []
    for e in range(hits0.n):
        if snap.state.toomany[e]:
            continue
        for s, j, r in snap.tracks_global.records(e):
            if r[L.TRK_STID] == 6:
                want.append((e, s * L.SLOTCAP + j, r.tobytes()))
    assert got == sorted(want)
