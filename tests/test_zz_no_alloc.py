"""or_yz_noalloc: the YZ stage on its static scratch area, through the C ABI,
against or_yz on the same buffers.

The file name sorts last so that pytest collects it after the other tests;
it builds its own events and context, so it also passes alone in a fresh
process.  Two calls in a row check that each call starts from cleared queue
counters.  A batch at the entry point's event limit (10,000 uneven-noise
events) holds far more heavy tracklets than its static queue (16,384), so
there the planning warps evaluate the tracklets that find the queue full;
the results must still equal or_yz's bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import count_tracks, mixed_events, track_mismatches


def test_noalloc_rejects_batches_above_the_limit():
    """The event-count check runs on the host before any CUDA call."""
    from orgpu import _lib, layout as L
    lb = _lib.lib()
    rc = lb.or_yz_noalloc(None, L.OrHitsView(), L.OrTracksView(), None, _lib.OR_YZ_NOALLOC_MAX_EVENTS + 1, None,
                          None)
    assert rc == _lib.OR_ERR_CAPACITY
    msg = lb.or_last_error().decode()
    assert str(_lib.OR_YZ_NOALLOC_MAX_EVENTS) in msg and "or_yz_noalloc" in msg
    assert lb.or_yz_noalloc(None, L.OrHitsView(), L.OrTracksView(), None, -1, None, None) == _lib.OR_ERR_ARG


@pytest.mark.gpu
def test_noalloc_matches_or_yz_twice(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import _lib, pipeline
    plane, wp = geometry
    _, _, _, hits0 = mixed_events(plane, wp, 150, 250, seed=23)
    rc = pipeline.Reconstruction(plane, 0)
    b = pipeline.DeviceBatch(hits0.n, 0)
    b.upload_hits(hits0)
    rc.event_reduce(b)
    rc.xz_tracking(b)
    rc.sync()
    ntracks_xz, tracks_xz = b.ntracks.clone(), b.tracks.clone()

    rc.yz_tracking(b)
    rc.sync()
    want = b.download_tracks()
    toomany = b.toomany.cpu().numpy()
    assert count_tracks(want, 5) > 0

    lb = _lib.lib()
    d_plane = torch.frombuffer(bytearray(plane.to_bytes()), dtype=torch.uint8).cuda()
    d_errw = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        b.ntracks.copy_(ntracks_xz)
        b.tracks.copy_(tracks_xz)
        status = lb.or_yz_noalloc(d_plane.data_ptr(), b.hits_view(), b.tracks_view(), b.toomany.data_ptr(), b.n,
                                  d_errw.data_ptr(), stream)
        _lib.check(status, f"or_yz_noalloc call {call}")
        torch.cuda.synchronize()
        assert int(d_errw.item()) == 0
        got = b.download_tracks()
        np.testing.assert_array_equal(got.ntracks, want.ntracks)
        assert track_mismatches(got, want, toomany) == [], f"call {call}"
    rc.close()


NOALLOC_HEAVY = 16384  # heavy-tracklet entries of the static queue (csrc/yz_noalloc.cu)


def _heavy_lower_bound(rc, b):
    """Tracklets that certainly go to the YZ queue (more than 32 live
    combinations), from the scorer features of the XZ output: per u2/v2
    projection at least ceil(windowed/2) pairs, per u3/v3 projection at least
    ceil(accepted/2) pairs with an accepted hit.  Tracklets whose windows
    could overflow the 100-entry lists are left out."""
    from orgpu import learned
    r = learned.TrackletRows(b.n, device=0)
    lrn = learned.Learned(rc)
    lrn.rows(b, r)
    lrn.features(b, r)
    rc.sync()
    n = r.n_rows()
    f = r.features[:n * learned.NF].view(n, learned.NF).cpu().numpy()
    win = np.rint(np.expm1(f[:, 7:11])).astype(np.int64)
    acc = np.rint(np.expm1(f[:, 11:15])).astype(np.int64)
    half = lambda x: (x + 1) // 2  # noqa: E731
    lb = half(acc[:, 2]) * half(acc[:, 3]) * half(win[:, 0]) * half(win[:, 1])
    return int(((lb > 32) & (win <= 18).all(axis=1)).sum())


@pytest.mark.gpu
def test_noalloc_at_its_event_limit_matches_or_yz(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import _lib, layout as L, pipeline, synth as S
    plane, wp = geometry
    n = _lib.OR_YZ_NOALLOC_MAX_EVENTS
    geo = S.Geometry(plane, wp)
    rec, off, _ = S.generate(geo, S.config_uneven(n, 906011))
    rec, off = S.cap_records(rec, off)
    rc = pipeline.Reconstruction(plane, 0)
    b = pipeline.DeviceBatch(n, 0)
    rc.pack(b, torch.from_numpy(rec.view(np.uint8)).cuda(), torch.from_numpy(off).cuda(),
            torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda())
    rc.event_reduce(b)
    rc.xz_tracking(b)
    rc.sync()
    heavy = _heavy_lower_bound(rc, b)
    assert heavy > 2 * NOALLOC_HEAVY, heavy  # the queue-full path must run
    ntracks_xz, tracks_xz = b.ntracks.clone(), b.tracks.clone()
    rc.yz_tracking(b)
    rc.sync()
    want_n, want_t = b.ntracks.clone(), b.tracks.clone()
    keep = (b.toomany == 0)
    valid = torch.arange(L.SLOTCAP, device="cuda")[None, None, :] < want_n.view(n, L.NSLOTS).long()[:, :, None]
    valid &= keep[:, None, None]
    assert int(valid.sum()) > 100000

    lb = _lib.lib()
    d_plane = torch.frombuffer(bytearray(plane.to_bytes()), dtype=torch.uint8).cuda()
    d_errw = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        b.ntracks.copy_(ntracks_xz)
        b.tracks.copy_(tracks_xz)
        status = lb.or_yz_noalloc(d_plane.data_ptr(), b.hits_view(), b.tracks_view(), b.toomany.data_ptr(), n,
                                  d_errw.data_ptr(), stream)
        _lib.check(status, f"or_yz_noalloc call {call}")
        torch.cuda.synchronize()
        assert int(d_errw.item()) == 0
        assert torch.equal(b.ntracks, want_n), f"call {call}: slot counts"
        got = b.tracks.view(torch.int32).view(n, L.NSLOTS, L.SLOTCAP, L.NTRKPARAM)
        ref = want_t.view(torch.int32).view(n, L.NSLOTS, L.SLOTCAP, L.NTRKPARAM)
        bad = ((got != ref).any(dim=3) & valid).sum()
        assert int(bad) == 0, f"call {call}: {int(bad)} track records differ"
    rc.close()
