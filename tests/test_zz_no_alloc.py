"""or_yz_noalloc: the YZ stage on its static scratch area, through the C ABI,
against or_yz on the same buffers.

The file name sorts last so that pytest collects it after the other tests;
it builds its own events and context, so it also passes alone in a fresh
process.  Two calls in a row check that each call starts from cleared queue
counters.
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
