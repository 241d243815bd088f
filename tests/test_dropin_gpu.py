"""The drop-in calls of include/or_dropin.h on the reference's own structs.

The reference host (online_reconstruction.cu:776-894) launches its kernels
on fixed-capacity structs of EstnEvtMax = 10000 events.  Here those structs
are laid out exactly as the reference allocates them (one buffer per
struct), filled with 400 mixed events followed by empty ones, and the five
drop-in calls are made in the reference's order with its arguments; the
result must equal or_run_batch on the same hits, bit for bit, and the
oracle's."""
import ctypes as C

import numpy as np
import pytest

from helpers import hit_mismatches, mixed_events, track_mismatches

pytestmark = pytest.mark.gpu


def _collection_buffers(torch, L, E):
    """gEventHitCollections / gEventTrackCollection as single device buffers,
    with typed views of their members (the reference's member order)."""
    hits = torch.zeros(int(L.REF_HITS_BYTES), dtype=torch.uint8, device="cuda")
    tracks = torch.zeros(int(L.REF_TRACKS_BYTES), dtype=torch.uint8, device="cuda")
    views, o = {}, 0
    for name, cnt, dt in (("nhits_cham", E * L.NCHAM, torch.int32), ("hits_cham", E * L.EVT_CHAM_FLOATS, torch.float32),
                          ("nhits_hodo", E * L.NHODO, torch.int32), ("hits_hodo", E * L.EVT_HODO_FLOATS, torch.float32),
                          ("nhits_prop", E * L.NPROP, torch.int32), ("hits_prop", E * L.EVT_PROP_FLOATS, torch.float32)):
        views[name] = hits[o:o + 4 * cnt].view(dt)
        o += 4 * cnt
    assert o == hits.numel()
    views["ntracks"] = tracks[:2 * E * L.NSLOTS].view(torch.int16)
    views["tracks"] = tracks[2 * E * L.NSLOTS:].view(torch.float32)
    return hits, tracks, views


def test_dropin_calls_equal_run_batch(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import pyoracle as O
    from orgpu import _lib, layout as L, pipeline
    plane, wp = geometry
    E = L.REF_EVTMAX
    _, _, _, h400 = mixed_events(plane, wp, 200, 200, seed=51)
    hits = L.HostHits(E)
    for big, small, per in zip(hits.arrays(), h400.arrays(), (L.NCHAM, L.EVT_CHAM_FLOATS, L.NHODO, L.EVT_HODO_FLOATS,
                                                               L.NPROP, L.EVT_PROP_FLOATS)):
        big[:small.size] = small
    # reference-layout structs
    hbuf, tbuf, v = _collection_buffers(torch, L, E)
    for name, arr in zip(("nhits_cham", "hits_cham", "nhits_hodo", "hits_hodo", "nhits_prop", "hits_prop"),
                         hits.arrays()):
        v[name].copy_(torch.from_numpy(arr.view(np.int32) if arr.dtype == np.uint32 else arr))
    d_plane = torch.frombuffer(bytearray(plane.to_bytes()), dtype=torch.uint8).cuda()
    flags = torch.zeros(E, dtype=torch.uint8, device="cuda")
    ntkl = torch.zeros(E, dtype=torch.int32, device="cuda")
    lb = _lib.lib()
    torch.cuda.synchronize()
    # online_reconstruction.cu:776-894, one call per launch
    for st in (lb.or_gkernel_eR(hbuf.data_ptr(), flags.data_ptr()),
               lb.or_gKernel_XZ_tracking(hbuf.data_ptr(), tbuf.data_ptr(), d_plane.data_ptr(), ntkl.data_ptr(),
                                         flags.data_ptr()),
               lb.or_gKernel_YZ_tracking(hbuf.data_ptr(), tbuf.data_ptr(), d_plane.data_ptr(), flags.data_ptr()),
               lb.or_gKernel_BackTrackCleaning(tbuf.data_ptr(), flags.data_ptr()),
               lb.or_gKernel_Global_tracking(hbuf.data_ptr(), tbuf.data_ptr(), d_plane.data_ptr(), flags.data_ptr())):
        _lib.check(st, "drop-in call")
    _lib.check(lb.or_dropin_sync(), "or_dropin_sync")
    torch.cuda.synchronize()
    # the same hits through or_run_batch
    rc = pipeline.Reconstruction(plane, 0)
    b = pipeline.DeviceBatch(E, 0)
    b.upload_hits(hits)
    rc.run_batch(b)
    rc.sync()
    assert torch.equal(flags, b.toomany)
    assert torch.equal(ntkl, b.ntracklets)
    for name in ("nhits_cham", "hits_cham", "nhits_hodo", "hits_hodo", "nhits_prop", "hits_prop"):
        a, c = v[name], getattr(b, name)
        if name.startswith("nhits"):
            assert torch.equal(a, c), name
    got_hits = b.download_hits()
    ref_hits = L.HostHits(E)
    for arr, name in zip(ref_hits.arrays(), ("nhits_cham", "hits_cham", "nhits_hodo", "hits_hodo", "nhits_prop",
                                             "hits_prop")):
        t = v[name].cpu().numpy()
        arr[:] = t.view(arr.dtype)
    assert hit_mismatches(ref_hits, got_hits) == []
    drop = L.HostTracks(E)
    drop.ntracks[:] = v["ntracks"].cpu().numpy().view(np.uint16)
    drop.tracks[:] = v["tracks"].cpu().numpy()
    toomany = flags.cpu().numpy()
    assert track_mismatches(drop, b.download_tracks(), toomany) == []
    # and the oracle, on the 400 filled events
    ho, to, st = h400.copy(), L.HostTracks(h400.n), O.OracleState(h400.n)
    O.run_all(plane, ho, to, st)
    assert np.array_equal(toomany[:h400.n], st.toomany)
    sub = L.HostTracks(h400.n)
    sub.ntracks[:] = drop.ntracks[:h400.n * L.NSLOTS]
    sub.tracks[:] = drop.tracks[:h400.n * L.EVT_TRK_FLOATS]
    assert track_mismatches(sub, to, st.toomany) == []
    rc.close()
