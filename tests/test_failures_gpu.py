"""Failures made on purpose, none of which faults, traps or hangs the GPU:

  - a bounded device wait that runs out: or_selftest_bounded_wait makes one
    warp wait on an mbarrier that nothing arrives at, for a few hundred
    polls; or_stream_sync must report OR_ERR_TIMEOUT, clear the error word,
    and the context must still give oracle-exact results afterwards;
  - hit records out of (det, elem, tdc) order given to or_pack_hits: the
    packer reports OR_ERR_ARG through or_stream_sync and writes nothing
    outside the event's slots;
  - records with detector ids outside 1..54 at the ends of an event: skipped,
    the rest packed as if they were absent;
  - serving admission refused when no slot fits in free device memory.

The reference has no recovery: its host aborts on a CUDA error
(online_reconstruction.cu:50-64) and its per-event soft failure is the
HasTooManyHits flag (reconstruction_kernels.cuh:135-139).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import hit_mismatches, make_events, track_mismatches

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _run_and_compare(torch, rc, plane, wp, seed):
    """A small batch through the whole path on `rc`, compared with the oracle."""
    from oracle import pyoracle as O
    from orgpu import layout as L, pipeline, synth as S
    geo, rec, off, hits, _ = make_events(plane, wp, S.config_small(48, seed))
    ref_h, ref_t, st = hits.copy(), L.HostTracks(hits.n), O.OracleState(hits.n)
    O.run_all(plane, ref_h, ref_t, st)
    b = pipeline.DeviceBatch(hits.n, 0)
    rc.pack(b, torch.from_numpy(rec.view(np.uint8)).cuda(), torch.from_numpy(off).cuda(),
            torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda())
    rc.run_batch(b)
    rc.sync()
    assert np.array_equal(b.toomany.cpu().numpy(), st.toomany)
    assert hit_mismatches(b.download_hits(), ref_h) == []
    assert track_mismatches(b.download_tracks(), ref_t, st.toomany) == []


def test_bounded_wait_runs_out_and_is_reported(cuda, geometry):
    from orgpu import _lib, pipeline
    torch = cuda
    plane, wp = geometry
    rc = pipeline.Reconstruction(plane, 0)
    lb = _lib.lib()
    assert lb.or_selftest_bounded_wait(rc.ctx, 0, _stream(torch)) == _lib.OR_ERR_ARG
    for _ in range(2):
        assert lb.or_selftest_bounded_wait(rc.ctx, 256, _stream(torch)) == _lib.OR_OK
        assert lb.or_stream_sync(rc.ctx, _stream(torch)) == _lib.OR_ERR_TIMEOUT
        assert "wait gave up" in lb.or_last_error().decode()
        # the error word was cleared by the report
        assert lb.or_stream_sync(rc.ctx, _stream(torch)) == _lib.OR_OK
    _run_and_compare(torch, rc, plane, wp, 906101)
    rc.close()


def test_unsorted_records_are_reported(cuda, geometry):
    from orgpu import _lib, pipeline, synth as S
    torch = cuda
    plane, wp = geometry
    geo, rec, off, hits, _ = make_events(plane, wp, S.config_small(32, 906102))
    bad = rec.copy()
    # event 0: its last record (highest detector id) moved to the front;
    # event 5: two records of different planes swapped in the middle
    r0, r1 = int(off[0]), int(off[1])
    bad[r0:r1] = np.concatenate([rec[r1 - 1:r1], rec[r0:r1 - 1]])
    a, b_ = int(off[5]) + 3, int(off[6]) - 4
    assert rec["det"][a] != rec["det"][b_]
    bad[a], bad[b_] = rec[b_], rec[a]
    rc = pipeline.Reconstruction(plane, 0)
    b = pipeline.DeviceBatch(hits.n, 0)
    d_wp = torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda()
    rc.pack(b, torch.from_numpy(bad.view(np.uint8)).cuda(), torch.from_numpy(off).cuda(), d_wp)
    with pytest.raises(_lib.OrError) as ei:
        rc.sync()
    assert ei.value.status == _lib.OR_ERR_ARG
    assert "not sorted" in _lib.lib().or_last_error().decode()
    rc.sync()  # cleared
    # the other events were packed as usual
    got = b.download_hits()
    from orgpu import layout as L
    for e in (1, 2, 3, 4, 6, 7, 31):
        for det in range(1, L.NDET):
            n1, d1 = got.plane(e, det)
            n2, d2 = hits.plane(e, det)
            assert n1 == n2 and np.array_equal(d1.view(np.uint32), d2.view(np.uint32)), (e, det)
    _run_and_compare(torch, rc, plane, wp, 906103)
    rc.close()


def test_out_of_range_detector_ids_are_skipped(cuda, geometry):
    from orgpu import layout as L, pipeline, synth as S
    torch = cuda
    plane, wp = geometry
    geo, rec, off, hits, _ = make_events(plane, wp, S.config_small(16, 906104))
    # each event gets a record with det 0 first and one with det 60 last
    lo = np.zeros(1, L.HIT_RECORD_DTYPE)
    lo["det"], lo["elem"], lo["tdc"], lo["flag"] = 0, 1, 1000.0, 2
    hi = lo.copy()
    hi["det"] = 60
    parts, noff = [], [0]
    for e in range(len(off) - 1):
        parts += [lo, rec[off[e]:off[e + 1]], hi]
        noff.append(noff[-1] + int(off[e + 1] - off[e]) + 2)
    rec2, off2 = np.concatenate(parts), np.array(noff, np.int64)
    rc = pipeline.Reconstruction(plane, 0)
    b = pipeline.DeviceBatch(hits.n, 0)
    rc.pack(b, torch.from_numpy(rec2.view(np.uint8)).cuda(), torch.from_numpy(off2).cuda(),
            torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda())
    rc.sync()
    assert hit_mismatches(b.download_hits(), hits) == []
    rc.close()


def test_serving_admission_refused_without_free_memory(cuda, geometry):
    from orgpu import _lib, serving
    plane, wp = geometry
    with pytest.raises(_lib.OrError) as ei:
        serving.Server(plane, wp, slot_events=256, max_slots=2, reserve_bytes=1 << 60)
    assert ei.value.status == _lib.OR_ERR_NOMEM
