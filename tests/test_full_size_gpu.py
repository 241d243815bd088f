"""The plain path at the configurations' full sizes.

Against the oracle, bit for bit (hit lists after the event reducer, the
HasTooManyHits flag, nTracklets, slot counts, every track record):

  - all 100,000 events of the uneven batch (seed 906002), run by one
    or_run_batch call on the whole batch; the oracle runs in chunks of
    5,000 events (events are independent), each chunk compared on the
    device with its rows of the GPU batch;
  - the small configuration at exactly its size: 1,000 one-dimuon events
    with Poisson(150) noise, seed 906001;
  - 20,000 events of the high-occupancy workload (two muons, Poisson(1000)
    noise, after-pulses), every one of which the event reducer rejects.

And through properties that do not need the oracle:

  - determinism: the same batch run twice gives the same buffers, bit for bit;
  - event independence: the batch run as four chunks gives, event by event,
    the same tracks and flags as the batch run whole (the work queue, the
    planning units and the overflow arenas differ between the two);
  - sized contexts: 20,000 events of the batch give the same buffers on a
    context sized for them (or_create_sized) and on one sized for 1,000
    events, whose YZ queue, survivor pool and window images overflow (the
    excess evaluated in the planning pass, on the combined path, or windowed
    again), as on the default context;
  - well-formed output: every global track has 5-18 hits with detector ids
    in the chamber range, charge +-1, a finite chi2 and 1/p in the window
    the global stage enforces;
  - R-T conversion: the packer with the calibration fused in equals the
    plain packer followed by the in-place conversion, bit for bit, and
    changes only the chamber and prop-tube drift fields.

Stage-by-stage parity (each stage fed the oracle's previous stage) is in
test_gpu_parity.py; this file adds the full-size behaviour of the queue and
the scratch limits.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_EVENTS = 100000


@pytest.fixture(scope="module")
def full(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import synth as S
    plane, wp = geometry
    geo = S.Geometry(plane, wp)
    rec, off, _ = S.generate(geo, S.config_uneven(N_EVENTS, 906002))
    rec, off = S.cap_records(rec, off)
    return plane, geo, rec, off


def _run(plane, geo, rec, off, max_events=None):
    import torch
    from orgpu import pipeline
    n = len(off) - 1
    rc = pipeline.Reconstruction(plane, 0, max_events=max_events)
    b = pipeline.DeviceBatch(n)
    rc.pack(b, torch.from_numpy(rec.view(np.uint8)).cuda(), torch.from_numpy(off).cuda(),
            torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda())
    rc.run_batch(b)
    rc.sync()
    t = b.download_tracks()
    return t.ntracks.reshape(n, -1).copy(), t.tracks.reshape(n, -1).copy(), b.toomany.cpu().numpy().copy()


def _run_device(plane, geo, rec, off):
    """or_run_batch on the whole batch; the DeviceBatch stays on the device."""
    import torch
    from orgpu import pipeline
    n = len(off) - 1
    rc = pipeline.Reconstruction(plane, 0)
    b = pipeline.DeviceBatch(n)
    rc.pack(b, torch.from_numpy(rec.view(np.uint8)).cuda(), torch.from_numpy(off).cuda(),
            torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda())
    rc.run_batch(b)
    rc.sync()
    return b


def _assert_oracle_equal(plane, geo, rec, off, chunk):
    from helpers import device_mismatches, oracle_chunk
    n = len(off) - 1
    b = _run_device(plane, geo, rec, off)
    total = {}
    for e0 in range(0, n, chunk):
        e1 = min(n, e0 + chunk)
        h, t, st = oracle_chunk(plane, geo, rec, off, e0, e1)
        m = device_mismatches(b, e0, h, t, st)
        for k, v in m.items():
            total[k] = total.get(k, 0) + v
        bad = {k: v for k, v in m.items() if v and k not in ("tracks_compared", "global_tracks")}
        assert not bad, f"events {e0}..{e1}: {bad}"
    return total


def test_full_batch_bit_exact_with_oracle(full):
    plane, geo, rec, off = full
    total = _assert_oracle_equal(plane, geo, rec, off, 5000)
    assert total["global_tracks"] > 100000
    print("uneven batch, 100,000 events:", total)


def test_small_config_1000_events_bit_exact_with_oracle(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import synth as S
    plane, wp = geometry
    geo = S.Geometry(plane, wp)
    rec, off, _ = S.generate(geo, S.config_small(1000, 906001))
    rec, off = S.cap_records(rec, off)
    total = _assert_oracle_equal(plane, geo, rec, off, 1000)
    assert total["global_tracks"] > 1000
    print("small configuration, 1,000 events:", total)


def test_high_occupancy_rejection_equals_oracle(geometry):
    """The high-occupancy workload (two muons, Poisson(1000) noise, 10 %
    after-pulses; 20,000 events): every stage's output equals the oracle's
    bit for bit, and the event reducer's station limits reject every event,
    in the library as in the oracle."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import synth as S
    plane, wp = geometry
    geo = S.Geometry(plane, wp)
    rec, off, _ = S.generate(geo, S.config_high_occupancy(20000, 906004))
    rec, off = S.cap_records(rec, off)
    b = _run_device(plane, geo, rec, off)
    assert bool((b.toomany != 0).all())
    _assert_oracle_equal(plane, geo, rec, off, 5000)


def _valid_tracks(nt, tr):
    """records of the valid slots only (the rest of a slot is never written)"""
    n = nt.shape[0]
    T = tr.reshape(n, 32, 16, 148)
    m = np.arange(16)[None, None, :] < nt.reshape(n, 32)[:, :, None].astype(np.int64)
    return T, m


def test_full_batch_deterministic_and_chunk_independent(full):
    plane, geo, rec, off = full
    nt1, tr1, f1 = _run(plane, geo, rec, off)
    nt2, tr2, f2 = _run(plane, geo, rec, off)
    np.testing.assert_array_equal(nt1, nt2)
    np.testing.assert_array_equal(f1, f2)
    T1, m1 = _valid_tracks(nt1, tr1)
    T2, _ = _valid_tracks(nt2, tr2)
    assert np.array_equal(T1[m1].view(np.uint32), T2[m1].view(np.uint32))
    # four chunks
    n = len(off) - 1
    cuts = np.linspace(0, n, 5).astype(int)
    for a, b in zip(cuts[:-1], cuts[1:]):
        r = rec[off[a]:off[b]]
        o = (off[a:b + 1] - off[a]).astype(off.dtype)
        ntc, trc, fc = _run(plane, geo, r, o)
        np.testing.assert_array_equal(ntc, nt1[a:b])
        np.testing.assert_array_equal(fc, f1[a:b])
        Tc, mc = _valid_tracks(ntc, trc)
        assert np.array_equal(Tc[mc].view(np.uint32), T1[a:b][mc].view(np.uint32))


def test_full_batch_tracks_well_formed(full):
    from orgpu import layout as L
    plane, geo, rec, off = full
    nt, tr, flags = _run(plane, geo, rec, off)
    T, m = _valid_tracks(nt, tr)
    recs = T[m & (flags == 0)[:, None, None]]
    g = recs[recs[:, L.TRK_STID] == 6]
    assert len(g) > 100000
    nh = g[:, L.TRK_NHITS].astype(int)
    assert ((nh >= 5) & (nh <= 18)).all()
    for row, k in zip(g, nh):
        d = row[L.TRK_HIT_DETID:L.TRK_HIT_DETID + k]
        assert ((d >= 1) & (d <= 30)).all()
    assert np.isin(g[:, L.TRK_CHARGE], (-1.0, 1.0)).all()
    assert np.isfinite(g[:, L.TRK_CHI2]).all()
    invp = g[:, L.TRK_INVP]
    assert ((invp > 0.0) & (invp < 0.25)).all()


def test_full_batch_rt_fused_equals_apply(full):
    """R-T conversion at full size: the packer with the calibration fused in
    gives the same hit buffers, bit for bit, as the plain packer followed by
    the in-place conversion; and only the drift field of chamber and
    prop-tube hits changes against the plain packer."""
    import torch
    from orgpu import CALIBRATION_E906, _lib, layout as L, pipeline
    plane, geo, rec, off = full
    n = len(off) - 1
    rc = pipeline.Reconstruction(plane, 0)
    d_rec = torch.from_numpy(rec.view(np.uint8)).cuda()
    d_off = torch.from_numpy(off).cuda()
    d_wp = torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda()
    rt, _ = _lib.rt_load(CALIBRATION_E906, plane)
    d_rt = pipeline.rt_to_device(rt)
    fused = pipeline.DeviceBatch(n, with_tracks=False)
    applied = pipeline.DeviceBatch(n, with_tracks=False)
    plain = pipeline.DeviceBatch(n, with_tracks=False)
    for b in (fused, applied, plain):
        for t in (b.hits_cham, b.hits_hodo, b.hits_prop):
            t.zero_()
    rc.pack_rt(fused, d_rec, d_off, d_wp, d_rt)
    rc.pack(applied, d_rec, d_off, d_wp)
    rc.rt_apply(applied, d_rt)
    rc.pack(plain, d_rec, d_off, d_wp)
    rc.sync()
    for name in ("nhits_cham", "hits_cham", "nhits_hodo", "hits_hodo", "nhits_prop", "hits_prop"):
        a, b = getattr(fused, name), getattr(applied, name)
        assert torch.equal(a.view(torch.int32), b.view(torch.int32)), name
    # hodoscopes untouched; chambers and prop tubes differ only in the drift field
    assert torch.equal(fused.hits_hodo.view(torch.int32), plain.hits_hodo.view(torch.int32))
    for name, per, cap in (("cham", L.NCHAM, L.MAXHITS_CHAM), ("prop", L.NPROP, L.MAXHITS_PROP)):
        f = getattr(fused, "hits_" + name).view(n, per, L.NHITSPARAM, cap)
        p = getattr(plain, "hits_" + name).view(n, per, L.NHITSPARAM, cap)
        # with the slot stride = count, the drift field is the last count
        # floats of each slot's 5*count head; the first four fields match
        cnt = getattr(plain, "nhits_" + name).view(n, per).long()
        flat_f = f.reshape(n * per, -1)
        flat_p = p.reshape(n * per, -1)
        idx = torch.arange(L.NHITSPARAM * cap, device=f.device)[None, :]
        head = idx < 4 * cnt.reshape(-1, 1)
        assert torch.equal(flat_f[head].view(torch.int32), flat_p[head].view(torch.int32)), name
        changed = (flat_f.view(torch.int32) != flat_p.view(torch.int32)).any(dim=1)
        assert bool(changed.any()), name


def test_sized_contexts_equal_default(full):
    plane, geo, rec, off = full
    n = 20000
    r, o = rec[:off[n]], off[:n + 1]
    nt0, tr0, f0 = _run(plane, geo, r, o)
    T0, m0 = _valid_tracks(nt0, tr0)
    for cap in (n, 1000):
        nt, tr, f = _run(plane, geo, r, o, max_events=cap)
        np.testing.assert_array_equal(nt, nt0)
        np.testing.assert_array_equal(f, f0)
        T, _ = _valid_tracks(nt, tr)
        assert np.array_equal(T[m0].view(np.uint32), T0[m0].view(np.uint32))
