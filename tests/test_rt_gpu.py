"""R-T conversion on the GPU: the device packer's drift field from the
calibration (or_pack_hits_rt) and the in-place conversion of packed hits
(or_rt_apply), against the CPU oracle, bit for bit.

The hit times are drawn to hit every branch of the conversion: inside the
window, below tmin (half a cell), above tmax (zero), exactly on tmin, tmax and
the calibration knots, and one float step either side of a knot (where the
piece index changes).
"""
import numpy as np
import pytest

from helpers import hit_mismatches, mixed_events
from oracle.rt_oracle import RtOracle, rt_plane
from orgpu import CALIBRATION_E906, layout as L, synth as S

pytestmark = pytest.mark.gpu


def _rt_times(rec, o, rng):
    """Replace the tdc of every record on a plane with a profile."""
    rec = rec.copy()
    det = rec["det"].astype(np.int64)
    tdc = rec["tdc"].copy()
    for p, (tmin, tmax, T, R, *_) in o.planes.items():
        sel = np.nonzero(det == p)[0]
        if len(sel) == 0:
            continue
        kind = rng.integers(0, 10, len(sel))
        t = rng.uniform(float(tmin) - 20.0, float(tmax) + 20.0, len(sel)).astype(np.float32)
        knot = T[rng.integers(0, len(T), len(sel))].astype(np.float32)
        t = np.where(kind == 0, knot, t)
        t = np.where(kind == 1, np.nextafter(knot, np.float32(np.inf)), t)
        t = np.where(kind == 2, np.nextafter(knot, np.float32(-np.inf)), t)
        t = np.where(kind == 3, np.where(rng.integers(0, 2, len(sel)) == 0, tmin, tmax), t)
        tdc[sel] = t.astype(np.float32)
    rec["tdc"] = tdc
    return rec


def _sorted(rec, off):
    ev = np.repeat(np.arange(len(off) - 1), np.diff(off))
    order = np.lexsort((rec["tdc"], rec["elem"], rec["det"], ev))
    return rec[order]


@pytest.fixture(scope="module")
def setup(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import _lib, pipeline
    plane, wp = geometry
    geo, rec, off, _ = mixed_events(plane, wp, 600, 600, seed=23)
    o = RtOracle.from_file(CALIBRATION_E906, plane.arr("cellwidth"))
    rec = _sorted(_rt_times(rec, o, np.random.default_rng(5)), off)
    want_rec = rec.copy()
    want_rec["drift"] = o.drift(rec["det"], rec["tdc"], rec["drift"])
    rt, _ = _lib.rt_load(CALIBRATION_E906, plane)
    rc = pipeline.Reconstruction(plane, 0)
    d_rt = pipeline.rt_to_device(rt)
    return plane, geo, rec, off, want_rec, rc, d_rt


def _dev(setup):
    import torch
    plane, geo, rec, off, want_rec, rc, d_rt = setup
    return (torch.from_numpy(rec.view(np.uint8)).cuda(), torch.from_numpy(off).cuda(),
            torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda())


def test_records_cover_every_branch(setup):
    plane, geo, rec, off, want_rec, rc, d_rt = setup
    on = rt_plane(rec["det"])
    assert on.sum() > 50000 and (~on).sum() > 1000   # hodoscope hits pass through
    cw = plane.arr("cellwidth")[rec["det"]]
    half = want_rec["drift"] == (cw * np.float32(0.5))
    zero = want_rec["drift"] == 0.0
    assert (on & half).sum() > 1000 and (on & zero).sum() > 1000 and (on & ~half & ~zero).sum() > 20000


def test_pack_rt_matches_oracle(setup):
    from orgpu import pipeline
    plane, geo, rec, off, want_rec, rc, d_rt = setup
    d_rec, d_off, d_wp = _dev(setup)
    n = len(off) - 1
    b = pipeline.DeviceBatch(n, rc.device, with_tracks=False)
    rc.pack_rt(b, d_rec, d_off, d_wp, d_rt)
    rc.sync()
    want = S.pack(want_rec, off, geo.wire_pos_f32())
    assert hit_mismatches(b.download_hits(), want) == []


def test_rt_apply_matches_pack_rt(setup):
    """Plain packing then the in-place conversion gives the same buffers."""
    from orgpu import pipeline
    plane, geo, rec, off, want_rec, rc, d_rt = setup
    d_rec, d_off, d_wp = _dev(setup)
    n = len(off) - 1
    b = pipeline.DeviceBatch(n, rc.device, with_tracks=False)
    rc.pack(b, d_rec, d_off, d_wp)
    plain = b.download_hits()
    assert hit_mismatches(plain, S.pack(rec, off, geo.wire_pos_f32())) == []
    rc.rt_apply(b, d_rt)
    rc.sync()
    assert hit_mismatches(b.download_hits(), S.pack(want_rec, off, geo.wire_pos_f32())) == []


def test_rt_single_plane_edges(setup):
    """One plane set by hand with 1, 2 and 3 knots: extrapolation outside the
    knots inside a wide window, and the knots themselves."""
    import ctypes as C
    import torch
    from orgpu import _lib, pipeline
    plane, geo, rec, off, want_rec, rc, d_rt = setup
    lb = _lib.lib()
    o = RtOracle(plane.arr("cellwidth"))
    rt = L.OrRtTable()
    planes = {2: ([1700.0], [0.25]), 9: ([1650.0, 1750.0], [0.4, 0.0]), 50: ([1500.0, 1510.5, 1600.0], [1.2, 0.7, 0.1])}
    for det, (T, R) in planes.items():
        T = np.array(T)
        R = np.array(R)
        _lib.check(lb.or_rt_set_plane(C.byref(rt), det, len(T), T.ctypes.data, R.ctypes.data, 1400.0, 1800.0,
                                      float(plane.arr("cellwidth")[det])), "or_rt_set_plane")
        o.set_plane(det, T, R, 1400.0, 1800.0)
    rng = np.random.default_rng(3)
    n_ev = 64
    dets = np.array(list(planes))
    per = 30
    det = np.tile(np.repeat(dets, per), n_ev).astype(np.int16)
    tdc = rng.uniform(1390.0, 1810.0, len(det)).astype(np.float32)
    tdc[::7] = np.float32(1510.5)
    tdc[1::7] = np.float32(1650.0)
    rec = np.zeros(len(det), L.HIT_RECORD_DTYPE)
    rec["det"], rec["elem"], rec["tdc"], rec["flag"] = det, 5, tdc, 2
    rec["drift"] = 0.125
    off = np.arange(n_ev + 1, dtype=np.int64) * (len(dets) * per)
    rec = _sorted(rec, off)
    want_rec = rec.copy()
    want_rec["drift"] = o.drift(rec["det"], rec["tdc"], rec["drift"])
    b = pipeline.DeviceBatch(n_ev, rc.device, with_tracks=False)
    rc.pack_rt(b, torch.from_numpy(rec.view(np.uint8)).cuda(), torch.from_numpy(off).cuda(),
               torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda(), pipeline.rt_to_device(rt))
    rc.sync()
    assert hit_mismatches(b.download_hits(), S.pack(want_rec, off, geo.wire_pos_f32())) == []
