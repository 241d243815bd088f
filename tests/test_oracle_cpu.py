"""CPU tests: geometry parsing (both loaders), oracle primitives with known
answers, event-reducer rules on hand-built planes, and the whole oracle
chain's invariants on seeded events."""
import ctypes as C
import struct

import numpy as np
import pytest

from oracle import pyoracle as O
from orgpu import GEOMETRY_E906, layout as L, synth as S


def f32(x):
    return struct.unpack("f", struct.pack("f", x))[0]


# ---------------------------------------------------------------- geometry --
def test_geometry_glued_columns(geometry):
    """Rows 45, 47, 48 of the table have glued columns; `istream >> float`
    splits them where a float literal ends (online_reconstruction.cu:133)."""
    p, wp = geometry
    assert p.resolution[47] == f32(2.749630657183)
    assert p.p1x_w1[47] == f32(0.4666022)
    assert p.p1y_w1[47] == f32(-178.7537614)
    assert p.p1x_w1[48] == f32(0.468201)
    assert p.resolution[45] == f32(11.34348941)
    assert p.p1x_w1[45] == f32(-145.1692364)
    assert p.nelem[1] == 201 and p.nelem[54] == 72
    assert p.z[31] == f32(666.681)


def test_geometry_derived_windows(geometry):
    """slope_max/inter_max get the pairwise widening on even planes, summed in
    double (online_reconstruction.cu:177-186)."""
    p, _ = geometry
    for ipl in (2, 16, 30, 54):
        c, s = p.costheta[ipl], p.sintheta[ipl]
        base = f32(f32(c * f32(0.15)) + f32(s * f32(0.1)))
        dsl = float(f32(f32(p.resolution[ipl] + p.resolution[ipl - 1]) / f32(p.z[ipl] - p.z[ipl - 1])))
        assert p.slope_max[ipl] == f32(base + dsl)


def test_wire_positions(geometry):
    """Chamber wire j of plane i sits at (j-(n+1)/2)*spacing + offsets
    (online_reconstruction.cu:191-218)."""
    p, wp = geometry
    i, j = 16, 40
    expect = (j - (p.nelem[i] + 1.0) / 2.0) * p.spacing[i] + p.xoffset[i]
    expect += float(f32(p.x0[i] * p.costheta[i])) + float(f32(p.y0[i] * p.sintheta[i]))
    assert abs(wp[i, j] - expect) < 0.2  # the per-plane survey offset is the rest
    assert abs((wp[i, j + 1] - wp[i, j]) - p.spacing[i]) < 1e-9
    assert wp[i, 0] == 0.0 and wp[i, p.nelem[i] + 1] == 0.0


def test_library_geometry_matches_oracle(geometry):
    """The library's C++ loader and the oracle's C loader agree byte for byte."""
    from orgpu import _lib
    p1, wp1 = geometry
    p2, wp2 = _lib.geometry_load(GEOMETRY_E906)
    assert p1.to_bytes() == p2.to_bytes()
    assert np.array_equal(wp1, wp2)


# -------------------------------------------------------------- primitives --
def test_matinv_known_answer():
    a = np.array([2.0, 1.0, 1.0, 3.0], np.float32)  # row-major [[2,1],[1,3]]
    ai = np.zeros(4, np.float32)
    O.lib().orc_matinv_2x2(a.ctypes.data, ai.ctypes.data)
    np.testing.assert_allclose(ai.reshape(2, 2) @ a.reshape(2, 2), np.eye(2), atol=1e-6)


def test_fit_line_known_answer():
    z = np.array([100.0, 200.0, 300.0, 400.0], np.float32)
    x = (3.0 + 0.05 * z).astype(np.float32)
    w = np.full(4, 0.5, np.float32)
    par, err = np.zeros(2, np.float32), np.zeros(2, np.float32)
    O.lib().orc_fit_2d(4, x.ctypes.data, z.ctypes.data, w.ctypes.data, par.ctypes.data, err.ctypes.data)
    assert abs(par[0] - 3.0) < 1e-3 and abs(par[1] - 0.05) < 1e-6
    # weights are the resolutions themselves (trackanalyticalminimizer.cuh:49-58):
    # Ainv scales as 1/w, so errors grow like 1/sqrt(w)
    par2, err2 = np.zeros(2, np.float32), np.zeros(2, np.float32)
    w2 = np.full(4, 2.0, np.float32)
    O.lib().orc_fit_2d(4, x.ctypes.data, z.ctypes.data, w2.ctypes.data, par2.ctypes.data, err2.ctypes.data)
    np.testing.assert_allclose(err2 * 2.0, err, rtol=1e-5)


def test_fit_drift_known_answer():
    z = np.array([100.0, 110.0, 300.0, 310.0], np.float32)
    truth = (1.0 + 0.02 * z).astype(np.float32)
    drift = np.array([0.3, 0.2, 0.1, 0.4], np.float32)
    sign = np.array([1, -1, -1, 1], np.int16)
    wires = (truth - drift * sign).astype(np.float32)
    w = np.ones(4, np.float32)
    par, err = np.zeros(2, np.float32), np.zeros(2, np.float32)
    O.lib().orc_fit_2d_drift(4, wires.ctypes.data, drift.ctypes.data, sign.ctypes.data, z.ctypes.data,
                             w.ctypes.data, par.ctypes.data, err.ctypes.data)
    assert abs(par[0] - 1.0) < 1e-4 and abs(par[1] - 0.02) < 1e-6


# ------------------------------------------------------------ event reducer --
def _plane(rows):
    """rows: (chan, pos, tdc, flag, drift) -> SoA slot image."""
    a = np.array(rows, np.float32).T.copy()
    return a.reshape(-1), a.shape[1]


def _reduce(rows, det):
    slot, n = _plane(rows)
    flags = np.zeros(n, np.int16)
    k = O.lib().orc_reduce_plane(slot.ctypes.data, n, det, flags.ctypes.data)
    return k, (flags > 0).tolist()


def test_er_out_of_time_dropped():
    k, keep = _reduce([(10, 1.0, 1100, 2, 0.1), (40, 5.0, 1100, 1, 0.1)], 31)
    assert keep == [True, False] and k == 1


def test_er_two_hit_cluster_keeps_smaller_drift():
    # neighbours 10,11 with both drifts large: the larger drift is dropped (H:276-283);
    # a hit after the cluster closes it (H:258)
    rows = [(10, 0.0, 1100, 2, 0.40), (11, 0.5, 1101, 2, 0.45), (20, 9.0, 1100, 2, 0.1)]
    k, keep = _reduce(rows, 16)
    assert keep == [True, False, True]


def test_er_dc3p_close_in_time_drops_both():
    # small drifts, |dt| < 8 ns on a DC3p plane (19..24): both dropped (H:290-294)
    rows = [(10, 0.0, 1100, 2, 0.05), (11, 2.0, 1103, 2, 0.04), (30, 9.0, 1100, 2, 0.1)]
    assert _reduce(rows, 20)[1] == [False, False, True]
    assert _reduce(rows, 16)[1] == [True, True, True]  # other planes keep both


def test_er_three_hit_cluster():
    # mean |dt| < 10: the whole cluster goes; otherwise all but the first (H:297-318)
    quiet = [(10, 0, 1100, 2, .1), (11, 1, 1102, 2, .1), (12, 2, 1104, 2, .1), (40, 9, 1100, 2, .1)]
    assert _reduce(quiet, 16)[1] == [False, False, False, True]
    loud = [(10, 0, 1100, 2, .1), (11, 1, 1130, 2, .1), (12, 2, 1160, 2, .1), (40, 9, 1100, 2, .1)]
    assert _reduce(loud, 16)[1] == [True, False, False, True]


def test_er_break_hit_does_not_start_cluster():
    # the hit that closes a cluster is not put in a new one (H:258-319): 10 | 20,21
    # -> 20 closes [10], 21 starts a fresh cluster that is never closed
    rows = [(10, 0, 1100, 2, .1), (20, 5, 1100, 2, .4), (21, 6, 1101, 2, .45), (50, 9, 1100, 1, .1)]
    assert _reduce(rows, 16)[1] == [True, True, True, False]


def test_er_same_channel_first_wins():
    rows = [(7, 1.0, 1100, 2, 0.1), (7, 1.0, 1180, 2, 0.2)]
    k, keep = _reduce(rows, 40)  # hodoscope: no declustering, dedup only
    assert keep == [True, False] and k == 1


# ------------------------------------------------------------ oracle chain --
@pytest.fixture(scope="module")
def chain(geometry):
    plane, wp = geometry
    geo = S.Geometry(plane, wp)
    rec, off, truth = S.generate(geo, S.config_small(150, 906001))
    rec, off = S.cap_records(rec, off)
    hits = S.pack(rec, off, geo.wire_pos_f32())
    t = L.HostTracks(hits.n)
    st = O.OracleState(hits.n)
    O.run_all(plane, hits.copy(), t, st, n_threads=4)
    return plane, rec, off, hits, t, st, truth


def test_chain_finds_tracks(chain):
    plane, rec, off, hits, t, st, truth = chain
    n6 = sum(int(r[L.TRK_STID] == 6) for e in range(t.n) for _, _, r in t.records(e))
    assert n6 > 0.4 * len(truth["event"])


def test_chain_threads_do_not_change_results(chain):
    plane, rec, off, hits, t, st, truth = chain
    t1 = L.HostTracks(hits.n)
    st1 = O.OracleState(hits.n)
    O.run_all(plane, hits.copy(), t1, st1, n_threads=1)
    assert np.array_equal(t1.tracks.view(np.uint32), t.tracks.view(np.uint32))
    assert np.array_equal(st1.toomany, st.toomany)


def test_chain_global_tracks_are_consistent(chain):
    """Global tracks: charge +-1, 1/p inside [0.01, 0.2], hits on station 1."""
    plane, rec, off, hits, t, st, truth = chain
    for e in range(t.n):
        for _, _, r in t.records(e):
            if r[L.TRK_STID] != 6:
                continue
            assert r[L.TRK_CHARGE] in (1.0, -1.0)
            assert 0.01 <= r[L.TRK_INVP] <= 0.2
            n = int(r[L.TRK_NHITS])
            dets = r[L.TRK_HIT_DETID:L.TRK_HIT_DETID + n]
            assert (dets <= 6).sum() >= 3


def test_packer_roundtrip(chain):
    """Packed planes hold the records of each (event, plane) in order."""
    plane, rec, off, hits, t, st, truth = chain
    e = 3
    r = rec[off[e]:off[e + 1]]
    for d in (16, 33, 50):
        n, arr = hits.plane(e, d)
        sel = r[r["det"] == d]
        assert n == len(sel)
        np.testing.assert_array_equal(arr[0], sel["elem"].astype(np.float32))
        np.testing.assert_array_equal(arr[2], sel["tdc"])
