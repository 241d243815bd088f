"""R-T calibration on the CPU: the oracle against an independent clamped
spline (scipy) and against the calibration points, and the library's host
loader (or_rt_load / or_rt_set_plane, no GPU) against the oracle bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

from oracle.rt_oracle import RtOracle, clamped_spline, parse_calibration, spline_eval
from orgpu import CALIBRATION_E906, _lib, layout as L


@pytest.fixture(scope="module")
def calib():
    return parse_calibration(CALIBRATION_E906)


def test_calibration_file_planes(calib):
    # every drift-chamber plane and every prop-tube plane has a profile
    assert sorted(calib) == list(range(1, 31)) + list(range(47, 55))
    for det, (tmin, tmax, T, R) in calib.items():
        assert np.all(np.diff(T) > 0)
        assert tmin <= T[0] and T[-1] <= tmax + 1e-3


def test_oracle_against_scipy_clamped(calib):
    """Same interpolant as scipy's clamped CubicSpline (a separate banded
    solver), to 1e-12 cm, on a dense grid of every plane."""
    interp = pytest.importorskip("scipy.interpolate")
    worst = 0.0
    for det, (tmin, tmax, T, R) in calib.items():
        b, c, d = clamped_spline(T, R)
        x = np.linspace(T[0], T[-1], 4001)
        ours = spline_eval(T, R, b, c, d, x)
        ref = interp.CubicSpline(T, R, bc_type="clamped")(x)
        worst = max(worst, float(np.max(np.abs(ours - ref))))
    assert worst < 1e-12, worst


def test_oracle_spline_properties(calib):
    """Interpolates the points, zero slope at both ends, C1 and C2 at the
    interior knots."""
    for det, (tmin, tmax, T, R) in calib.items():
        b, c, d = clamped_spline(T, R)
        n = len(T)
        at = spline_eval(T, R, b, c, d, T)
        assert np.max(np.abs(at - R)) < 1e-12
        # float drift at a knot equals the calibration value rounded to float
        # (where R is not ~0: there a 1e-19 residue stays visible in float)
        big = np.abs(R) >= 1e-4
        assert np.array_equal(at[big].astype(np.float32), R[big].astype(np.float32))
        h = np.diff(T)
        k = np.arange(n - 1)
        slope_end = b[k] + 2 * c[k] * h + 3 * d[k] * h * h   # derivative at the right end of piece k
        curv_end = 2 * c[k] + 6 * d[k] * h
        assert b[0] == 0.0 and abs(slope_end[-1]) < 1e-12
        assert np.max(np.abs(slope_end[:-1] - b[1:n - 1])) < 1e-12
        assert np.max(np.abs(curv_end[:-1] - 2 * c[1:n - 1])) < 1e-9


def test_oracle_reproduces_clamped_cubic():
    """A cubic with zero slope at both ends is its own clamped spline."""
    T = np.array([0.0, 0.7, 1.5, 2.0, 3.1, 4.0])
    f = lambda x: 2.0 * x ** 3 - 3.0 * 4.0 * x ** 2 + 5.0  # f'(0) = f'(4) = 0
    b, c, d = clamped_spline(T, f(T))
    x = np.linspace(0.0, 4.0, 101)
    assert np.max(np.abs(spline_eval(T, f(T), b, c, d, x) - f(x))) < 1e-12


def test_oracle_window_rule():
    o = RtOracle(np.full(L.NDET, 2.0, np.float32))
    o.set_plane(5, [10.0, 12.0, 14.0], [0.9, 0.5, 0.1], 10.0, 14.0)
    det = np.array([5, 5, 5, 5, 5, 33, 7])
    tdc = np.array([9.5, 10.0, 14.0, 14.5, 12.0, 9.0, 9.0], np.float32)
    drift = np.full(7, 0.25, np.float32)
    out = o.drift(det, tdc, drift)
    # below the window: half a cell; above: 0; at the edges: the spline
    assert out[0] == np.float32(1.0) and out[3] == 0.0
    assert out[1] == np.float32(0.9) and out[2] == np.float32(0.1) and out[4] == np.float32(0.5)
    # hodoscope and planes without a profile keep the record's value
    assert out[5] == np.float32(0.25) and out[6] == np.float32(0.25)


def _table_fields(rt, det, n):
    return {f: np.ctypeslib.as_array(getattr(rt, f))[det][:n].copy() for f in ("t", "r", "b", "c", "d")}


def test_library_loader_matches_oracle(geometry, calib):
    plane, _ = geometry
    rt, nplanes = _lib.rt_load(CALIBRATION_E906, plane)
    assert nplanes == 38
    o = RtOracle.from_file(CALIBRATION_E906, plane.arr("cellwidth"))
    nk = rt.arr("nknots")
    for det in range(L.NDET):
        if det not in o.planes:
            assert nk[det] == 0
            continue
        tmin, tmax, T, R, B, Cc, D = o.planes[det]
        n = len(T)
        assert nk[det] == n
        assert rt.tmin[det] == tmin and rt.tmax[det] == tmax
        assert np.float32(rt.cellwidth[det]) == plane.arr("cellwidth")[det]
        got = _table_fields(rt, det, n)
        for f, want in (("t", T), ("r", R), ("b", B), ("c", Cc), ("d", D)):
            assert np.array_equal(got[f].view(np.uint64), np.asarray(want).view(np.uint64)), (det, f)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 7, 500])
def test_library_set_plane_matches_oracle(n):
    rng = np.random.default_rng(n)
    T = np.cumsum(rng.uniform(0.5, 3.0, n)) + 1000.0
    R = rng.uniform(0.0, 1.0, n)
    rt = L.OrRtTable()
    lb = _lib.lib()
    _lib.check(lb.or_rt_set_plane(C.byref(rt), 48, n, T.ctypes.data, R.ctypes.data, float(T[0]), float(T[-1]), 2.54),
               "or_rt_set_plane")
    b, c, d = clamped_spline(T, R)
    got = _table_fields(rt, 48, n)
    for f, want in (("b", b), ("c", c), ("d", d)):
        assert np.array_equal(got[f].view(np.uint64), want.view(np.uint64)), f


def test_library_set_plane_rejects_bad_input():
    lb = _lib.lib()
    rt = L.OrRtTable()
    T = np.array([1.0, 2.0, 2.0, 3.0])
    R = np.zeros(4)
    args = (T.ctypes.data, R.ctypes.data, 0.0, 10.0, 1.0)
    assert lb.or_rt_set_plane(C.byref(rt), 3, 4, *args) == _lib.OR_ERR_ARG        # repeated knot
    T2 = np.arange(4.0)
    ok = (T2.ctypes.data, R.ctypes.data, 0.0, 10.0, 1.0)
    assert lb.or_rt_set_plane(C.byref(rt), 35, 4, *ok) == _lib.OR_ERR_ARG         # hodoscope plane
    assert lb.or_rt_set_plane(C.byref(rt), 3, 0, *ok) == _lib.OR_ERR_ARG          # no points
    assert lb.or_rt_set_plane(C.byref(rt), 3, L.RT_MAXKNOTS + 1, *ok) == _lib.OR_ERR_ARG
    assert lb.or_rt_set_plane(C.byref(rt), 3, 4, *ok) == _lib.OR_OK
    assert lb.or_rt_table_bytes() == C.sizeof(L.OrRtTable)


def test_library_loader_errors(tmp_path, geometry):
    plane, _ = geometry
    lb = _lib.lib()
    rt = L.OrRtTable()
    assert lb.or_rt_load(str(tmp_path / "missing.txt").encode(), C.byref(plane), C.byref(rt), None) == _lib.OR_ERR_IO
    bad = tmp_path / "bad.txt"
    bad.write_text("3 4 1650.0 1750.0 D1U\n0 1650.0 0.3\n1 1660.0 0.2\n")  # truncated
    assert lb.or_rt_load(str(bad).encode(), C.byref(plane), C.byref(rt), None) == _lib.OR_ERR_IO
    ok = tmp_path / "ok.txt"
    ok.write_text("3 3 1650.0 1750.0 D1U\n0 1650.0 0.3\n1 1700.0 0.2\n2 1750.0 0.0\n\n"
                  "40 2 0.0 1.0 H4Y\n0 0.0 0.0\n1 1.0 1.0\n")  # hodoscope entry: read, not applied
    n = C.c_int(-1)
    assert lb.or_rt_load(str(ok).encode(), C.byref(plane), C.byref(rt), C.byref(n)) == _lib.OR_OK
    assert n.value == 1 and rt.nknots[3] == 3 and rt.nknots[40] == 0
