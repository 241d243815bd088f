"""CPU oracle for the R-T (drift time -> drift distance) conversion.

TEST INFRASTRUCTURE ONLY: used by the tests as the checker of the library's
R-T calibration loader and of its device packer's drift field.  The library
never imports it.

What it restates (OnlineReconstruction/online_reconstruction.cu):
  - :220-242  the calibration file: header "detectorID nBin tmin tmax name",
    then nBin lines "iBin T R"; tmin/tmax stored as float (:121, :232-233);
    a spline per plane with nBin > 0, ROOT TSpline3(name, T, R, nBin, "b1e1");
  - :387-396  per hit of a chamber or prop-tube plane (detid < 31 or > 46):
    tdc < tmin -> cellwidth*0.5; tdc > tmax -> 0; else the spline at tdc,
    stored in a float.

The spline itself lives in ROOT (TSpline3, the ROOT 6 series the reference
links through root-config; no version is pinned and ROOT is neither vendored
with the reference nor installed here).  "b1e1" with the default end values
is the complete cubic spline interpolant with zero first derivative at both
ends, the construction of de Boor, A Practical Guide to Splines (1978),
ch. IV, which is restated here independently of the library's C++ builder:
numpy float64 operations, one rounding each, the same equations and order.
The bit pattern of ROOT's coefficients is not reproduced from ROOT itself, so
parity against ROOT is pinned by value (the interpolant is unique), not by
bits: the tests check this oracle against scipy's clamped CubicSpline and
the calibration points, and the library against this oracle bit for bit.

Piece convention: piece k covers (t[k], t[k+1]]; x <= t[0] uses piece 0 and
x >= t[-1] uses the last piece, R = r[k] + dx*(b[k] + dx*(c[k] + dx*d[k])).
"""
import numpy as np

NCHAM, NHODO, NDET = 30, 16, 55


def rt_plane(det):
    """Planes the conversion applies to (online_reconstruction.cu:389)."""
    det = np.asarray(det)
    return ((det >= 1) & (det <= NCHAM)) | ((det > NCHAM + NHODO) & (det < NDET))


def parse_calibration(path):
    """-> {det: (tmin f32, tmax f32, T float64[n], R float64[n])} for nBin > 0."""
    out = {}
    with open(path) as f:
        lines = f.read().split("\n")
    i = 0
    while i < len(lines):
        tok = lines[i].split()
        i += 1
        if not tok:
            continue
        det, nbin = int(tok[0]), int(tok[1])
        tmin, tmax = np.float32(float(tok[2])), np.float32(float(tok[3]))
        T = np.empty(nbin)
        R = np.empty(nbin)
        for k in range(nbin):
            p = lines[i].split()
            i += 1
            T[k], R[k] = float(p[1]), float(p[2])
        if nbin > 0:
            out[det] = (tmin, tmax, T, R)
    return out


def clamped_spline(t, r):
    """Coefficients (b, c, d) of the clamped cubic spline through (t, r), zero
    end slopes: slopes from the tridiagonal system by forward elimination and
    back substitution, then the Hermite cubic of each piece."""
    t = np.asarray(t, np.float64)
    r = np.asarray(r, np.float64)
    n = len(t)
    b = np.zeros(n)
    c = np.zeros(n)
    d = np.zeros(n)
    if n < 2:
        return b, c, d
    h = [float(t[k + 1] - t[k]) for k in range(n - 1)]
    dd = [float((r[k + 1] - r[k]) / h[k]) for k in range(n - 1)]
    diag = [0.0] * n
    rhs = [0.0] * n
    s = [0.0] * n
    for k in range(1, n - 1):
        diag[k] = 2.0 * (h[k - 1] + h[k])
        rhs[k] = 3.0 * (h[k] * dd[k - 1] + h[k - 1] * dd[k])
    for k in range(2, n - 1):
        w = h[k] / diag[k - 1]
        diag[k] = diag[k] - w * h[k - 2]
        rhs[k] = rhs[k] - w * rhs[k - 1]
    for k in range(n - 2, 0, -1):
        s[k] = (rhs[k] - h[k - 1] * s[k + 1]) / diag[k]
    for k in range(n - 1):
        b[k] = s[k]
        c[k] = (3.0 * dd[k] - 2.0 * s[k] - s[k + 1]) / h[k]
        d[k] = (s[k] + s[k + 1] - 2.0 * dd[k]) / (h[k] * h[k])
    return b, c, d


def spline_eval(t, r, b, c, d, x):
    """The spline at x (float64 array), with the piece convention above."""
    t = np.asarray(t, np.float64)
    x = np.asarray(x, np.float64)
    n = len(t)
    if n == 1:
        k = np.zeros(x.shape, np.int64)
    else:
        k = np.clip(np.searchsorted(t, x, side="left") - 1, 0, n - 2)
    dx = x - t[k]
    return r[k] + dx * (b[k] + dx * (c[k] + dx * d[k]))


class RtOracle:
    """The calibration of one file (or of planes set one by one)."""

    def __init__(self, cellwidth):
        self.cellwidth = np.asarray(cellwidth, np.float32)
        self.planes = {}

    @classmethod
    def from_file(cls, path, cellwidth):
        o = cls(cellwidth)
        for det, (tmin, tmax, T, R) in parse_calibration(path).items():
            if rt_plane(det):
                o.set_plane(det, T, R, tmin, tmax)
        return o

    def set_plane(self, det, T, R, tmin, tmax):
        T = np.asarray(T, np.float64)
        R = np.asarray(R, np.float64)
        self.planes[int(det)] = (np.float32(tmin), np.float32(tmax), T, R) + clamped_spline(T, R)

    def drift(self, det, tdc, drift):
        """Drift distances (float32) of hits (det, tdc float32, record drift)."""
        det = np.asarray(det, np.int64)
        tdc = np.asarray(tdc, np.float32)
        out = np.array(drift, np.float32, copy=True)
        for p, (tmin, tmax, T, R, B, C, D) in self.planes.items():
            sel = det == p
            if not sel.any():
                continue
            x = tdc[sel]
            v = spline_eval(T, R, B, C, D, x.astype(np.float64)).astype(np.float32)
            v = np.where(x > tmax, np.float32(0.0), v)
            v = np.where(x < tmin, np.float32(self.cellwidth[p] * np.float32(0.5)), v)
            out[sel] = v
        return out
