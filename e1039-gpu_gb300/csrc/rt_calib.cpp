// rt_calib.cpp -- R-T calibration loader for the C-ABI.
//
// The reference host reads a plain-text calibration file and builds, per
// drift-chamber and prop-tube plane, a ROOT TSpline3 through the (T, R)
// points with option "b1e1" (first derivative prescribed at both ends, both
// zero): OnlineReconstruction/online_reconstruction.cu:220-242.  It then
// evaluates the spline once per hit while packing (:387-396).  This file does
// the one-off part on the host, as the reference does: parse the file and
// turn every plane's points into the coefficients of its clamped cubic
// spline.  Evaluation runs on the device (pack_kernel.cu).
//
// File format (online_reconstruction.cu:229-239): a header line
//     detectorID nBin tmin tmax name
// followed by nBin lines
//     iBin T R
// tmin and tmax are kept as float, the type of the reference's arrays
// (:121, :232-233).
//
// The spline is the complete (clamped) cubic spline interpolant, the
// published construction of de Boor, A Practical Guide to Splines (1978),
// ch. IV: slopes s_k at the knots from the tridiagonal system
//     h_k s_{k-1} + 2 (h_{k-1} + h_k) s_k + h_{k-1} s_{k+1}
//         = 3 (h_k D_{k-1} + h_{k-1} D_k),        k = 1 .. n-2,
// with h_k = t_{k+1} - t_k, D_k = (r_{k+1} - r_k) / h_k and s_0 = s_{n-1} = 0,
// solved by forward elimination and back substitution; then on every piece
// the Hermite cubic of the end values and slopes,
//     b_k = s_k,  c_k = (3 D_k - 2 s_k - s_{k+1}) / h_k,
//     d_k = (s_k + s_{k+1} - 2 D_k) / h_k^2.
// All in double; compiled without floating-point contraction so each
// operation rounds once.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/or_gb300.h"

static bool rt_plane_ok(int det) {
    return (det >= 1 && det <= OR_NCHAM) || (det > OR_NCHAM + OR_NHODO && det < OR_NDET);
}

extern "C" int or_rt_set_plane(or_rt_table_t *rt, int det, int n, const double *t, const double *r, float tmin,
                               float tmax, float cellwidth) {
    if (!rt || !rt_plane_ok(det) || n < 1 || n > OR_RT_MAXKNOTS || !t || !r) return OR_ERR_ARG;
    for (int k = 1; k < n; ++k)
        if (!(t[k] > t[k - 1])) return OR_ERR_ARG;  // knots strictly increasing
    double *T = rt->t[det], *R = rt->r[det], *B = rt->b[det], *C = rt->c[det], *D = rt->d[det];
    for (int k = 0; k < OR_RT_MAXKNOTS; ++k) T[k] = R[k] = B[k] = C[k] = D[k] = 0.0;
    for (int k = 0; k < n; ++k) {
        T[k] = t[k];
        R[k] = r[k];
    }
    if (n >= 2) {
        std::vector<double> h(n - 1), dd(n - 1), diag(n), rhs(n), s(n, 0.0);
        for (int k = 0; k + 1 < n; ++k) {
            h[k] = t[k + 1] - t[k];
            dd[k] = (r[k + 1] - r[k]) / h[k];
        }
        // interior equations k = 1..n-2; the end slopes are zero, so the
        // first and last equations lose their boundary terms
        for (int k = 1; k + 1 < n; ++k) {
            diag[k] = 2.0 * (h[k - 1] + h[k]);
            rhs[k] = 3.0 * (h[k] * dd[k - 1] + h[k - 1] * dd[k]);
        }
        for (int k = 2; k + 1 < n; ++k) {
            const double w = h[k] / diag[k - 1];  // sub-diagonal of row k over the previous pivot
            diag[k] = diag[k] - w * h[k - 2];     // super-diagonal of row k-1 is h_{k-2}
            rhs[k] = rhs[k] - w * rhs[k - 1];
        }
        for (int k = n - 2; k >= 1; --k) s[k] = (rhs[k] - h[k - 1] * s[k + 1]) / diag[k];
        for (int k = 0; k + 1 < n; ++k) {
            B[k] = s[k];
            C[k] = (3.0 * dd[k] - 2.0 * s[k] - s[k + 1]) / h[k];
            D[k] = (s[k] + s[k + 1] - 2.0 * dd[k]) / (h[k] * h[k]);
        }
    }
    rt->nknots[det] = n;
    rt->tmin[det] = tmin;
    rt->tmax[det] = tmax;
    rt->cellwidth[det] = cellwidth;
    return OR_OK;
}

extern "C" size_t or_rt_table_bytes(void) { return sizeof(or_rt_table_t); }

extern "C" int or_rt_load(const char *path, const or_plane_t *plane, or_rt_table_t *rt, int *nplanes_out) {
    if (!path || !plane || !rt) return OR_ERR_ARG;
    if (nplanes_out) *nplanes_out = 0;
    std::ifstream in(path);
    if (!in) return OR_ERR_IO;
    std::memset(rt, 0, sizeof(*rt));
    std::string line;
    std::vector<double> t, r;
    int nplanes = 0;
    while (std::getline(in, line)) {
        std::istringstream hd(line);
        int det = 0, nbin = 0;
        double tmin = 0.0, tmax = 0.0;
        if (!(hd >> det >> nbin >> tmin >> tmax)) {
            // blank or trailing line; anything else is malformed
            if (line.find_first_not_of(" \t\r") == std::string::npos) continue;
            return OR_ERR_IO;
        }
        if (det < 1 || det >= OR_NDET || nbin < 0 || nbin > OR_RT_MAXKNOTS) return OR_ERR_IO;
        t.assign(nbin, 0.0);
        r.assign(nbin, 0.0);
        for (int i = 0; i < nbin; ++i) {
            if (!std::getline(in, line)) return OR_ERR_IO;
            std::istringstream pt(line);
            int ibin = 0;
            if (!(pt >> ibin >> t[i] >> r[i])) return OR_ERR_IO;
        }
        // the reference builds a spline only for nBin > 0 (:240) and applies
        // it to chambers and prop tubes only (:389)
        if (nbin > 0 && rt_plane_ok(det)) {
            const int rc = or_rt_set_plane(rt, det, nbin, t.data(), r.data(), (float)tmin, (float)tmax,
                                           plane->cellwidth[det]);
            if (rc != OR_OK) return rc;
            ++nplanes;
        }
    }
    if (nplanes_out) *nplanes_out = nplanes;
    return OR_OK;
}
