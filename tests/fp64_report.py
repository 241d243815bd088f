"""FP32 fit error against the FP64 oracle.

The oracle built with -DORC_FIT_T=double computes every fit (2x2 solve),
residual and chi2 sum in double; inputs and stored results stay float.  Both
instances run the whole chain on the same seeded events; for the global
tracks (stationID 6) whose discrete content (hits, signs, charge) is the same
in both, the relative difference of x0, tx, y0, ty, chi2 and 1/p is the FP32
error of the plain path (which is bit-exact with the float oracle).

    python tests/fp64_report.py [n_events]
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (REPO, os.path.join(REPO, "e1039-gpu_gb300"), os.path.join(HERE, "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

import golden_io as G  # noqa: E402
from oracle import pyoracle as O  # noqa: E402
from orgpu import GEOMETRY_E906, layout as L, synth as S  # noqa: E402

FIELDS = {"x0": L.TRK_X0, "tx": L.TRK_TX, "y0": L.TRK_Y0, "ty": L.TRK_TY, "chi2": L.TRK_CHI2, "invP": L.TRK_INVP}


def fp64_errors(cfg):
    plane, wp = O.parse_geometry(GEOMETRY_E906)
    geo = S.Geometry(plane, wp)
    rec, off, _ = S.generate(geo, cfg)
    rec, off = S.cap_records(rec, off)
    h = S.pack(rec, off, geo.wire_pos_f32())
    out = {}
    for fp64 in (False, True):
        hh, t, st = h.copy(), L.HostTracks(h.n), O.OracleState(h.n)
        O.run_all(plane, hh, t, st, fp64=fp64)
        out[fp64] = (G.compact_tracks(t, st.toomany), st.toomany.copy())
    (n32, w32, r32), f32 = out[False]
    (n64, w64, r64), f64 = out[True]
    assert np.array_equal(f32, f64)
    same_events = np.nonzero((n32 == n64).all(axis=1))[0]
    k32 = np.isin(w32[:, 0], same_events)
    k64 = np.isin(w64[:, 0], same_events)
    w32, r32, w64, r64 = w32[k32], r32[k32], w64[k64], r64[k64]
    assert np.array_equal(w32, w64)
    glob = (r32[:, L.TRK_STID] == 6) & (r64[:, L.TRK_STID] == 6)
    disc = (r32[:, G.DISCRETE_FIELDS] == r64[:, G.DISCRETE_FIELDS]).all(axis=1)
    sel = glob & disc
    res = {"global_tracks_fp32": int((r32[:, L.TRK_STID] == 6).sum()),
           "global_tracks_fp64": int((r64[:, L.TRK_STID] == 6).sum()),
           "compared": int(sel.sum()), "discrete_differ": int((glob & ~disc).sum())}
    for name, f in FIELDS.items():
        a = r32[sel, f].astype(np.float64)
        b = r64[sel, f].astype(np.float64)
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-30)
        rel[(a == 0) & (b == 0)] = 0.0
        res[name] = {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)), "max": float(rel.max()),
                     "abs_p99": float(np.quantile(np.abs(a - b), 0.99))}
    return res


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 2000
    rep = {"small": fp64_errors(S.config_small(n, 906011)), "uneven": fp64_errors(S.config_uneven(n, 906012))}
    print(json.dumps(rep, indent=1))


if __name__ == "__main__":
    main()
