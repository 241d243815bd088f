"""ctypes binding of the CPU oracle (or_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The library path never imports
this module.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "e1039-gpu_gb300"))
from orgpu import layout as L  # noqa: E402

LIB_PATH = os.path.join(HERE, "liborc.so")
LIB64_PATH = os.path.join(HERE, "liborc64.so")  # the same code with FP64 fits, residuals and chi2 sums
SOURCES = [os.path.join(HERE, "or_oracle.c"), os.path.join(HERE, "or_physics.c")]

ST_TOOMANY_ER, ST_TOOMANY_XZBIN, ST_TOOMANY_TKL = 1, 2, 4
NCOUNTS = 8


def _build_one(path, extra, force):
    if not force and os.path.exists(path) and all(
            os.path.getmtime(path) >= os.path.getmtime(s) for s in SOURCES + [
                os.path.join(HERE, "or_oracle.h"), os.path.join(REPO, "include", "or_layout.h")]):
        return path
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread"] + extra + ["-o", path + ".tmp"] + SOURCES + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(path + ".tmp", path)
    return path


def build(force=False):
    """Compile the oracle with one rounding per float operation, and its FP64
    instance (fits, residuals and chi2 sums in double)."""
    _build_one(LIB64_PATH, ["-DORC_FIT_T=double"], force)
    return _build_one(LIB_PATH, [], force)


_lib = None
_lib64 = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = _load(LIB_PATH)
    return _lib


def lib64():
    """The FP64 instance (same entry points)."""
    global _lib64
    if _lib64 is None:
        build()
        _lib64 = _load(LIB64_PATH)
    return _lib64


def _load(path):
    _lib = C.CDLL(path)
    if True:
        P = C.POINTER
        _lib.orc_parse_geometry.argtypes = [C.c_char_p, P(L.OrPlane), C.c_void_p]
        _lib.orc_event_reduce.argtypes = [L.OrHitsView, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        _lib.orc_xz.argtypes = [P(L.OrPlane), L.OrHitsView, L.OrTracksView, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_int, C.c_int]
        _lib.orc_yz.argtypes = [P(L.OrPlane), L.OrHitsView, L.OrTracksView, C.c_void_p, C.c_int, C.c_int]
        _lib.orc_back_clean.argtypes = [L.OrTracksView, C.c_void_p, C.c_int, C.c_int]
        _lib.orc_global.argtypes = [P(L.OrPlane), L.OrHitsView, L.OrTracksView, C.c_void_p, C.c_int, C.c_int]
        _lib.orc_run_all.argtypes = [P(L.OrPlane), L.OrHitsView, L.OrTracksView, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_int, C.c_int]
        _lib.orc_run_all_counted.argtypes = [P(L.OrPlane), L.OrHitsView, L.OrTracksView, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        _lib.orc_fit_2d.argtypes = [C.c_int] + [C.c_void_p] * 5
        _lib.orc_fit_2d_drift.argtypes = [C.c_int] + [C.c_void_p] * 7
        _lib.orc_matinv_2x2.argtypes = [C.c_void_p, C.c_void_p]
        _lib.orc_reduce_plane.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        _lib.orc_reduce_plane.restype = C.c_int
        _lib.orc_hardware_threads.restype = C.c_int
        _lib.orc_prop_matching.argtypes = [P(L.OrPlane), L.OrHitsView, L.OrTracksView, C.c_void_p, C.c_int, C.c_int]
        _lib.orc_global_clean.argtypes = [L.OrTracksView, C.c_void_p, C.c_int, C.c_int]
        _lib.orc_tracklet_features.argtypes = [P(L.OrPlane), L.OrHitsView, L.OrTracksView, C.c_void_p, C.c_int,
                                               C.c_void_p, C.c_void_p, C.c_int64]
        _lib.orc_tracklet_features.restype = C.c_int64
        _lib.orc_yz_outer_dump.argtypes = [P(L.OrPlane), L.OrHitsView, L.OrTracksView, C.c_void_p, C.c_int,
                                            C.c_void_p, C.c_int64]
        _lib.orc_yz_outer_dump.restype = C.c_int64
        _lib.orc_vertexing.argtypes = [P(L.OrPlane), L.OrTracksView, C.c_void_p, C.c_int, C.c_int]
        _lib.orc_dimuons.argtypes = [P(L.OrPlane), L.OrTracksView, L.OrDimuonsView, C.c_void_p, C.c_int, C.c_int]
        _lib.orc_hist_table.argtypes = [P(L.OrHists)]
        _lib.orc_fill_histograms.argtypes = [L.OrTracksView, L.OrDimuonsView, P(L.OrHists), C.c_void_p, C.c_void_p,
                                             C.c_int]
    return _lib


def parse_geometry(path):
    p = L.OrPlane()
    wp = np.zeros(L.NDET * L.WIREPOS_STRIDE, np.float64)
    rc = lib().orc_parse_geometry(path.encode(), C.byref(p), wp.ctypes.data)
    if rc != 0:
        raise OSError(f"oracle could not read geometry {path}")
    return p, wp.reshape(L.NDET, L.WIREPOS_STRIDE)


class OracleState:
    """Per-event outputs of an oracle run, on top of HostHits/HostTracks."""

    def __init__(self, n):
        self.toomany = np.zeros(n, np.uint8)
        self.status = np.zeros(n, np.uint32)
        self.ntracklets = np.zeros(n, np.int32)
        self.counts = np.zeros(NCOUNTS * n, np.int64)


def event_reduce(hits, state, n_threads=0):
    lib().orc_event_reduce(hits.view(), state.toomany.ctypes.data, state.status.ctypes.data, hits.n, n_threads)


def xz(plane, hits, tracks, state, n_threads=0):
    lib().orc_xz(C.byref(plane), hits.view(), tracks.view(), state.ntracklets.ctypes.data,
                 state.toomany.ctypes.data, state.status.ctypes.data, hits.n, n_threads)


def yz(plane, hits, tracks, state, n_threads=0):
    lib().orc_yz(C.byref(plane), hits.view(), tracks.view(), state.toomany.ctypes.data, hits.n, n_threads)


def back_clean(tracks, state, n_threads=0):
    lib().orc_back_clean(tracks.view(), state.toomany.ctypes.data, tracks.n, n_threads)


def global_tracking(plane, hits, tracks, state, n_threads=0):
    lib().orc_global(C.byref(plane), hits.view(), tracks.view(), state.toomany.ctypes.data, hits.n, n_threads)


def prop_matching(plane, hits, tracks, state, n_threads=0):
    lib().orc_prop_matching(C.byref(plane), hits.view(), tracks.view(), state.toomany.ctypes.data, hits.n, n_threads)


def global_clean(tracks, state, n_threads=0):
    lib().orc_global_clean(tracks.view(), state.toomany.ctypes.data, tracks.n, n_threads)


def run_all(plane, hits, tracks, state, n_threads=0, counted=False, fp64=False):
    lb = lib64() if fp64 else lib()
    if counted:
        lb.orc_run_all_counted(C.byref(plane), hits.view(), tracks.view(), state.ntracklets.ctypes.data,
                                  state.toomany.ctypes.data, state.status.ctypes.data, state.counts.ctypes.data,
                                  hits.n, n_threads)
    else:
        lb.orc_run_all(C.byref(plane), hits.view(), tracks.view(), state.ntracklets.ctypes.data,
                       state.toomany.ctypes.data, state.status.ctypes.data, hits.n, n_threads)


def tracklet_features(plane, hits, tracks, toomany, max_rows=None):
    """(row_off [n+1], features [rows, 16]) of the tracklets in `tracks`
    (the state after XZ)."""
    n = hits.n
    cap = int(max_rows if max_rows is not None else n * L.TRKMAX)
    row_off = np.zeros(n + 1, np.int32)
    feat = np.zeros((max(cap, 1), L.NFEAT), np.float32)
    rows = lib().orc_tracklet_features(C.byref(plane), hits.view(), tracks.view(),
                                       np.ascontiguousarray(toomany, np.uint8).ctypes.data, n, row_off.ctypes.data,
                                       feat.ctypes.data, cap)
    return row_off, feat[:min(rows, cap)]


def vertexing(plane, tracks, state, n_threads=0):
    lib().orc_vertexing(C.byref(plane), tracks.view(), state.toomany.ctypes.data, tracks.n, n_threads)


def dimuons(plane, tracks, dims, state, n_threads=0):
    lib().orc_dimuons(C.byref(plane), tracks.view(), dims.view(), state.toomany.ctypes.data, tracks.n, n_threads)


def hist_table():
    h = L.OrHists()
    lib().orc_hist_table(C.byref(h))
    return h


def fill_histograms(tracks, dims, hists, trigger_bits, state):
    tb = None if trigger_bits is None else np.ascontiguousarray(trigger_bits, np.int32)
    lib().orc_fill_histograms(tracks.view(), dims.view(), C.byref(hists), None if tb is None else tb.ctypes.data,
                              state.toomany.ctypes.data, tracks.n)


def yz_outer_dump(plane, hits, tracks, state, cap=20_000_000):
    """YZ on `tracks` (single thread) with one record per live (u3, v3) outer
    iteration: float32 [n, 24] (see orc_yz_outer_dump)."""
    buf = np.zeros(cap * 24, np.float32)
    n = lib().orc_yz_outer_dump(C.byref(plane), hits.view(), tracks.view(), state.toomany.ctypes.data, hits.n,
                                buf.ctypes.data, cap)
    return buf[:n * 24].reshape(n, 24)


def hardware_threads():
    return int(lib().orc_hardware_threads())
