"""Python mirror of include/or_layout.h: constants, the geometry struct and the
buffer views, as ctypes types shared by the CUDA library binding and the
tests.

The layout is the reference's (OnlineReconstruction/reconstruction_classes.cuh
:4-104, :542-655, :947-977 and reconstruction_constants.h:166-185).
"""
import ctypes as C

import numpy as np

NCHAM, NHODO, NPROP, NDET = 30, 16, 8, 55
NHITSPARAM = 5
MAXHITS_CHAM, MAXHITS_HODO, MAXHITS_PROP = 200, 60, 120
EVT_CHAM_FLOATS = NCHAM * NHITSPARAM * MAXHITS_CHAM
EVT_HODO_FLOATS = NHODO * NHITSPARAM * MAXHITS_HODO
EVT_PROP_FLOATS = NPROP * NHITSPARAM * MAXHITS_PROP
NTRKPARAM, TRKMAX, NSLOTS = 148, 512, 32
MAXHITS_PER_TRACK = 18
SLOTCAP = TRKMAX // NSLOTS
EVT_TRK_FLOATS = TRKMAX * NTRKPARAM
WIREPOS_STRIDE = 400
REF_EVTMAX = 10000
COLLECT_STRIDE = NTRKPARAM + 2

# track record field offsets (reconstruction_classes.cuh:558-635)
TRK_STID, TRK_THREAD, TRK_NHITS, TRK_CHI2 = 0, 1, 2, 3
TRK_TX, TRK_TY, TRK_X0, TRK_Y0, TRK_INVP = 5, 6, 7, 8, 9
TRK_ERR_TX, TRK_ERR_TY, TRK_ERR_X0, TRK_ERR_Y0, TRK_ERR_INVP, TRK_CHARGE = 10, 11, 12, 13, 14, 15
TRK_HIT_DETID, TRK_HIT_CHAN, TRK_HIT_POS, TRK_HIT_DRIFT = 22, 40, 58, 76
TRK_HIT_SIGN, TRK_HIT_TDC, TRK_HIT_RESID = 94, 112, 130

TRK_VX, TRK_PX = 16, 19  # vertex position and momentum, written by vertexing

# dimuon collections (reconstruction_classes.cuh:870-936, reconstruction_constants.h:183-184)
DIMUON_MAX, NDIMUONPARAM = 16, 36
EVT_DIM_FLOATS = DIMUON_MAX * NDIMUONPARAM
DIM_MASS, DIM_PT, DIM_XF, DIM_X1, DIM_X2, DIM_COSTHETA, DIM_PHI = 0, 1, 2, 3, 4, 5, 6
DIM_MASS_SINGLE, DIM_CHI2_SINGLE, DIM_VTX, DIM_POS_VTX, DIM_NEG_VTX = 7, 8, 9, 12, 15
DIM_POS_P, DIM_NEG_P, DIM_POS_P_SINGLE, DIM_NEG_P_SINGLE = 18, 22, 26, 30
DIM_CHI2_VTX, DIM_CHI2_KF = 34, 35
# fields the reference never computes (stored as 0 here)
DIM_UNSET_FIELDS = (DIM_MASS_SINGLE, DIM_CHI2_SINGLE, DIM_CHI2_VTX, DIM_CHI2_KF)

# monitoring histograms (reconstruction_classes.cuh:938-944, reconstruction_constants.h:216-266)
HIST_NTRIGGERS, HIST_NVARS, HIST_NVARS_TRACKS, HIST_NBINS_MAX = 11, 18, 6, 256

# the 24 chamber planes the E1039 configuration reads (reconstruction_constants.h:60)
EFF_DETID_CHAMBERS = (1, 2, 3, 4, 5, 6, 13, 14, 15, 16, 17, 18,
                      19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30)
PATH_PLANES = EFF_DETID_CHAMBERS + tuple(range(31, 55))

_PLANE_FLOAT_FIELDS = ("z",)
_PLANE_FIELDS = [
    ("z", C.c_float * NDET), ("nelem", C.c_int * NDET), ("cellwidth", C.c_float * NDET),
    ("spacing", C.c_float * NDET), ("xoffset", C.c_float * NDET), ("scalex", C.c_float * NDET),
    ("x0", C.c_float * NDET), ("x1", C.c_float * NDET), ("x2", C.c_float * NDET),
    ("costheta", C.c_float * NDET), ("scaley", C.c_float * NDET), ("y0", C.c_float * NDET),
    ("y1", C.c_float * NDET), ("y2", C.c_float * NDET), ("sintheta", C.c_float * NDET),
    ("resolution", C.c_float * NDET), ("p1x_w1", C.c_float * NDET), ("p1y_w1", C.c_float * NDET),
    ("p1z_w1", C.c_float * NDET), ("deltapx", C.c_float * NDET), ("deltapy", C.c_float * NDET),
    ("deltapz", C.c_float * NDET), ("dp1x", C.c_float * NDET), ("dp1y", C.c_float * NDET),
    ("dp1z", C.c_float * NDET), ("slope_max", C.c_float * NDET), ("inter_max", C.c_float * NDET),
]


class OrPlane(C.Structure):
    """or_plane_t == the reference's gPlane."""
    _fields_ = _PLANE_FIELDS

    def arr(self, name):
        """Field as a numpy array (a copy)."""
        return np.ctypeslib.as_array(getattr(self, name)).copy()

    def to_bytes(self):
        return bytes(C.string_at(C.addressof(self), C.sizeof(self)))

    @classmethod
    def from_bytes(cls, b):
        p = cls()
        C.memmove(C.addressof(p), b, C.sizeof(p))
        return p


RT_MAXKNOTS = 500


class OrRtTable(C.Structure):
    """or_rt_table_t: per plane the clamped cubic R-T spline (knots t, values
    r, piece coefficients b, c, d), the time window and the cell width."""
    _fields_ = [
        ("nknots", C.c_int32 * NDET), ("tmin", C.c_float * NDET), ("tmax", C.c_float * NDET),
        ("cellwidth", C.c_float * NDET),
        ("t", (C.c_double * RT_MAXKNOTS) * NDET), ("r", (C.c_double * RT_MAXKNOTS) * NDET),
        ("b", (C.c_double * RT_MAXKNOTS) * NDET), ("c", (C.c_double * RT_MAXKNOTS) * NDET),
        ("d", (C.c_double * RT_MAXKNOTS) * NDET),
    ]

    def arr(self, name):
        """Field as a numpy array (a copy)."""
        return np.ctypeslib.as_array(getattr(self, name)).copy()

    def to_bytes(self):
        return bytes(C.string_at(C.addressof(self), C.sizeof(self)))


class OrHitsView(C.Structure):
    _fields_ = [
        ("nhits_cham", C.c_void_p), ("hits_cham", C.c_void_p),
        ("nhits_hodo", C.c_void_p), ("hits_hodo", C.c_void_p),
        ("nhits_prop", C.c_void_p), ("hits_prop", C.c_void_p),
    ]


class OrTracksView(C.Structure):
    _fields_ = [("ntracks", C.c_void_p), ("tracks", C.c_void_p)]


NFEAT, MLP_H = 16, 64
MLP_NPARAM = MLP_H * NFEAT + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 1


class OrMlp(C.Structure):
    """or_mlp_t: the learned scorer's model as the kernels read it."""
    _fields_ = [("mean", C.c_float * NFEAT), ("inv_std", C.c_float * NFEAT),
                ("w1", C.c_uint16 * (MLP_H * NFEAT)), ("b1", C.c_float * MLP_H),
                ("w2", C.c_uint16 * (MLP_H * MLP_H)), ("b2", C.c_float * MLP_H),
                ("w3", C.c_float * MLP_H), ("b3", C.c_float), ("pad", C.c_float * 3)]


HIT_RECORD_DTYPE = np.dtype([("det", "<i2"), ("elem", "<i2"), ("tdc", "<f4"),
                             ("drift", "<f4"), ("flag", "<i4")])
assert HIT_RECORD_DTYPE.itemsize == 16


def plane_type(det):
    """0 chamber, 1 hodoscope, 2 prop tube."""
    return 0 if det <= NCHAM else (1 if det <= NCHAM + NHODO else 2)


def slot_of(det):
    """(type, plane index within type, per-event float stride, slot capacity)."""
    t = plane_type(det)
    if t == 0:
        return t, det - 1, EVT_CHAM_FLOATS, MAXHITS_CHAM
    if t == 1:
        return t, det - NCHAM - 1, EVT_HODO_FLOATS, MAXHITS_HODO
    return t, det - NCHAM - NHODO - 1, EVT_PROP_FLOATS, MAXHITS_PROP


class HostHits:
    """Hit collections of n events in the reference layout, as numpy arrays."""

    def __init__(self, n_events):
        self.n = n_events
        self.nhits_cham = np.zeros(n_events * NCHAM, np.uint32)
        self.hits_cham = np.zeros(n_events * EVT_CHAM_FLOATS, np.float32)
        self.nhits_hodo = np.zeros(n_events * NHODO, np.uint32)
        self.hits_hodo = np.zeros(n_events * EVT_HODO_FLOATS, np.float32)
        self.nhits_prop = np.zeros(n_events * NPROP, np.uint32)
        self.hits_prop = np.zeros(n_events * EVT_PROP_FLOATS, np.float32)

    def arrays(self):
        return (self.nhits_cham, self.hits_cham, self.nhits_hodo, self.hits_hodo,
                self.nhits_prop, self.hits_prop)

    def copy(self):
        h = HostHits.__new__(HostHits)
        h.n = self.n
        (h.nhits_cham, h.hits_cham, h.nhits_hodo, h.hits_hodo,
         h.nhits_prop, h.hits_prop) = (a.copy() for a in self.arrays())
        return h

    def view(self):
        v = OrHitsView()
        (v.nhits_cham, v.hits_cham, v.nhits_hodo, v.hits_hodo, v.nhits_prop,
         v.hits_prop) = (a.ctypes.data for a in self.arrays())
        return v

    def counts(self, e):
        """Hit count per detector id (index 1..54) of event e."""
        c = np.zeros(NDET, np.int64)
        c[1:NCHAM + 1] = self.nhits_cham[e * NCHAM:(e + 1) * NCHAM]
        c[NCHAM + 1:NCHAM + NHODO + 1] = self.nhits_hodo[e * NHODO:(e + 1) * NHODO]
        c[NCHAM + NHODO + 1:NDET] = self.nhits_prop[e * NPROP:(e + 1) * NPROP]
        return c

    def plane(self, e, det):
        """(n, [5, n] array) of event e, plane det."""
        t, k, stride, cap = slot_of(det)
        cnt = (self.nhits_cham, self.nhits_hodo, self.nhits_prop)[t]
        data = (self.hits_cham, self.hits_hodo, self.hits_prop)[t]
        per = (NCHAM, NHODO, NPROP)[t]
        n = int(cnt[e * per + k])
        base = e * stride + NHITSPARAM * cap * k
        return n, data[base:base + NHITSPARAM * n].reshape(NHITSPARAM, n)


class OrDimuonsView(C.Structure):
    _fields_ = [("ndimuons", C.c_void_p), ("dimuons", C.c_void_p)]


class OrHists(C.Structure):
    """or_hists_t == the reference's gHistsArrays."""
    _fields_ = [("nbins", C.c_int16 * (HIST_NTRIGGERS * HIST_NVARS)),
                ("pts_hw", C.c_float * (HIST_NTRIGGERS * HIST_NVARS)),
                ("xpts", C.c_float * (HIST_NTRIGGERS * HIST_NVARS * HIST_NBINS_MAX)),
                ("values", C.c_float * (HIST_NTRIGGERS * HIST_NVARS * HIST_NBINS_MAX))]

    def values_array(self):
        """values as [trigger, variable, bin] (a copy)."""
        return np.ctypeslib.as_array(self.values).reshape(HIST_NTRIGGERS, HIST_NVARS, HIST_NBINS_MAX).copy()

    def to_bytes(self):
        return bytes(C.string_at(C.addressof(self), C.sizeof(self)))

    @classmethod
    def from_bytes(cls, b):
        h = cls()
        C.memmove(C.addressof(h), bytes(b), C.sizeof(cls))
        return h


class HostDimuons:
    """Dimuon collections of n events."""

    def __init__(self, n_events):
        self.n = n_events
        self.ndimuons = np.zeros(n_events, np.uint16)
        self.dimuons = np.zeros(n_events * EVT_DIM_FLOATS, np.float32)

    def view(self):
        v = OrDimuonsView()
        v.ndimuons = self.ndimuons.ctypes.data
        v.dimuons = self.dimuons.ctypes.data
        return v

    def records(self, e):
        n = min(int(self.ndimuons[e]), DIMUON_MAX)
        return self.dimuons[e * EVT_DIM_FLOATS:e * EVT_DIM_FLOATS + n * NDIMUONPARAM].reshape(n, NDIMUONPARAM)


# event output rows (include/or_layout.h, or_output_view_t; the fields of the
# reference's ORoutput_tree, OnlineReconstruction/OROutput.h:25-102)
OUT_EV_FIELDS, OUT_HIT_FIELDS, OUT_TRACK_FIELDS, OUT_TRACKHIT_FIELDS, OUT_DIMUON_FIELDS = 9, 5, 20, 7, 39
OUT_TRACK_SRC = (TRK_STID, TRK_NHITS, TRK_CHI2, TRK_X0, TRK_Y0, TRK_TX, TRK_TY, TRK_INVP, TRK_ERR_X0, TRK_ERR_Y0,
                 TRK_ERR_TX, TRK_ERR_TY, TRK_ERR_INVP, TRK_CHARGE, TRK_VX, TRK_VX + 1, TRK_VX + 2, TRK_PX,
                 TRK_PX + 1, TRK_PX + 2)
# dimuon row fields from the 36-float record; ("sum", k) = pos + neg momentum component k
OUT_DIMUON_SRC = (DIM_MASS, DIM_PT, DIM_XF, DIM_X1, DIM_X2, DIM_COSTHETA, DIM_PHI, DIM_MASS_SINGLE, DIM_CHI2_SINGLE,
                  DIM_VTX, DIM_VTX + 1, DIM_VTX + 2, ("sum", 0), ("sum", 1), ("sum", 2), DIM_POS_VTX, DIM_POS_VTX + 1,
                  DIM_POS_VTX + 2, DIM_NEG_VTX, DIM_NEG_VTX + 1, DIM_NEG_VTX + 2, DIM_POS_P + 3, DIM_POS_P,
                  DIM_POS_P + 1, DIM_POS_P + 2, DIM_NEG_P + 3, DIM_NEG_P, DIM_NEG_P + 1, DIM_NEG_P + 2,
                  DIM_POS_P_SINGLE + 3, DIM_POS_P_SINGLE, DIM_POS_P_SINGLE + 1, DIM_POS_P_SINGLE + 2,
                  DIM_NEG_P_SINGLE + 3, DIM_NEG_P_SINGLE, DIM_NEG_P_SINGLE + 1, DIM_NEG_P_SINGLE + 2, DIM_CHI2_VTX,
                  DIM_CHI2_KF)


class OrOutputView(C.Structure):
    _fields_ = [("events", C.c_void_p), ("hits", C.c_void_p), ("tracks", C.c_void_p), ("track_hits", C.c_void_p),
                ("dimuons", C.c_void_p), ("cap_events", C.c_int64), ("cap_hits", C.c_int64),
                ("cap_tracks", C.c_int64), ("cap_track_hits", C.c_int64), ("cap_dimuons", C.c_int64),
                ("counts", C.c_void_p)]


class HostTracks:
    """Track collections of n events in the reference layout."""

    def __init__(self, n_events):
        self.n = n_events
        self.ntracks = np.zeros(n_events * NSLOTS, np.uint16)
        self.tracks = np.zeros(n_events * EVT_TRK_FLOATS, np.float32)

    def view(self):
        v = OrTracksView()
        v.ntracks = self.ntracks.ctypes.data
        v.tracks = self.tracks.ctypes.data
        return v

    def copy(self):
        t = HostTracks.__new__(HostTracks)
        t.n = self.n
        t.ntracks = self.ntracks.copy()
        t.tracks = self.tracks.copy()
        return t

    def records(self, e):
        """List of (slot, position, 148-float record) of event e."""
        out = []
        for s in range(NSLOTS):
            for k in range(int(self.ntracks[e * NSLOTS + s])):
                base = e * EVT_TRK_FLOATS + (s * SLOTCAP + k) * NTRKPARAM
                out.append((s, k, self.tracks[base:base + NTRKPARAM]))
        return out


# byte sizes of the reference's fixed-capacity structs (REF_EVTMAX events):
# gEventHitCollections (reconstruction_classes.cuh:76-87, 4-byte members, no
# padding) and gEventTrackCollection (:542-544: uint16 counts, then floats)
REF_HITS_BYTES = REF_EVTMAX * (4 * (NCHAM + NHODO + NPROP) + 4 * (EVT_CHAM_FLOATS + EVT_HODO_FLOATS + EVT_PROP_FLOATS))
REF_TRACKS_BYTES = REF_EVTMAX * (2 * NSLOTS + 4 * EVT_TRK_FLOATS)
