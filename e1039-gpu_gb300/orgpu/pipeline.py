"""Host-side mirror of the reference's launch chain
(OnlineReconstruction/online_reconstruction.cu:738-1033) on top of the C ABI.

`Reconstruction` owns a library context on one device; `DeviceBatch` owns the
device buffers of a batch of events in the reference layout (hit
collections, track collections, HasTooManyHits, nTracklets).  The stage
methods keep the reference kernel names' meaning and order:

    gkernel_eR                  -> Reconstruction.event_reduce
    gKernel_XZ_tracking         -> Reconstruction.xz_tracking
    gKernel_YZ_tracking         -> Reconstruction.yz_tracking
    gKernel_BackTrackCleaning*  -> Reconstruction.back_track_cleaning
    gKernel_Global_tracking     -> Reconstruction.global_tracking

PyTorch is used for device memory and streams only; all work runs in the
library's sm_103a kernels.
"""
import ctypes as C

import numpy as np

from . import _lib
from . import layout as L


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise _lib.OrError(_lib.OR_ERR_CUDA, "no CUDA device: the reconstruction path runs on the GPU only")
    return torch


def rt_to_device(rt, device=0):
    """Copy an OrRtTable (host, from _lib.rt_load) to a device uint8 tensor,
    the `rt_dev` argument of Reconstruction.pack_rt / rt_apply."""
    torch = _torch()
    raw = np.frombuffer(rt.to_bytes(), np.uint8)
    return torch.from_numpy(raw.copy()).to(torch.device("cuda", device))


class DeviceBatch:
    """Device buffers of n events in the reference layout."""

    def __init__(self, n_events, device=0, with_tracks=True):
        torch = _torch()
        self.n = int(n_events)
        dev = torch.device("cuda", device)
        u32, f32 = torch.int32, torch.float32
        n = self.n
        self.nhits_cham = torch.zeros(n * L.NCHAM, dtype=u32, device=dev)
        self.hits_cham = torch.empty(n * L.EVT_CHAM_FLOATS, dtype=f32, device=dev)
        self.nhits_hodo = torch.zeros(n * L.NHODO, dtype=u32, device=dev)
        self.hits_hodo = torch.empty(n * L.EVT_HODO_FLOATS, dtype=f32, device=dev)
        self.nhits_prop = torch.zeros(n * L.NPROP, dtype=u32, device=dev)
        self.hits_prop = torch.empty(n * L.EVT_PROP_FLOATS, dtype=f32, device=dev)
        self.toomany = torch.zeros(n, dtype=torch.uint8, device=dev)
        self.ntracklets = torch.zeros(n, dtype=torch.int32, device=dev)
        if with_tracks:
            self.ntracks = torch.zeros(n * L.NSLOTS, dtype=torch.int16, device=dev)
            self.tracks = torch.zeros(n * L.EVT_TRK_FLOATS, dtype=f32, device=dev)
        else:
            self.ntracks = self.tracks = None

    def hits_view(self):
        v = L.OrHitsView()
        (v.nhits_cham, v.hits_cham, v.nhits_hodo, v.hits_hodo, v.nhits_prop,
         v.hits_prop) = (t.data_ptr() for t in (self.nhits_cham, self.hits_cham, self.nhits_hodo, self.hits_hodo,
                                                 self.nhits_prop, self.hits_prop))
        return v

    def tracks_view(self):
        v = L.OrTracksView()
        v.ntracks = self.ntracks.data_ptr()
        v.tracks = self.tracks.data_ptr()
        return v

    # -- host <-> device ----------------------------------------------------
    def upload_hits(self, h):
        """Copy a layout.HostHits (numpy) of the same size to the device."""
        torch = _torch()
        assert h.n == self.n
        for dst, src in zip((self.nhits_cham, self.hits_cham, self.nhits_hodo, self.hits_hodo, self.nhits_prop,
                             self.hits_prop), h.arrays()):
            dst.copy_(torch.from_numpy(src.view(np.int32) if src.dtype == np.uint32 else src))

    def upload_tracks(self, t):
        torch = _torch()
        self.ntracks.copy_(torch.from_numpy(t.ntracks.view(np.int16)))
        self.tracks.copy_(torch.from_numpy(t.tracks))

    def download_hits(self):
        h = L.HostHits.__new__(L.HostHits)
        h.n = self.n
        h.nhits_cham = self.nhits_cham.cpu().numpy().view(np.uint32)
        h.hits_cham = self.hits_cham.cpu().numpy()
        h.nhits_hodo = self.nhits_hodo.cpu().numpy().view(np.uint32)
        h.hits_hodo = self.hits_hodo.cpu().numpy()
        h.nhits_prop = self.nhits_prop.cpu().numpy().view(np.uint32)
        h.hits_prop = self.hits_prop.cpu().numpy()
        return h

    def download_tracks(self):
        t = L.HostTracks.__new__(L.HostTracks)
        t.n = self.n
        t.ntracks = self.ntracks.cpu().numpy().view(np.uint16)
        t.tracks = self.tracks.cpu().numpy()
        return t


class DeviceDimuons:
    """Device dimuon collections of n events (reference layout)."""

    def __init__(self, n_events, device=0):
        torch = _torch()
        dev = torch.device("cuda", device)
        self.n = int(n_events)
        self.ndimuons = torch.zeros(self.n, dtype=torch.int16, device=dev)
        self.dimuons = torch.zeros(self.n * L.EVT_DIM_FLOATS, dtype=torch.float32, device=dev)

    def view(self):
        v = L.OrDimuonsView()
        v.ndimuons = self.ndimuons.data_ptr()
        v.dimuons = self.dimuons.data_ptr()
        return v

    def download(self):
        d = L.HostDimuons.__new__(L.HostDimuons)
        d.n = self.n
        d.ndimuons = self.ndimuons.cpu().numpy().view(np.uint16)
        d.dimuons = self.dimuons.cpu().numpy()
        return d


class DeviceHists:
    """The histogram tables (or_hists_t) in device memory, initialised with
    the reference's binning (or_hist_table_init) and zero counts."""

    def __init__(self, device=0):
        torch = _torch()
        h = L.OrHists()
        _lib.lib().or_hist_table_init(C.byref(h))
        raw = np.frombuffer(h.to_bytes(), np.uint8).copy()
        self.buf = torch.from_numpy(raw).to(torch.device("cuda", device))

    def ptr(self):
        return self.buf.data_ptr()

    def zero_counts(self):
        off = L.OrHists.values.offset
        self.buf[off:].zero_()

    def download(self):
        return L.OrHists.from_bytes(self.buf.cpu().numpy().tobytes())


class Reconstruction:
    """One library context (one device) with its geometry."""

    def __init__(self, plane, device=0, lib=None, max_events=None):
        """lib: a library handle from _lib.load() (default: the product
        build, _lib.lib()).  max_events: size the YZ scratch for batches of at
        most that many events (or_create_sized; larger batches stay correct,
        only slower); None: or_create's 100,000-event sizes."""
        torch = _torch()
        self.device = device
        self.lib = lib if lib is not None else _lib.lib()
        self.ctx = C.c_void_p()
        if max_events is None:
            _lib.check(self.lib.or_create(device, C.byref(self.ctx)), "or_create")
        else:
            _lib.check(self.lib.or_create_sized(device, int(max_events), C.byref(self.ctx)), "or_create_sized")
        self.plane = plane
        _lib.check(self.lib.or_set_geometry(self.ctx, C.byref(plane)), "or_set_geometry")
        self._torch = torch

    def close(self):
        if self.ctx:
            self.lib.or_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _stream(self, stream):
        if stream is None:
            stream = self._torch.cuda.current_stream(self.device)
        return C.c_void_p(stream.cuda_stream)

    # stage entry points (online_reconstruction.cu:776-894)
    def event_reduce(self, b, stream=None):
        _lib.check(self.lib.or_event_reduce(self.ctx, b.hits_view(), b.toomany.data_ptr(), b.n,
                                            self._stream(stream)), "or_event_reduce")

    def xz_tracking(self, b, stream=None):
        _lib.check(self.lib.or_xz(self.ctx, b.hits_view(), b.tracks_view(), b.ntracklets.data_ptr(),
                                  b.toomany.data_ptr(), b.n, self._stream(stream)), "or_xz")

    def yz_tracking(self, b, stream=None):
        _lib.check(self.lib.or_yz(self.ctx, b.hits_view(), b.tracks_view(), b.toomany.data_ptr(), b.n,
                                  self._stream(stream)), "or_yz")

    def back_track_cleaning(self, b, stream=None):
        _lib.check(self.lib.or_back_clean(self.ctx, b.tracks_view(), b.toomany.data_ptr(), b.n,
                                          self._stream(stream)), "or_back_clean")

    def global_tracking(self, b, stream=None):
        _lib.check(self.lib.or_global(self.ctx, b.hits_view(), b.tracks_view(), b.toomany.data_ptr(), b.n,
                                      self._stream(stream)), "or_global")

    # post-global selection (online_reconstruction.cu:914-933)
    def prop_segment_matching(self, b, stream=None):
        _lib.check(self.lib.or_prop_matching(self.ctx, b.hits_view(), b.tracks_view(), b.toomany.data_ptr(), b.n,
                                             self._stream(stream)), "or_prop_matching")

    def global_track_cleaning(self, b, stream=None):
        _lib.check(self.lib.or_global_clean(self.ctx, b.tracks_view(), b.toomany.data_ptr(), b.n,
                                            self._stream(stream)), "or_global_clean")

    def selection(self, b, stream=None):
        _lib.check(self.lib.or_run_selection(self.ctx, b.hits_view(), b.tracks_view(), b.toomany.data_ptr(), b.n,
                                             self._stream(stream)), "or_run_selection")

    # after the selection (online_reconstruction.cu:939-983)
    def vertexing(self, b, stream=None):
        _lib.check(self.lib.or_vertexing(self.ctx, b.tracks_view(), b.toomany.data_ptr(), b.n, self._stream(stream)),
                   "or_vertexing")

    def dimuons(self, b, d, stream=None):
        _lib.check(self.lib.or_dimuons(self.ctx, b.tracks_view(), d.view(), b.toomany.data_ptr(), b.n,
                                       self._stream(stream)), "or_dimuons")

    def fill_histograms(self, b, d, hists, trigger_bits=None, stream=None):
        """Add this batch's counts into hists (DeviceHists); trigger_bits: a
        device int32 tensor of b.n entries or None."""
        tb = None if trigger_bits is None else trigger_bits.data_ptr()
        _lib.check(self.lib.or_fill_histograms(self.ctx, b.tracks_view(), d.view(), tb, b.toomany.data_ptr(),
                                               hists.ptr(), b.n, self._stream(stream)), "or_fill_histograms")

    def run_physics(self, b, d, hists=None, trigger_bits=None, stream=None):
        tb = None if trigger_bits is None else trigger_bits.data_ptr()
        _lib.check(self.lib.or_run_physics(self.ctx, b.tracks_view(), d.view(), tb, b.toomany.data_ptr(),
                                           None if hists is None else hists.ptr(), b.n, self._stream(stream)),
                   "or_run_physics")

    def output_rows(self, b, d, raw_hits=None, event_ids=None, min_stid=7.0, caps=None, stream=None):
        """The reference's per-event output (ORoutput_tree fields) as row
        tables, read back to the host: a dict of numpy arrays "events" [n, 9]
        int64, "hits" [n, 5], "tracks" [n, 20], "track_hits" [n, 7],
        "dimuons" [n, 39] float32.  raw_hits / event_ids: device int32
        tensors of b.n entries or None.  caps: rows per table; when given and
        too small, OrError (capacity); when None, the tables are sized from
        the counts of a first call if the defaults do not hold them."""
        fixed = caps is not None
        if caps is None:
            caps = (b.n, b.n * 512, b.n * 8, b.n * 8 * L.MAXHITS_PER_TRACK, b.n * 4)
        t, n = self._output_rows_once(b, d, raw_hits, event_ids, min_stid, caps, stream)
        if any(a > c for a, c in zip(n, caps)):
            if fixed:
                raise _lib.OrError(_lib.OR_ERR_CAPACITY, f"output rows {n} exceed capacities {tuple(caps)}")
            t, n = self._output_rows_once(b, d, raw_hits, event_ids, min_stid, tuple(n), stream)
        widths = (L.OUT_EV_FIELDS, L.OUT_HIT_FIELDS, L.OUT_TRACK_FIELDS, L.OUT_TRACKHIT_FIELDS, L.OUT_DIMUON_FIELDS)
        return {k: t[k][:m * w].view(m, w).cpu().numpy()
                for k, m, w in zip(("events", "hits", "tracks", "track_hits", "dimuons"), n, widths)}

    def _output_rows_once(self, b, d, raw_hits, event_ids, min_stid, caps, stream):
        torch = _torch()
        dev = b.toomany.device
        t = {"events": torch.empty(max(1, caps[0]) * L.OUT_EV_FIELDS, dtype=torch.int64, device=dev),
             "hits": torch.empty(max(1, caps[1]) * L.OUT_HIT_FIELDS, dtype=torch.float32, device=dev),
             "tracks": torch.empty(max(1, caps[2]) * L.OUT_TRACK_FIELDS, dtype=torch.float32, device=dev),
             "track_hits": torch.empty(max(1, caps[3]) * L.OUT_TRACKHIT_FIELDS, dtype=torch.float32, device=dev),
             "dimuons": torch.empty(max(1, caps[4]) * L.OUT_DIMUON_FIELDS, dtype=torch.float32, device=dev)}
        counts = torch.zeros(5, dtype=torch.int64, device=dev)
        v = L.OrOutputView()
        v.events, v.hits, v.tracks, v.track_hits, v.dimuons = (t[k].data_ptr() for k in
                                                                ("events", "hits", "tracks", "track_hits", "dimuons"))
        v.cap_events, v.cap_hits, v.cap_tracks, v.cap_track_hits, v.cap_dimuons = (int(c) for c in caps)
        v.counts = counts.data_ptr()
        _lib.check(self.lib.or_output_rows(self.ctx, b.hits_view(), b.tracks_view(), d.view(), b.toomany.data_ptr(),
                                           None if raw_hits is None else raw_hits.data_ptr(),
                                           None if event_ids is None else event_ids.data_ptr(), float(min_stid), v,
                                           b.n, self._stream(stream)), "or_output_rows")
        self.sync(stream)
        return t, [int(x) for x in counts.cpu().tolist()]

    def run_batch(self, b, stream=None):
        _lib.check(self.lib.or_run_batch(self.ctx, b.hits_view(), b.tracks_view(), b.ntracklets.data_ptr(),
                                         b.toomany.data_ptr(), b.n, self._stream(stream)), "or_run_batch")

    def pack(self, b, d_records, d_offsets, d_wire_pos_f, stream=None):
        """Device packer: compact records (device uint8 tensor of HIT_RECORD_DTYPE
        bytes) + int64 offsets -> b's hit collections."""
        _lib.check(self.lib.or_pack_hits(self.ctx, d_records.data_ptr(), d_offsets.data_ptr(), b.n,
                                          d_wire_pos_f.data_ptr(), b.hits_view(), self._stream(stream)),
                   "or_pack_hits")

    def set_yz_pool_limit(self, entries):
        """Survivor-pool entries the split YZ path may use (-1: all); units
        that do not fit run whole, with the same results."""
        _lib.check(self.lib.or_set_yz_pool_limit(self.ctx, int(entries)), "or_set_yz_pool_limit")

    def pack_rt(self, b, d_records, d_offsets, d_wire_pos_f, d_rt, stream=None):
        """Device packer with the drift distance from the R-T calibration
        (d_rt: device uint8 tensor holding an OrRtTable, see rt_to_device)."""
        _lib.check(self.lib.or_pack_hits_rt(self.ctx, d_records.data_ptr(), d_offsets.data_ptr(), b.n,
                                             d_wire_pos_f.data_ptr(), d_rt.data_ptr(), b.hits_view(),
                                             self._stream(stream)), "or_pack_hits_rt")

    def rt_apply(self, b, d_rt, stream=None):
        """R-T conversion in place on b's packed hits (drift from tdc)."""
        _lib.check(self.lib.or_rt_apply(self.ctx, d_rt.data_ptr(), b.hits_view(), b.n, self._stream(stream)),
                   "or_rt_apply")

    def collect(self, b, d_out, d_count, stid=6.0, stream=None):
        """Gather tracks with stationID == stid into d_out (float32 rows of
        COLLECT_STRIDE); d_count (int64[1]) gets the number found."""
        cap = d_out.numel() // L.COLLECT_STRIDE
        _lib.check(self.lib.or_collect_tracks(self.ctx, b.tracks_view(), b.toomany.data_ptr(), b.n, float(stid),
                                              d_out.data_ptr(), cap, d_count.data_ptr(), self._stream(stream)),
                   "or_collect_tracks")

    def set_yz_work_counting(self, enabled):
        """Let YZ calls on this context add up their work counters (costs
        about 2 % of the stage; off by default)."""
        _lib.check(self.lib.or_set_yz_work_counting(self.ctx, 1 if enabled else 0), "or_set_yz_work_counting")

    def yz_work_counts(self):
        """(fitted combinations, sum of their hit counts, first-cut survivors)
        of the last YZ call on this context; call after sync()."""
        c = (C.c_int64 * 3)()
        _lib.check(self.lib.or_yz_work_counts(self.ctx, c), "or_yz_work_counts")
        return int(c[0]), int(c[1]), int(c[2])

    def sync(self, stream=None):
        """Wait for the stream and raise on device-side error words."""
        _lib.check(self.lib.or_stream_sync(self.ctx, self._stream(stream)), "or_stream_sync")
