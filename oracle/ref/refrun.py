"""Run the reference's own kernels, compiled by build_ref.py, on the GPU
through the CUDA driver API.  TEST INFRASTRUCTURE ONLY: used to pin the CPU
oracle (tests/golden/make_golden.py); the library never loads these images.

The kernels take the reference's fixed-capacity structs (EstnEvtMax = 10000
events, reconstruction_constants.h:20): gEventHitCollections
(reconstruction_classes.cuh:76-87), gEventTrackCollection (:542-544), gPlane
(:947-977) and a bool per event.  Each stage is launched as the reference
host launches it (online_reconstruction.cu:776-894): one block per event,
8 threads for the event reducer, 32 for the others.

The reference's XZ kernel (reconstruction_kernels.cuh:182-855) is not
exposed: it calls __syncthreads() inside thread-dependent branches (K:684,
K:724, K:767, K:807), which CUDA leaves undefined and which may hang.

Inputs must stay inside the reference's array bounds (raw chamber hits per
plane <= 120, windowed hits and pairs <= 100 per projection); callers filter
events with the oracle's domain counters before launching.
"""
import ctypes as C
import os

import numpy as np

from orgpu import layout as L

from . import build_ref

E = L.REF_EVTMAX
HITS_BYTES = 4 * E * (L.NCHAM + L.NHODO + L.NPROP) + 4 * E * (L.EVT_CHAM_FLOATS + L.EVT_HODO_FLOATS +
                                                             L.EVT_PROP_FLOATS)
TRACKS_BYTES = 2 * E * L.NSLOTS + 4 * E * L.EVT_TRK_FLOATS

KERNELS = {
    "er": "_Z10gkernel_eRP20gEventHitCollectionsPb",
    "yz": "_Z19gKernel_YZ_trackingP20gEventHitCollectionsP21gEventTrackCollectionPK6gPlanePb",
    "clean": "_Z25gKernel_BackTrackCleaningP21gEventTrackCollectionPKb",
    "clean_x": "_Z38gKernel_BackTrackCleaning_crossthreadsP21gEventTrackCollectionPKb",
    "global": "_Z23gKernel_Global_trackingP20gEventHitCollectionsP21gEventTrackCollectionPK6gPlanePb",
    "prop": "_Z27gKernel_PropSegmentMatchingP20gEventHitCollectionsP21gEventTrackCollectionPKfPKb",
    "gclean": "_Z27gKernel_GlobalTrackCleaningP21gEventTrackCollectionPKb",
    "gclean_x": "_Z40gKernel_GlobalTrackCleaning_crossthreadsP21gEventTrackCollectionPKb",
    "vertexing": "_Z17gKernel_VertexingP21gEventTrackCollectionPKfPb",
    "dimuons": "_Z22gKernel_DimuonBuildingP21gEventTrackCollectionP22gEventDimuonCollectionPKfPKb",
    "hists": "_Z31gKernel_fill_display_histogramsP21gEventTrackCollectionP22gEventDimuonCollectionP12gHistsArraysPKiPKb",
    # test-only kernel of oracle/ref/xz_pin.cuh: the XZ candidates on the reference's helpers
    "xz_pin": "xz_pin_kernel",
}
XZ_REC = 32  # floats per candidate record of xz_pin_kernel
# gEventDimuonCollection (reconstruction_classes.cuh:870-872): unsigned short
# NDimuons[E], then float DimuonsRawData[E*16*36] (4-byte aligned after 2*E bytes)
DIM_DATA_OFF = 2 * E
DIMS_BYTES = DIM_DATA_OFF + 4 * E * L.EVT_DIM_FLOATS

# byte offsets of the members of gEventHitCollections (4-byte members, no padding)
_HIT_SECTIONS = []
_o = 0
for _name, _cnt, _dt in (("nhits_cham", E * L.NCHAM, np.uint32), ("hits_cham", E * L.EVT_CHAM_FLOATS, np.float32),
                         ("nhits_hodo", E * L.NHODO, np.uint32), ("hits_hodo", E * L.EVT_HODO_FLOATS, np.float32),
                         ("nhits_prop", E * L.NPROP, np.uint32), ("hits_prop", E * L.EVT_PROP_FLOATS, np.float32)):
    _HIT_SECTIONS.append((_name, _o, _dt))
    _o += 4 * _cnt
assert _o == HITS_BYTES
_TRK_OFF = 2 * E * L.NSLOTS


class CudaDriverError(RuntimeError):
    pass


class RefKernels:
    """One loaded image ("fmad0" or "fmad1") plus the device structs."""

    def __init__(self, variant="fmad0", device=0):
        import torch
        self.torch = torch
        path = build_ref.image_path(variant)
        if not os.path.exists(path):
            raise FileNotFoundError(f"reference image {path} not built (oracle/ref/build_ref.py)")
        torch.cuda.set_device(device)
        torch.zeros(1, device="cuda")  # the primary context is current from here on
        self.cu = C.CDLL("libcuda.so.1")
        self.mod = C.c_void_p()
        self._chk(self.cu.cuModuleLoad(C.byref(self.mod), path.encode()), "cuModuleLoad")
        self.fn = {}
        for key, name in KERNELS.items():
            f = C.c_void_p()
            self._chk(self.cu.cuModuleGetFunction(C.byref(f), self.mod, name.encode()), f"cuModuleGetFunction {key}")
            self.fn[key] = f
        dev = torch.device("cuda", device)
        self.hits = torch.zeros(HITS_BYTES, dtype=torch.uint8, device=dev)
        self.tracks = torch.zeros(TRACKS_BYTES, dtype=torch.uint8, device=dev)
        self.plane = torch.zeros(C.sizeof(L.OrPlane), dtype=torch.uint8, device=dev)
        self.flags = torch.zeros(E, dtype=torch.uint8, device=dev)
        self.dims = torch.zeros(DIMS_BYTES, dtype=torch.uint8, device=dev)
        self.hists = torch.zeros(C.sizeof(L.OrHists), dtype=torch.uint8, device=dev)
        self.trig = torch.zeros(E, dtype=torch.int32, device=dev)
        self.flags_hist = torch.zeros(E, dtype=torch.uint8, device=dev)
        # when a dict: device milliseconds of every launch, accumulated by
        # kernel key (CUDA events on the launching stream around the launch)
        self.timing = None

    def _chk(self, rc, what):
        if rc != 0:
            name = C.c_char_p()
            self.cu.cuGetErrorName(rc, C.byref(name))
            raise CudaDriverError(f"{what}: CUresult {rc} ({name.value.decode() if name.value else '?'})")

    def close(self):
        if self.mod:
            self.torch.cuda.synchronize()
            self.cu.cuModuleUnload(self.mod)
            self.mod = C.c_void_p()

    # -- struct I/O ------------------------------------------------------------
    def view(self, name, n):
        """Typed device view of the first n events of one member: a hit
        section by name ("nhits_cham", "hits_cham", ...), "ntracks",
        "tracks" or "flags" -- for device-to-device copies and comparisons
        against the library's DeviceBatch buffers, which use the same layout."""
        t = self.torch
        assert n <= E
        if name == "flags":
            return self.flags[:n]
        if name == "ntracks":
            return self.tracks[:2 * n * L.NSLOTS].view(t.int16)
        if name == "tracks":
            return self.tracks[_TRK_OFF:_TRK_OFF + 4 * n * L.EVT_TRK_FLOATS].view(t.float32)
        per = {"nhits_cham": L.NCHAM, "hits_cham": L.EVT_CHAM_FLOATS, "nhits_hodo": L.NHODO,
               "hits_hodo": L.EVT_HODO_FLOATS, "nhits_prop": L.NPROP, "hits_prop": L.EVT_PROP_FLOATS}[name]
        off = {nm: o for nm, o, _ in _HIT_SECTIONS}[name]
        v = self.hits[off:off + 4 * n * per]
        return v.view(t.int32) if name.startswith("nhits") else v.view(t.float32)

    def set_plane(self, plane):
        self.plane.copy_(self.torch.frombuffer(bytearray(plane.to_bytes()), dtype=self.torch.uint8))

    def put_hits(self, h):
        assert h.n <= E
        t = self.torch
        for (name, off, dt), arr in zip(_HIT_SECTIONS, h.arrays()):
            b = arr.view(np.uint8)
            self.hits[off:off + b.size].copy_(t.from_numpy(b))

    def get_hits(self, n):
        h = L.HostHits(n)
        for (name, off, dt), arr in zip(_HIT_SECTIONS, h.arrays()):
            b = self.hits[off:off + arr.nbytes].cpu().numpy()
            arr[:] = b.view(dt)
        return h

    def put_tracks(self, t):
        assert t.n <= E
        self.tracks[:t.ntracks.nbytes].copy_(self.torch.from_numpy(t.ntracks.view(np.uint8)))
        self.tracks[_TRK_OFF:_TRK_OFF + t.tracks.nbytes].copy_(self.torch.from_numpy(t.tracks.view(np.uint8)))

    def get_tracks(self, n):
        t = L.HostTracks(n)
        t.ntracks[:] = self.tracks[:t.ntracks.nbytes].cpu().numpy().view(np.uint16)
        t.tracks[:] = self.tracks[_TRK_OFF:_TRK_OFF + t.tracks.nbytes].cpu().numpy().view(np.float32)
        return t

    def put_flags(self, toomany):
        n = toomany.size
        self.flags[:n].copy_(self.torch.from_numpy(np.ascontiguousarray(toomany, np.uint8)))

    def get_flags(self, n):
        return self.flags[:n].cpu().numpy().copy()

    # -- launches --------------------------------------------------------------
    def _launch(self, key, n, threads, *ptrs):
        vals = [C.c_void_p(p) for p in ptrs]
        args = (C.c_void_p * len(vals))(*[C.cast(C.byref(v), C.c_void_p) for v in vals])
        stream = C.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        if self.timing is not None:
            ev = [self.torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record()
        self._chk(self.cu.cuLaunchKernel(self.fn[key], n, 1, 1, threads, 1, 1, 0, stream, args, None),
                  f"launch {key}")
        if self.timing is not None:
            ev[1].record()
        self.torch.cuda.synchronize()
        self._chk(self.cu.cuCtxSynchronize(), f"after {key}")
        if self.timing is not None:
            self.timing[key] = self.timing.get(key, 0.0) + ev[0].elapsed_time(ev[1])

    def event_reduce(self, n):
        self._launch("er", n, 8, self.hits.data_ptr(), self.flags.data_ptr())

    def yz(self, n):
        self._launch("yz", n, 32, self.hits.data_ptr(), self.tracks.data_ptr(), self.plane.data_ptr(),
                     self.flags.data_ptr())

    def back_clean(self, n):
        self._launch("clean", n, 32, self.tracks.data_ptr(), self.flags.data_ptr())
        self._launch("clean_x", n, 32, self.tracks.data_ptr(), self.flags.data_ptr())

    def selection(self, n):
        """PropSegmentMatching (z = the plane's z array, its first member),
        then GlobalTrackCleaning and ..._crossthreads (M:914-933)."""
        self._launch("prop", n, 32, self.hits.data_ptr(), self.tracks.data_ptr(), self.plane.data_ptr(),
                     self.flags.data_ptr())
        self._launch("gclean", n, 32, self.tracks.data_ptr(), self.flags.data_ptr())
        self._launch("gclean_x", n, 32, self.tracks.data_ptr(), self.flags.data_ptr())

    def vertexing(self, n):
        """gKernel_Vertexing<<<n, 32>>>(tracks, plane z, flags) (M:939-945)."""
        self._launch("vertexing", n, 32, self.tracks.data_ptr(), self.plane.data_ptr(), self.flags.data_ptr())

    def dimuons(self, n):
        """gKernel_DimuonBuilding<<<n, 1>>>(tracks, dimuons, plane z, flags) (M:962-968)."""
        self._launch("dimuons", n, 1, self.tracks.data_ptr(), self.dims.data_ptr(), self.plane.data_ptr(),
                     self.flags.data_ptr())

    def histograms(self, events, table, trigger_bits):
        """gKernel_fill_display_histograms<<<., 1>>> (M:983) on the given
        events, one event per launch: the kernel adds with a plain "+=" from
        every block, so concurrent blocks would lose counts.  The kernel
        indexes every per-event array with blockIdx.x, so event e runs as
        block e of a grid of e+1 blocks whose other blocks see the "too many
        hits" flag and return at once.  `table` is an OrHists with the binning
        and the starting counts; returns the OrHists after the fills."""
        self.hists.copy_(self.torch.frombuffer(bytearray(table.to_bytes()), dtype=self.torch.uint8))
        n = len(trigger_bits)
        self.trig[:n].copy_(self.torch.from_numpy(np.ascontiguousarray(trigger_bits, np.int32)))
        for e in events:
            e = int(e)
            self.flags_hist[:e].fill_(1)
            self.flags_hist[e] = self.flags[e]
            self._launch("hists", e + 1, 1, self.tracks.data_ptr(), self.dims.data_ptr(), self.hists.data_ptr(),
                         self.trig.data_ptr(), self.flags_hist.data_ptr())
        return L.OrHists.from_bytes(self.hists.cpu().numpy().tobytes())

    def put_dimuons(self, d):
        assert d.n <= E
        self.dims[:d.ndimuons.nbytes].copy_(self.torch.from_numpy(d.ndimuons.view(np.uint8)))
        self.dims[DIM_DATA_OFF:DIM_DATA_OFF + d.dimuons.nbytes].copy_(self.torch.from_numpy(d.dimuons.view(np.uint8)))

    def get_dimuons(self, n):
        d = L.HostDimuons(n)
        d.ndimuons[:] = self.dims[:2 * n].cpu().numpy().view(np.uint16)
        d.dimuons[:] = self.dims[DIM_DATA_OFF:DIM_DATA_OFF + 4 * n * L.EVT_DIM_FLOATS].cpu().numpy().view(np.float32)
        return d

    def xz_candidates(self, n, cap=64):
        """The XZ stage's accepted candidates of the first n events on the
        loaded hits (put_hits: the reduced hits) and flags (put_flags: the
        event reducer's), computed by xz_pin_kernel with the reference's
        helpers: (records float32 [n, 32, cap, 32], counts int32 [n, 32],
        status int32 [n, 32]) per (event, reference thread); see
        oracle/ref/xz_pin.cuh for the record layout and status bits."""
        t = self.torch
        dev = self.hits.device
        out = t.zeros(n * 32 * cap * XZ_REC, dtype=t.float32, device=dev)
        nout = t.zeros(n * 32, dtype=t.int32, device=dev)
        status = t.zeros(n * 32, dtype=t.int32, device=dev)
        vals = [C.c_void_p(self.hits.data_ptr()), C.c_void_p(self.plane.data_ptr()), C.c_void_p(self.flags.data_ptr()),
                C.c_int(n), C.c_void_p(out.data_ptr()), C.c_int(cap), C.c_void_p(nout.data_ptr()),
                C.c_void_p(status.data_ptr())]
        args = (C.c_void_p * len(vals))(*[C.cast(C.byref(v), C.c_void_p) for v in vals])
        stream = C.c_void_p(t.cuda.current_stream().cuda_stream)
        threads = 128
        blocks = (n * 32 + threads - 1) // threads
        if blocks:
            self._chk(self.cu.cuLaunchKernel(self.fn["xz_pin"], blocks, 1, 1, threads, 1, 1, 0, stream, args, None),
                      "launch xz_pin")
        t.cuda.synchronize()
        self._chk(self.cu.cuCtxSynchronize(), "after xz_pin")
        return (out.view(n, 32, cap, XZ_REC).cpu().numpy(), nout.view(n, 32).cpu().numpy(),
                status.view(n, 32).cpu().numpy())

    def global_tracking(self, n):
        self._launch("global", n, 32, self.hits.data_ptr(), self.tracks.data_ptr(), self.plane.data_ptr(),
                     self.flags.data_ptr())
