"""ctypes binding of liborgpu.so (include/or_gb300.h).

The library is the product: there is no Python or CPU fallback.  If the
shared object is missing or cannot be loaded, every entry point raises.
"""
import ctypes as C
import os

from . import layout as L

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "liborgpu.so")

OR_OK, OR_ERR_ARG, OR_ERR_CUDA, OR_ERR_IO, OR_ERR_NOMEM, OR_ERR_CAPACITY, OR_ERR_TIMEOUT, OR_ERR_NOGEOM = range(8)

# every symbol include/or_gb300.h declares
EXPORTS = ("or_version", "or_last_error", "or_status_string", "or_geometry_load", "or_create", "or_create_sized", "or_context_bytes", "or_destroy",
           "or_set_geometry", "or_stream_sync", "or_event_reduce", "or_xz", "or_yz", "or_back_clean", "or_global",
           "or_run_batch", "or_hits_view_from_collection", "or_tracks_view_from_collection", "or_hits_view_bytes",
           "or_tracks_view_bytes", "or_pack_hits", "or_collect_tracks", "or_yz_noalloc", "or_tracklet_rows",
           "or_tracklet_features", "or_mlp_score", "or_keep_mask", "or_yz_pruned", "or_run_batch_learned",
           "or_tracklet_labels", "or_track_agreement", "or_mlp_grad_blocks", "or_mlp_forward", "or_mlp_gradient",
           "or_mlp_adam", "or_prop_matching", "or_global_clean", "or_run_selection", "or_set_launch",
           "or_get_launch", "or_vertexing", "or_dimuons", "or_fill_histograms", "or_hist_table_init",
           "or_run_physics", "or_output_rows", "or_rt_load", "or_rt_set_plane", "or_rt_table_bytes",
           "or_pack_hits_rt", "or_rt_apply", "or_set_yz_pool_limit", "or_selftest_bounded_wait",
           "or_yz_work_counts", "or_set_yz_work_counting", "or_gkernel_eR", "or_gKernel_XZ_tracking", "or_gKernel_YZ_tracking",
           "or_gKernel_BackTrackCleaning", "or_gKernel_Global_tracking", "or_dropin_sync", "or_yz_scored",
           "or_outer_labels", "or_run_batch_scored")

# tunable kernels (or_kernel_id_t)
KERNELS = {"event_reduce": 0, "xz": 1, "yz": 2, "back_clean": 3, "global": 4, "select": 5, "features": 6}

OR_YZ_NOALLOC_MAX_EVENTS = 10000
OR_ERRW_CAPACITY = 2


class OrError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


_lib = None


def lib():
    """Load liborgpu.so (built by build_lib.build()); raise if it is absent."""
    global _lib
    if _lib is None:
        _lib = load(LIB_PATH)
    return _lib


def load(path):
    """Load a build of the library at `path` with the C-ABI signatures set
    (lib() is load(LIB_PATH), once per process)."""
    if not os.path.exists(path):
        raise OrError(-1, f"liborgpu.so not built at {path}; run __graft_entry__.build()")
    lb = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    lb.or_version.restype = C.c_char_p
    lb.or_last_error.restype = C.c_char_p
    lb.or_status_string.restype = C.c_char_p
    lb.or_status_string.argtypes = [C.c_int]
    lb.or_geometry_load.argtypes = [C.c_char_p, P(L.OrPlane), vp]
    lb.or_create.argtypes = [C.c_int, P(vp)]
    lb.or_create_sized.argtypes = [C.c_int, C.c_int, P(vp)]
    lb.or_context_bytes.argtypes = [C.c_int, C.c_int]
    lb.or_context_bytes.restype = C.c_size_t
    lb.or_destroy.argtypes = [vp]
    lb.or_set_geometry.argtypes = [vp, P(L.OrPlane)]
    lb.or_stream_sync.argtypes = [vp, vp]
    lb.or_event_reduce.argtypes = [vp, L.OrHitsView, vp, C.c_int, vp]
    lb.or_xz.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, vp, C.c_int, vp]
    lb.or_yz.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, C.c_int, vp]
    lb.or_back_clean.argtypes = [vp, L.OrTracksView, vp, C.c_int, vp]
    lb.or_global.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, C.c_int, vp]
    lb.or_run_batch.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, vp, C.c_int, vp]
    lb.or_hits_view_from_collection.argtypes = [vp]
    lb.or_hits_view_from_collection.restype = L.OrHitsView
    lb.or_tracks_view_from_collection.argtypes = [vp]
    lb.or_tracks_view_from_collection.restype = L.OrTracksView
    lb.or_hits_view_bytes.argtypes = [C.c_int]
    lb.or_hits_view_bytes.restype = C.c_size_t
    lb.or_tracks_view_bytes.argtypes = [C.c_int]
    lb.or_tracks_view_bytes.restype = C.c_size_t
    lb.or_pack_hits.argtypes = [vp, vp, vp, C.c_int, vp, L.OrHitsView, vp]
    lb.or_collect_tracks.argtypes = [vp, L.OrTracksView, vp, C.c_int, C.c_float, vp, C.c_int64, vp, vp]
    lb.or_yz_noalloc.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, C.c_int, vp, vp]
    lb.or_selftest_bounded_wait.argtypes = [vp, C.c_int, vp]
    lb.or_yz_work_counts.argtypes = [vp, vp]
    lb.or_set_yz_work_counting.argtypes = [vp, C.c_int]
    # include/or_dropin.h: the reference's launches on its own structs
    lb.or_gkernel_eR.argtypes = [vp, vp]
    lb.or_gKernel_XZ_tracking.argtypes = [vp, vp, vp, vp, vp]
    lb.or_gKernel_YZ_tracking.argtypes = [vp, vp, vp, vp]
    lb.or_gKernel_BackTrackCleaning.argtypes = [vp, vp]
    lb.or_gKernel_Global_tracking.argtypes = [vp, vp, vp, vp]
    lb.or_dropin_sync.argtypes = []
    lb.or_yz_scored.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, C.c_int, vp, C.c_float, C.c_float, vp, vp, vp,
                                vp, vp, C.c_int64, vp]
    lb.or_outer_labels.argtypes = [vp, L.OrTracksView, vp, vp, vp, C.c_int64, vp, vp]
    lb.or_run_batch_scored.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, vp, C.c_int, vp, C.c_float, C.c_float,
                                       vp, vp, vp, vp, vp, C.c_int64, vp]
    i64, f32, i32 = C.c_int64, C.c_float, C.c_int
    lb.or_tracklet_rows.argtypes = [vp, L.OrTracksView, vp, i32, vp, vp]
    lb.or_tracklet_features.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, i32, vp, vp, i64, vp]
    lb.or_mlp_score.argtypes = [vp, vp, vp, i64, vp, vp]
    lb.or_keep_mask.argtypes = [vp, vp, vp, i32, f32, f32, vp, i64, vp]
    lb.or_yz_pruned.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, i32, vp, vp, i64, vp]
    lb.or_run_batch_learned.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, vp, i32, vp, f32, f32, vp, vp, vp, vp,
                                        i64, vp]
    lb.or_tracklet_labels.argtypes = [vp, L.OrTracksView, vp, i32, vp, vp, i64, vp]
    lb.or_track_agreement.argtypes = [vp, L.OrTracksView, L.OrTracksView, vp, i32, vp, vp]
    lb.or_mlp_grad_blocks.argtypes = [i32]
    lb.or_mlp_forward.argtypes = [vp, vp, vp, vp, i32, vp, vp]
    lb.or_mlp_gradient.argtypes = [vp, vp, vp, vp, vp, i32, f32, vp, vp, vp]
    lb.or_mlp_adam.argtypes = [vp, vp, vp, vp, vp, i32, i32, f32, f32, f32, f32, vp, vp]
    lb.or_set_launch.argtypes = [vp, i32, i32]
    lb.or_get_launch.argtypes = [vp, i32]
    lb.or_prop_matching.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, i32, vp]
    lb.or_global_clean.argtypes = [vp, L.OrTracksView, vp, i32, vp]
    lb.or_run_selection.argtypes = [vp, L.OrHitsView, L.OrTracksView, vp, i32, vp]
    lb.or_vertexing.argtypes = [vp, L.OrTracksView, vp, i32, vp]
    lb.or_dimuons.argtypes = [vp, L.OrTracksView, L.OrDimuonsView, vp, i32, vp]
    lb.or_fill_histograms.argtypes = [vp, L.OrTracksView, L.OrDimuonsView, vp, vp, vp, i32, vp]
    lb.or_hist_table_init.argtypes = [C.POINTER(L.OrHists)]
    lb.or_hist_table_init.restype = None
    lb.or_run_physics.argtypes = [vp, L.OrTracksView, L.OrDimuonsView, vp, vp, vp, i32, vp]
    lb.or_output_rows.argtypes = [vp, L.OrHitsView, L.OrTracksView, L.OrDimuonsView, vp, vp, vp, f32, L.OrOutputView,
                                  i32, vp]
    lb.or_rt_load.argtypes = [C.c_char_p, P(L.OrPlane), P(L.OrRtTable), P(C.c_int)]
    lb.or_rt_set_plane.argtypes = [P(L.OrRtTable), i32, i32, vp, vp, f32, f32, f32]
    lb.or_rt_table_bytes.argtypes = []
    lb.or_rt_table_bytes.restype = C.c_size_t
    lb.or_pack_hits_rt.argtypes = [vp, vp, vp, i32, vp, vp, L.OrHitsView, vp]
    lb.or_rt_apply.argtypes = [vp, vp, L.OrHitsView, i32, vp]
    lb.or_set_yz_pool_limit.argtypes = [vp, i64]
    for name in EXPORTS:
        getattr(lb, name)
    return lb


def check(rc, what="call"):
    if rc != OR_OK:
        raise OrError(rc, f"{what} failed: {lib().or_status_string(rc).decode()}: {lib().or_last_error().decode()}")


def geometry_load(path):
    """Parse a geometry table with the library's loader -> (OrPlane, wire_pos[55,400])."""
    import numpy as np
    p = L.OrPlane()
    wp = np.zeros(L.NDET * L.WIREPOS_STRIDE, np.float64)
    check(lib().or_geometry_load(str(path).encode(), C.byref(p), wp.ctypes.data), "or_geometry_load")
    return p, wp.reshape(L.NDET, L.WIREPOS_STRIDE)


def rt_load(path, plane):
    """Parse an R-T calibration file with the library's loader -> (OrRtTable,
    number of planes with a profile).  `plane` supplies the cell widths."""
    rt = L.OrRtTable()
    n = C.c_int(0)
    check(lib().or_rt_load(str(path).encode(), C.byref(plane), C.byref(rt), C.byref(n)), "or_rt_load")
    return rt, n.value
