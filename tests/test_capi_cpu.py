"""The C-ABI library without a GPU: it loads, exports every function that
include/*.h declares, and its host-side argument checks return the
documented status codes before any CUDA call."""
import ctypes as C
import os
import re

from conftest import REPO


def _declared_functions():
    names = set()
    for h in ("or_gb300.h", "or_layout.h", "or_dropin.h"):
        text = open(os.path.join(REPO, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^[A-Za-z_][\w \*]*?\b(or_\w+)\s*\(", text, flags=re.M))
    return names


def test_library_exports_every_declared_function():
    from orgpu import _lib
    lb = _lib.lib()
    declared = _declared_functions()
    assert "or_run_batch" in declared and "or_yz_noalloc" in declared and "or_gKernel_YZ_tracking" in declared
    assert declared == set(_lib.EXPORTS)
    for name in declared:
        getattr(lb, name)


def test_status_strings_and_version():
    from orgpu import _lib
    lb = _lib.lib()
    assert b"sm_103a" in lb.or_version()
    assert lb.or_status_string(_lib.OR_ERR_CAPACITY) == b"capacity exceeded"
    assert lb.or_status_string(99) == b"unknown status"


def test_host_argument_checks():
    from orgpu import _lib, layout as L
    lb = _lib.lib()
    assert lb.or_create(0, None) == _lib.OR_ERR_ARG
    assert lb.or_destroy(None) == _lib.OR_OK
    assert lb.or_yz(None, L.OrHitsView(), L.OrTracksView(), None, 1, None) == _lib.OR_ERR_ARG
    assert b"null context" in lb.or_last_error()
    assert lb.or_geometry_load(b"/nonexistent/geometry.txt", C.byref(L.OrPlane()), None) == _lib.OR_ERR_IO


def test_collection_views_follow_reference_layout():
    from orgpu import _lib, layout as L
    lb = _lib.lib()
    base = 1 << 40
    v = lb.or_hits_view_from_collection(base)
    E = L.REF_EVTMAX
    assert v.nhits_cham == base
    assert v.hits_cham == base + 4 * E * L.NCHAM
    assert v.nhits_hodo == v.hits_cham + 4 * E * L.EVT_CHAM_FLOATS
    assert v.hits_prop == v.nhits_prop + 4 * E * L.NPROP
    t = lb.or_tracks_view_from_collection(base)
    assert t.tracks == base + 2 * E * L.NSLOTS
    assert lb.or_hits_view_bytes(3) == 3 * (4 * (L.NCHAM + L.NHODO + L.NPROP) + 4 * (
        L.EVT_CHAM_FLOATS + L.EVT_HODO_FLOATS + L.EVT_PROP_FLOATS))


def test_context_bytes_scale_with_the_largest_batch():
    """or_context_bytes: what or_create_sized(max_events) allocates on a
    152-SM GB300 -- the 100,000-event default (0) about 10.8 GB, a 10,000-event
    slot under 2 GB, growing with max_events, 0 for invalid arguments; and
    or_create_sized checks its arguments before touching a device."""
    from orgpu import _lib
    lb = _lib.lib()
    full = lb.or_context_bytes(0, 152)
    assert 10.0e9 < full < 11.5e9
    assert lb.or_context_bytes(100000, 152) == full == lb.or_context_bytes(250000, 152)
    slot = lb.or_context_bytes(10000, 152)
    assert 0.5e9 < slot < 2.0e9
    assert lb.or_context_bytes(1000, 152) <= slot <= lb.or_context_bytes(50000, 152) < full
    assert lb.or_context_bytes(-1, 152) == 0 and lb.or_context_bytes(10000, 0) == 0
    ctx = C.c_void_p()
    assert lb.or_create_sized(0, -5, C.byref(ctx)) == _lib.OR_ERR_ARG
    assert lb.or_create_sized(0, 10000, None) == _lib.OR_ERR_ARG


def test_serving_slot_bytes_use_a_sized_context():
    """A serving slot of 10,000 events is admitted by its real footprint: its
    batch buffers plus a context sized for 10,000 events, not the 100,000-
    event default."""
    from orgpu import _lib, layout as L
    from orgpu.serving import Server
    lb = _lib.lib()
    cap, rec = 10000, 400
    base = (lb.or_hits_view_bytes(cap) + lb.or_tracks_view_bytes(cap) + cap * rec * 16 +
            4 * cap * L.COLLECT_STRIDE * 4)
    assert Server.slot_bytes(cap, rec, False, 152) == base + lb.or_context_bytes(cap, 152)
    assert Server.slot_bytes(cap, rec, True, 152) > Server.slot_bytes(cap, rec, False, 152)
    assert Server.slot_bytes(cap, rec, False, 152) < base + lb.or_context_bytes(0, 152) - 5e9
