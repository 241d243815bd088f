"""The continuous-batching server: every request's result is the same when it
runs alone and when it shares slots with others, and equals a direct
or_run_batch of its events; graphs and eager launches agree."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import synth as S
    plane, wp = geometry
    geo = S.Geometry(plane, wp)
    rec, off, _ = S.generate(geo, S.config_small(3000, 5151))
    rec, off = S.cap_records(rec, off)
    return plane, wp, geo, rec, off


def _requests(rec, off, sizes):
    out, e = [], 0
    for n in sizes:
        r0, r1 = off[e], off[e + n]
        out.append((rec[r0:r1], (off[e:e + n + 1] - r0).astype(np.int64)))
        e += n
    return out


def _direct(plane, wp, geo, rec, off):
    """Track rows of a plain run_batch + collect of the events."""
    import torch
    from orgpu import layout as L, pipeline
    n = len(off) - 1
    rc = pipeline.Reconstruction(plane, 0)
    b = pipeline.DeviceBatch(n)
    rc.pack(b, torch.from_numpy(rec.view(np.uint8)).cuda(), torch.from_numpy(off).cuda(),
            torch.from_numpy(geo.wire_pos_f32().reshape(-1)).cuda())
    rc.run_batch(b)
    out = torch.zeros(4 * n * L.COLLECT_STRIDE, dtype=torch.float32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc.collect(b, out, cnt, 6.0)
    rc.sync()
    k = int(cnt.item())
    r = out[:k * L.COLLECT_STRIDE].cpu().numpy().reshape(k, L.COLLECT_STRIDE)
    return r[np.lexsort((r[:, 1], r[:, 0]))]


@pytest.mark.parametrize("graphs", [True, False])
def test_alone_and_in_the_mix_agree(env, graphs):
    from orgpu import serving
    plane, wp, geo, rec, off = env
    sizes = [700, 1, 1500, 37, 300, 462]
    reqs = _requests(rec, off, sizes)
    srv = serving.Server(plane, wp, slot_events=1024, max_slots=3, rec_per_event=600, graphs=graphs,
                         reserve_bytes=1 << 30)
    assert len(srv.slots) >= 2
    alone = []
    for r, o in reqs:
        q = srv.submit(r, o)
        srv.drain()
        alone.append(q)
    mixed = [srv.submit(r, o) for r, o in reqs]
    srv.drain()
    for a, m, (r, o) in zip(alone, mixed, reqs):
        ra, rm = a.result(), m.result()
        assert ra.shape == rm.shape
        assert np.array_equal(ra.view(np.uint32), rm.view(np.uint32))
        np.testing.assert_array_equal(a.flags, m.flags)
        rd = _direct(plane, wp, geo, r, o)
        assert np.array_equal(ra.view(np.uint32), rd.view(np.uint32))
    assert sum(len(q.result()) for q in mixed) > 1000


def test_schedule_reports_latency(env):
    from orgpu import serving
    plane, wp, geo, rec, off = env
    reqs = _requests(rec, off, [200] * 10)
    srv = serving.Server(plane, wp, slot_events=1024, max_slots=2, rec_per_event=600, reserve_bytes=1 << 30)
    done = srv.serve([(0.002 * i, r, o) for i, (r, o) in enumerate(reqs)])
    st = serving.latency_stats(done)
    assert st["requests"] == 10 and st["events"] == 2000
    assert 0 < st["p50_ms"] <= st["p99_ms"]
