"""The learned tracklet scorer on the GPU, against the CPU oracle.

- tracklet rows and features: the C restatement (orc_tracklet_features);
- training gradients: the float64 oracle with the same BF16 rounding points
  (oracle/mlp_oracle.py);
- tensor-core scores (tcgen05): the same oracle's forward pass and the CUDA-
  core forward of the training kernel;
- pruned YZ: kept tracklets get the plain result bit for bit, pruned ones
  are left as tracklets no combination extends.
"""
import numpy as np
import pytest

from helpers import Snapshots, mixed_events, track_mismatches

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(geometry):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orgpu import learned, pipeline
    plane, wp = geometry
    geo, rec, off, hits0 = mixed_events(plane, wp, 150, 150, seed=31)
    snap = Snapshots(plane, hits0)
    rc = pipeline.Reconstruction(plane, 0)
    return plane, hits0, snap, rc, learned.Learned(rc)


def _xz_batch(env):
    import torch
    from orgpu import pipeline
    plane, hits0, snap, rc, lr = env
    b = pipeline.DeviceBatch(hits0.n, 0)
    b.upload_hits(snap.hits_er)
    b.toomany.copy_(torch.from_numpy(snap.toomany_xz))
    b.upload_tracks(snap.tracks_xz)
    return b


def test_rows_and_features_match_oracle(env):
    from oracle import pyoracle as O
    from orgpu import learned
    plane, hits0, snap, rc, lr = env
    b = _xz_batch(env)
    r = learned.TrackletRows(b.n)
    lr.rows(b, r)
    lr.features(b, r)
    rc.sync()
    ro, f = O.tracklet_features(plane, snap.hits_er, snap.tracks_xz, snap.toomany_xz)
    np.testing.assert_array_equal(r.row_off.cpu().numpy(), ro)
    n = int(ro[-1])
    assert n > 100
    got = r.features.cpu().numpy()[:n * 16].reshape(n, 16)
    # identical arithmetic except log1pf, which may differ in the last bit
    np.testing.assert_allclose(got, f, rtol=2e-7, atol=0)


def _random_model(seed):
    from orgpu import learned
    rng = np.random.default_rng(seed)
    sp = learned.ScorerParams.init(rng.normal(0, 1, 16).astype(np.float32),
                                   rng.uniform(0.5, 2, 16).astype(np.float32), seed=seed)
    sp.params[learned.P_B1:learned.P_W2] = rng.normal(0, 0.1, 64)
    sp.params[learned.P_B2:learned.P_W3] = rng.normal(0, 0.1, 64)
    return sp


def test_gradient_matches_cpu_oracle(env):
    import torch
    from oracle import mlp_oracle as M
    from orgpu import learned
    plane, hits0, snap, rc, lr = env
    sp = _random_model(3)
    rng = np.random.default_rng(4)
    n = 1000
    X = rng.normal(0, 1.5, (n, 16)).astype(np.float32)
    y = (rng.random(n) < 0.2).astype(np.uint8)
    model = learned.DeviceModel(sp)
    fx = torch.from_numpy(X.reshape(-1)).cuda()
    fy = torch.from_numpy(y).cuda()
    idx = torch.arange(n, dtype=torch.int64, device="cuda")
    nblk = lr.lib.or_mlp_grad_blocks(n)
    grad = torch.zeros(nblk * learned.NP, dtype=torch.float32, device="cuda")
    loss = torch.zeros(nblk, dtype=torch.float32, device="cuda")
    from orgpu import _lib
    _lib.check(lr.lib.or_mlp_gradient(rc.ctx, model.ptr(), fx.data_ptr(), fy.data_ptr(), idx.data_ptr(), n, 3.0,
                                      grad.data_ptr(), loss.data_ptr(), None), "or_mlp_gradient")
    rc.sync()
    g_gpu = grad.cpu().numpy().reshape(nblk, -1).sum(0)
    g_ref, l_ref = M.gradient(sp.params, sp.mean, sp.inv_std, X, y, 3.0)
    assert abs(float(loss.sum()) - l_ref) < 1e-5 * max(1.0, abs(l_ref))
    scale = np.abs(g_ref).max()
    np.testing.assert_allclose(g_gpu, g_ref, rtol=0, atol=2e-5 * scale)


def test_tensor_core_scores_match_oracle(env):
    import torch
    from oracle import mlp_oracle as M
    from orgpu import _lib, learned
    plane, hits0, snap, rc, lr = env
    sp = _random_model(5)
    rng = np.random.default_rng(6)
    n = 128 * 37 + 11  # ragged last tile
    X = rng.normal(0, 1.5, (n, 16)).astype(np.float32)
    model = learned.DeviceModel(sp)
    fx = torch.from_numpy(X.reshape(-1)).cuda()
    out = torch.full((n + 5,), -1.0, dtype=torch.float32, device="cuda")
    lr.score(model, fx, n, out)
    prob = torch.zeros(n, dtype=torch.float32, device="cuda")
    idx = torch.arange(n, dtype=torch.int64, device="cuda")
    _lib.check(lr.lib.or_mlp_forward(rc.ctx, model.ptr(), fx.data_ptr(), idx.data_ptr(), n, prob.data_ptr(), None),
               "or_mlp_forward")
    rc.sync()
    s_tc = out.cpu().numpy()
    assert np.all(s_tc[n:] == -1.0)  # nothing written past the last row
    p_ref, _ = M.forward(sp.params, sp.mean, sp.inv_std, X)
    # FP32 sums in different orders; a BF16 rounding of h1 may flip in rare rows
    assert np.quantile(np.abs(s_tc[:n] - p_ref), 0.999) < 1e-4
    assert np.abs(s_tc[:n] - p_ref).max() < 2e-2
    assert np.quantile(np.abs(s_tc[:n] - prob.cpu().numpy()), 0.999) < 1e-4


def test_pruned_yz_keeps_plain_results(env):
    import torch
    from orgpu import learned
    plane, hits0, snap, rc, lr = env
    # all kept: identical to plain YZ
    b = _xz_batch(env)
    r = learned.TrackletRows(b.n)
    lr.rows(b, r)
    r.keep.fill_(1)
    lr.yz_pruned(b, r)
    rc.sync()
    assert track_mismatches(b.download_tracks(), snap.tracks_yz, snap.toomany_xz) == []
    # random half pruned
    b = _xz_batch(env)
    lr.rows(b, r)
    nrows = r.n_rows()
    keep = (np.random.default_rng(7).random(r.max_rows) < 0.5).astype(np.uint8)
    r.keep.copy_(torch.from_numpy(keep))
    lr.yz_pruned(b, r)
    rc.sync()
    got = b.download_tracks()
    ro = r.row_off.cpu().numpy()
    from orgpu import layout as Lt
    checked_kept = checked_pruned = 0
    for e in range(b.n):
        if snap.toomany_xz[e]:
            continue
        row = int(ro[e])
        for s in range(Lt.NSLOTS):
            for k in range(int(snap.tracks_xz.ntracks[e * 32 + s])):
                base = e * Lt.EVT_TRK_FLOATS + (s * 16 + k) * Lt.NTRKPARAM
                g = got.tracks[base:base + Lt.NTRKPARAM].view(np.uint32)
                if keep[row]:
                    w = snap.tracks_yz.tracks[base:base + Lt.NTRKPARAM].view(np.uint32)
                    checked_kept += 1
                else:
                    w = snap.tracks_xz.tracks[base:base + Lt.NTRKPARAM].copy()
                    w[Lt.TRK_STID] = 3.0
                    w = w.view(np.uint32)
                    checked_pruned += 1
                assert np.array_equal(g, w), (e, s, k, bool(keep[row]))
                row += 1
    assert row <= nrows + 1 and checked_kept > 50 and checked_pruned > 50


def test_training_reduces_loss(env):
    import torch
    from orgpu import learned
    plane, hits0, snap, rc, lr = env
    rng = np.random.default_rng(9)
    n = 8192 * 4
    X = rng.normal(0, 1, (n, 16)).astype(np.float32)
    y = ((X[:, 0] + 0.5 * X[:, 3] - 0.3 * X[:, 7]) > 1.0).astype(np.uint8)
    sp = learned.ScorerParams.init(np.zeros(16, np.float32), np.ones(16, np.float32), seed=1)
    tr = learned.Trainer(lr, sp, torch.from_numpy(X.reshape(-1)).cuda(), torch.from_numpy(y).cuda(), batch=4096,
                         lr=3e-3, pos_weight=1.0)
    first = tr.epoch(rng)
    for _ in range(6):
        last = tr.epoch(rng)
    assert last < 0.5 * first
    res = tr.result()
    from oracle import mlp_oracle as M
    p, _ = M.forward(res.params, res.mean, res.inv_std, X[:4096])
    acc = np.mean((p > 0.5) == (y[:4096] == 1))
    assert acc > 0.95


def _plain_and_learned(env, sp, n, seed, cfg_name="small"):
    import torch
    from orgpu import learned, pipeline, synth as S
    plane, hits0, snap, rc, lr = env
    from oracle import pyoracle as O
    from orgpu import GEOMETRY_E906
    _, wp = O.parse_geometry(GEOMETRY_E906)
    geo = S.Geometry(plane, wp)
    cfg = S.config_small(n, seed) if cfg_name == "small" else S.config_uneven(n, seed)
    rec, off, _ = S.generate(geo, cfg)
    rec, off = S.cap_records(rec, off)
    h = S.pack(rec, off, geo.wire_pos_f32())
    bp = pipeline.DeviceBatch(n)
    bl = pipeline.DeviceBatch(n)
    bp.upload_hits(h)
    bl.upload_hits(h)
    rc.run_batch(bp)
    r = learned.TrackletRows(n)
    lr.run_batch(bl, r, learned.DeviceModel(sp), sp.t_keep, sp.t_unc)
    rc.sync()
    return lr.agreement(bp, bl), r


def test_learned_batch_keep_all_equals_plain(env):
    from orgpu import learned
    sp = learned.ScorerParams.load()
    sp.t_keep = sp.t_unc = 0.0  # every score >= 0: nothing pruned
    (n_ref, n_match, n_new), r = _plain_and_learned(env, sp, 600, 77)
    assert n_ref > 300 and n_match == n_ref == n_new
    assert int(r.keep[:r.n_rows()].sum()) == r.n_rows()


def test_committed_scorer_recall_small_events(env):
    """The committed model at its own threshold keeps >= 99.5 % of the plain
    global tracks of one-dimuon events (held-out seed)."""
    from orgpu import learned
    sp = learned.ScorerParams.load()
    (n_ref, n_match, n_new), r = _plain_and_learned(env, sp, 3000, 424242)
    assert n_ref > 2000
    assert n_match / n_ref >= 0.995
    assert int(r.keep[:r.n_rows()].sum()) < r.n_rows()  # something was pruned
