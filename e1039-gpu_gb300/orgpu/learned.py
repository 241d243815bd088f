"""The learned tracklet scorer around the plain path.

A 16-64-64-1 MLP (BF16 weights and activations, FP32 sums, sigmoid) scores
every XZ tracklet from 16 features (or_tracklet_features); the YZ
combinatorics of tracklets scoring below a threshold are skipped
(or_yz_pruned), everything else is the plain path, so every kept tracklet
gets the plain result bit for bit and the plain method stays the arbiter:
recall = share of the plain run's global tracks that the learned run
reproduces exactly (or_track_agreement).

Labels come from the plain method itself: a tracklet is positive when it
ended as a global track (stationID 6).  Training runs on the GPU through the
library's own kernels (or_mlp_gradient: forward + backward, or_mlp_adam);
inference runs on the tensor cores (or_mlp_score).  PyTorch only holds the
device buffers.
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from . import layout as L

NF, H, NP = L.NFEAT, L.MLP_H, L.MLP_NPARAM
# offsets in the FP32 parameter vector (w1, b1, w2, b2, w3, b3)
P_W1, P_B1 = 0, H * NF
P_W2 = P_B1 + H
P_B2 = P_W2 + H * H
P_W3 = P_B2 + H
P_B3 = P_W3 + H

MODEL_E906 = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data", "scorer_e906.npz")


def bf16_bits(x):
    """float32 -> BF16 bits, round to nearest even (what __float2bfloat16_rn does)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    nan = np.isnan(np.asarray(x, np.float32))
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    r[nan] = 0x7FC0
    return r


def bf16_round(x):
    return (bf16_bits(x).astype(np.uint32) << 16).view(np.float32)


def split(params):
    """FP32 parameter vector -> (w1[64,16], b1, w2[64,64], b2, w3, b3)."""
    p = np.asarray(params, np.float32)
    return (p[P_W1:P_B1].reshape(H, NF), p[P_B1:P_W2], p[P_W2:P_B2].reshape(H, H), p[P_B2:P_W3], p[P_W3:P_B3],
            float(p[P_B3]))


class ScorerParams:
    """Host copy of a scorer: FP32 parameters, input normalisation, and the
    thresholds of the keep rule."""

    def __init__(self, params, mean, inv_std, t_keep=0.5, t_unc=0.5, meta=None):
        self.params = np.asarray(params, np.float32).copy()
        self.mean = np.asarray(mean, np.float32).copy()
        self.inv_std = np.asarray(inv_std, np.float32).copy()
        self.t_keep = float(t_keep)
        self.t_unc = float(t_unc)
        self.meta = dict(meta or {})

    @classmethod
    def init(cls, mean, inv_std, seed=0):
        """He-normal hidden layers, small output layer, zero biases."""
        rng = np.random.default_rng(seed)
        p = np.zeros(NP, np.float32)
        p[P_W1:P_B1] = rng.normal(0, np.sqrt(2.0 / NF), H * NF)
        p[P_W2:P_B2] = rng.normal(0, np.sqrt(2.0 / H), H * H)
        p[P_W3:P_B3] = rng.normal(0, np.sqrt(1.0 / H), H)
        return cls(p, mean, inv_std)

    def to_struct(self):
        w1, b1, w2, b2, w3, b3 = split(self.params)
        m = L.OrMlp()
        m.mean[:] = self.mean.tolist()
        m.inv_std[:] = self.inv_std.tolist()
        m.w1[:] = bf16_bits(w1.reshape(-1)).tolist()
        m.b1[:] = b1.tolist()
        m.w2[:] = bf16_bits(w2.reshape(-1)).tolist()
        m.b2[:] = b2.tolist()
        m.w3[:] = w3.tolist()
        m.b3 = b3
        return m

    def save(self, path):
        np.savez(path, params=self.params, mean=self.mean, inv_std=self.inv_std, t_keep=self.t_keep,
                 t_unc=self.t_unc, meta=np.array(repr(self.meta)))

    @classmethod
    def load(cls, path=MODEL_E906):
        z = np.load(path)
        meta = {}
        if "meta" in z:
            try:
                import ast
                meta = ast.literal_eval(str(z["meta"]))
            except (ValueError, SyntaxError):
                meta = {}
        return cls(z["params"], z["mean"], z["inv_std"], float(z["t_keep"]), float(z["t_unc"]), meta)


def _torch():
    import torch
    return torch


class DeviceModel:
    """An or_mlp_t in device memory."""

    def __init__(self, sp, device=0):
        torch = _torch()
        self.bytes = torch.zeros(C.sizeof(L.OrMlp), dtype=torch.uint8, device=torch.device("cuda", device))
        self.load(sp)

    def load(self, sp):
        torch = _torch()
        s = sp.to_struct()
        raw = bytearray(C.string_at(C.addressof(s), C.sizeof(s)))
        self.bytes.copy_(torch.frombuffer(raw, dtype=torch.uint8))

    def ptr(self):
        return self.bytes.data_ptr()


class TrackletRows:
    """Row buffers of one batch: offsets, features, scores, keep flags,
    labels.  `max_rows` caps the rows; rows past it are always kept."""

    def __init__(self, n_events, max_rows=None, device=0):
        torch = _torch()
        dev = torch.device("cuda", device)
        self.n = n_events
        self.max_rows = int(max_rows if max_rows is not None else max(1024, 64 * n_events))
        self.row_off = torch.zeros(n_events + 1, dtype=torch.int32, device=dev)
        self.features = torch.zeros(self.max_rows * NF, dtype=torch.float32, device=dev)
        self.scores = torch.zeros(self.max_rows, dtype=torch.float32, device=dev)
        self.keep = torch.ones(self.max_rows, dtype=torch.uint8, device=dev)
        self.labels = torch.zeros(self.max_rows, dtype=torch.uint8, device=dev)

    def n_rows(self):
        return min(int(self.row_off[self.n].item()), self.max_rows)


class Learned:
    """Learned-path calls on a pipeline.Reconstruction context."""

    def __init__(self, rc):
        self.rc = rc
        self.lib = rc.lib

    def rows(self, b, r, stream=None):
        _lib.check(self.lib.or_tracklet_rows(self.rc.ctx, b.tracks_view(), b.toomany.data_ptr(), b.n,
                                             r.row_off.data_ptr(), self.rc._stream(stream)), "or_tracklet_rows")

    def features(self, b, r, stream=None):
        _lib.check(self.lib.or_tracklet_features(self.rc.ctx, b.hits_view(), b.tracks_view(), b.toomany.data_ptr(),
                                                 b.n, r.row_off.data_ptr(), r.features.data_ptr(), r.max_rows,
                                                 self.rc._stream(stream)), "or_tracklet_features")

    def score(self, model, features, n_rows, scores, stream=None):
        _lib.check(self.lib.or_mlp_score(self.rc.ctx, model.ptr(), features.data_ptr(), int(n_rows),
                                         scores.data_ptr(), self.rc._stream(stream)), "or_mlp_score")

    def keep(self, r, t_keep, t_unc, stream=None):
        _lib.check(self.lib.or_keep_mask(self.rc.ctx, r.scores.data_ptr(), r.row_off.data_ptr(), r.n, float(t_keep),
                                         float(t_unc), r.keep.data_ptr(), r.max_rows, self.rc._stream(stream)),
                   "or_keep_mask")

    def yz_pruned(self, b, r, stream=None):
        _lib.check(self.lib.or_yz_pruned(self.rc.ctx, b.hits_view(), b.tracks_view(), b.toomany.data_ptr(), b.n,
                                         r.row_off.data_ptr(), r.keep.data_ptr(), r.max_rows,
                                         self.rc._stream(stream)), "or_yz_pruned")

    def labels(self, b, r, stream=None):
        _lib.check(self.lib.or_tracklet_labels(self.rc.ctx, b.tracks_view(), b.toomany.data_ptr(), b.n,
                                               r.row_off.data_ptr(), r.labels.data_ptr(), r.max_rows,
                                               self.rc._stream(stream)), "or_tracklet_labels")

    def run_batch(self, b, r, model, t_keep, t_unc, stream=None):
        """The whole learned path in one call (or_run_batch_learned)."""
        _lib.check(self.lib.or_run_batch_learned(self.rc.ctx, b.hits_view(), b.tracks_view(), b.ntracklets.data_ptr(),
                                                 b.toomany.data_ptr(), b.n, model.ptr(), float(t_keep), float(t_unc),
                                                 r.row_off.data_ptr(), r.features.data_ptr(), r.scores.data_ptr(),
                                                 r.keep.data_ptr(), r.max_rows, self.rc._stream(stream)),
                   "or_run_batch_learned")

    def agreement(self, b_ref, b_new, stream=None):
        """(global tracks of the reference run, of those reproduced exactly,
        global tracks of the new run)."""
        torch = _torch()
        cnt = torch.zeros(3, dtype=torch.int64, device=b_ref.toomany.device)
        _lib.check(self.lib.or_track_agreement(self.rc.ctx, b_ref.tracks_view(), b_new.tracks_view(),
                                               b_ref.toomany.data_ptr(), b_ref.n, cnt.data_ptr(),
                                               self.rc._stream(stream)), "or_track_agreement")
        return tuple(int(x) for x in cnt.cpu().tolist())

    def plain_with_rows(self, b, r, stream=None):
        """Plain chain, with the tracklet rows, features (after XZ) and labels
        (after global tracking) of the batch: the training data."""
        rc = self.rc
        b.ntracklets.zero_()
        rc.event_reduce(b, stream)
        rc.xz_tracking(b, stream)
        self.rows(b, r, stream)
        self.features(b, r, stream)
        rc.yz_tracking(b, stream)
        rc.back_track_cleaning(b, stream)
        rc.global_tracking(b, stream)
        self.labels(b, r, stream)


class Trainer:
    """Mini-batch Adam on the GPU through or_mlp_gradient / or_mlp_adam."""

    def __init__(self, learned, sp, features, labels, batch=8192, lr=1e-3, pos_weight=4.0, device=0):
        torch = _torch()
        self.lib = learned.lib
        self.ctx = learned.rc.ctx
        self.stream = learned.rc._stream(None)
        dev = torch.device("cuda", device)
        self.sp = sp
        self.model = DeviceModel(sp, device)
        self.param = torch.from_numpy(sp.params.copy()).to(dev)
        self.m1 = torch.zeros(NP, dtype=torch.float32, device=dev)
        self.m2 = torch.zeros(NP, dtype=torch.float32, device=dev)
        self.features = features
        self.labels = labels
        self.n = labels.numel()
        self.batch = batch
        self.lr = lr
        self.pos_weight = pos_weight
        self.nblk = self.lib.or_mlp_grad_blocks(batch)
        self.grad = torch.zeros(self.nblk * NP, dtype=torch.float32, device=dev)
        self.loss = torch.zeros(self.nblk, dtype=torch.float32, device=dev)
        self.step_no = 0
        self.dev = dev

    def epoch(self, rng):
        """One pass over the rows in a random order; returns the mean batch loss."""
        torch = _torch()
        perm = torch.from_numpy(rng.permutation(self.n).astype(np.int64)).to(self.dev)
        total = torch.zeros((), dtype=torch.float32, device=self.dev)
        nb = 0
        for s in range(0, self.n - self.batch + 1, self.batch):
            idx = perm[s:s + self.batch]
            _lib.check(self.lib.or_mlp_gradient(self.ctx, self.model.ptr(), self.features.data_ptr(),
                                                self.labels.data_ptr(), idx.data_ptr(), self.batch,
                                                float(self.pos_weight), self.grad.data_ptr(), self.loss.data_ptr(),
                                                self.stream), "or_mlp_gradient")
            self.step_no += 1
            _lib.check(self.lib.or_mlp_adam(self.ctx, self.param.data_ptr(), self.m1.data_ptr(), self.m2.data_ptr(),
                                            self.grad.data_ptr(), self.nblk, self.step_no, float(self.lr), 0.9, 0.999,
                                            1e-8, self.model.ptr(), self.stream), "or_mlp_adam")
            total += self.loss.sum()
            nb += 1
        return float(total.item()) / max(nb, 1)

    def result(self):
        return ScorerParams(self.param.cpu().numpy(), self.sp.mean, self.sp.inv_std, self.sp.t_keep, self.sp.t_unc,
                            self.sp.meta)


# ---------------------------------------------------------------------------
# The combination scorer: one row per live (u3, v3) outer iteration of every
# tracklet the YZ stage queues (or_yz_scored)
# ---------------------------------------------------------------------------
MODEL_COMBO_E906 = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data",
                                "combo_scorer_e906.npz")


class OuterRows:
    """Device buffers of the combination scorer for one batch: features,
    outer indices, scores, labels, the row counter and the uncertain-event
    flags.  `max_rows` caps the rows; tracklets past it are not pruned."""

    def __init__(self, n_events, max_rows=None, device=0):
        torch = _torch()
        dev = torch.device("cuda", device)
        self.n = int(n_events)
        self.max_rows = int(max_rows if max_rows is not None else max(4096, 200 * n_events))
        self.features = torch.zeros(self.max_rows * NF, dtype=torch.float32, device=dev)
        self.outer = torch.zeros(self.max_rows, dtype=torch.int32, device=dev)
        self.scores = torch.zeros(self.max_rows, dtype=torch.float32, device=dev)
        self.labels = torch.zeros(self.max_rows, dtype=torch.uint8, device=dev)
        self.rows = torch.zeros(1, dtype=torch.int32, device=dev)
        self.uncertain = torch.zeros(max(1, self.n), dtype=torch.uint8, device=dev)

    def n_rows(self):
        return min(int(self.rows.item()), self.max_rows)

    def args(self):
        return (self.features.data_ptr(), self.outer.data_ptr(), self.scores.data_ptr(), self.rows.data_ptr(),
                self.uncertain.data_ptr(), self.max_rows)


class ComboScorer:
    """Calls of the combination scorer on a pipeline.Reconstruction context."""

    def __init__(self, rc):
        self.rc = rc
        self.lib = rc.lib

    def yz(self, b, orows, model=None, t_keep=0.5, t_unc=0.5, stream=None):
        """or_yz_scored: model None writes the rows and prunes nothing."""
        f, o, s, r, u, cap = orows.args()
        _lib.check(self.lib.or_yz_scored(self.rc.ctx, b.hits_view(), b.tracks_view(), b.toomany.data_ptr(), b.n,
                                         None if model is None else model.ptr(), float(t_keep), float(t_unc), f, o, s,
                                         r, u, cap, self.rc._stream(stream)), "or_yz_scored")

    def labels(self, b, orows, stream=None):
        _lib.check(self.lib.or_outer_labels(self.rc.ctx, b.tracks_view(), b.toomany.data_ptr(),
                                            orows.outer.data_ptr(), orows.rows.data_ptr(), orows.max_rows,
                                            orows.labels.data_ptr(), self.rc._stream(stream)), "or_outer_labels")

    def run_batch(self, b, orows, model, t_keep, t_unc, stream=None):
        """The whole path with the combination scorer (or_run_batch_scored)."""
        f, o, s, r, u, cap = orows.args()
        _lib.check(self.lib.or_run_batch_scored(self.rc.ctx, b.hits_view(), b.tracks_view(), b.ntracklets.data_ptr(),
                                                b.toomany.data_ptr(), b.n, model.ptr(), float(t_keep), float(t_unc),
                                                f, o, s, r, u, cap, self.rc._stream(stream)), "or_run_batch_scored")

    def plain_with_rows(self, b, orows, stream=None):
        """The plain chain with the rows of its queued tracklets and their
        labels: the training data."""
        rc = self.rc
        b.ntracklets.zero_()
        rc.event_reduce(b, stream)
        rc.xz_tracking(b, stream)
        self.yz(b, orows, None, stream=stream)
        rc.back_track_cleaning(b, stream)
        rc.global_tracking(b, stream)
        self.labels(b, orows, stream)


def dimuon_agreement(rc, b_ref, b_new, device=0):
    """Dimuons of the plain-method run b_ref reproduced by the run b_new:
    both batches go through the post-global selection, vertexing and dimuon
    building (on copies of their tracks), and a plain dimuon counts as
    reproduced when the same event of b_new holds a dimuon record equal to
    it bit for bit (which needs both of its tracks reproduced exactly).
    Returns (plain dimuons, reproduced, new dimuons, tracks of plain dimuons,
    those reproduced)."""
    from . import pipeline
    out = []
    for b in (b_ref, b_new):
        d = pipeline.DeviceDimuons(b.n, device)
        t_n, t_t = b.ntracks.clone(), b.tracks.clone()
        rc.selection(b)
        rc.vertexing(b)
        rc.dimuons(b, d)
        rc.sync()
        b.ntracks.copy_(t_n)
        b.tracks.copy_(t_t)
        out.append(d.download())
    ref, new = out
    n_ref = n_rep = n_new = 0
    nd_r = ref.ndimuons.astype(np.int64)
    nd_n = new.ndimuons.astype(np.int64)
    R = ref.dimuons.reshape(ref.n, -1, L.NDIMUONPARAM).view(np.uint32)
    N = new.dimuons.reshape(new.n, -1, L.NDIMUONPARAM).view(np.uint32)
    for e in np.nonzero((nd_r > 0) | (nd_n > 0))[0]:
        a = {R[e, k].tobytes() for k in range(min(nd_r[e], R.shape[1]))}
        c = {N[e, k].tobytes() for k in range(min(nd_n[e], N.shape[1]))}
        n_ref += len(a)
        n_new += len(c)
        n_rep += len(a & c)
    return n_ref, n_rep, n_new, 2 * n_ref, 2 * n_rep
