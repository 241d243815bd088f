"""Continuous-batching event server on one GPU.

A request is a batch of events (hit records + offsets, on the host).  The
server keeps `slots`: each a resident device batch of up to `slot_events`
events with its own library context (so its own YZ work queue), its own CUDA
stream, record/offset/output buffers and, optionally, CUDA graphs of the
whole step (pack -> reconstruction -> track gather) captured for a few
bucket sizes.  The number of slots is set by the free device memory when the
server starts (admission by HBM): a slot is only created when its buffers
fit, and a request is only started when a slot is free.

Scheduling: pending requests are packed in arrival order into the next free
slot, a large request split across slots, several small ones sharing a slot;
so requests that arrive while others are on the GPU start as soon as a slot
frees, and work of different slots overlaps on the device.  Each event is
reconstructed independently, so a request's result does not depend on what
it shares a slot with; results are the global tracks of its events
(or_collect_tracks rows, event index relative to the request).

Latency of a request = time its last track row is on the host - its arrival.
"""
import collections
import time

import numpy as np

from . import _lib, layout as L, learned, pipeline

BUCKETS = (256, 1024, 4096, 10000)


def _torch():
    import torch
    return torch


class Request:
    def __init__(self, rid, records, offsets, arrival):
        self.rid = rid
        self.records = records
        self.offsets = np.asarray(offsets, np.int64)
        self.n = len(self.offsets) - 1
        self.arrival = arrival
        self.next_event = 0
        self.pending_pieces = 0
        self.rows = []
        self.flags = np.zeros(self.n, np.uint8)
        self.done_time = None

    def result(self):
        """Track rows of the request (float32 [k, OR_COLLECT_STRIDE]),
        sorted by (event, slot*16 + position)."""
        if not self.rows:
            return np.zeros((0, L.COLLECT_STRIDE), np.float32)
        r = np.concatenate(self.rows)
        order = np.lexsort((r[:, 1], r[:, 0]))
        return r[order]


class Slot:
    """A resident batch of up to `cap` events and everything its step needs."""

    def __init__(self, plane, wire_pos_f, cap, rec_cap, device, scorer=None, graphs=True):
        torch = _torch()
        self.dev = torch.device("cuda", device)
        self.cap = cap
        self.rec_cap = rec_cap
        self.rc = pipeline.Reconstruction(plane, device, max_events=cap)
        self.stream = torch.cuda.Stream(device=self.dev)
        self.b = pipeline.DeviceBatch(cap, device)
        self.d_rec = torch.zeros(rec_cap * L.HIT_RECORD_DTYPE.itemsize, dtype=torch.uint8, device=self.dev)
        self.d_off = torch.zeros(cap + 1, dtype=torch.int64, device=self.dev)
        self.d_wp = wire_pos_f
        self.out_cap = 4 * cap
        self.d_out = torch.zeros(self.out_cap * L.COLLECT_STRIDE, dtype=torch.float32, device=self.dev)
        self.d_cnt = torch.zeros(1, dtype=torch.int64, device=self.dev)
        self.h_rec = torch.empty(rec_cap * L.HIT_RECORD_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
        self.h_off = torch.empty(cap + 1, dtype=torch.int64).pin_memory()
        self.h_cnt = torch.zeros(1, dtype=torch.int64).pin_memory()
        self.h_flags = torch.empty(cap, dtype=torch.uint8).pin_memory()
        self.h_out = torch.empty(self.out_cap * L.COLLECT_STRIDE, dtype=torch.float32).pin_memory()
        self.scorer = scorer
        # a combination-scorer model (its rows are the live (u3, v3) outer
        # iterations of queued tracklets) runs or_run_batch_scored; a
        # tracklet-scorer model or_run_batch_learned
        self.combo = scorer is not None and "candidates" in scorer.meta
        if scorer is not None:
            self.model = learned.DeviceModel(scorer, device)
            if self.combo:
                self.lrn = learned.ComboScorer(self.rc)
                self.rows = learned.OuterRows(cap, device=device)
            else:
                self.lrn = learned.Learned(self.rc)
                self.rows = learned.TrackletRows(cap, device=device)
        self.graphs = {}
        self.use_graphs = graphs
        self.pieces = None
        self.stage = None
        self.ev = torch.cuda.Event()
        self.n_used = 0

    # one step on `n` events (the device work of a batch)
    def _step(self, n):
        b = self.b
        view_n = b.n
        b.n = n
        try:
            self.rc.pack(b, self.d_rec, self.d_off, self.d_wp)
            if self.scorer is not None:
                self.lrn.run_batch(b, self.rows, self.model, self.scorer.t_keep, self.scorer.t_unc)  # either scorer
            else:
                self.rc.run_batch(b)
            self.rc.collect(b, self.d_out, self.d_cnt, 6.0)
        finally:
            b.n = view_n

    def capture(self):
        """CUDA graphs of the step for every bucket size (after one eager run
        of each, so every kernel and attribute is set up)."""
        torch = _torch()
        if not self.use_graphs:
            return
        with torch.cuda.stream(self.stream):
            self.d_off.zero_()
            for B in BUCKETS:
                if B > self.cap:
                    continue
                self._step(B)
        self.stream.synchronize()
        for B in BUCKETS:
            if B > self.cap:
                continue
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=self.stream):
                self._step(B)
            self.graphs[B] = g
        self.stream.synchronize()

    def bucket(self, n):
        for B in BUCKETS:
            if n <= B <= self.cap and B in self.graphs:
                return B
        return None

    def launch(self, pieces):
        """Stage the pieces' records, run the step asynchronously on the slot's
        stream, then read back the track count."""
        torch = _torch()
        self.pieces = pieces
        n = sum(p[2] for p in pieces)
        recs, offs = [], [0]
        for req, e0, ne in pieces:
            r0, r1 = req.offsets[e0], req.offsets[e0 + ne]
            recs.append(req.records[r0:r1])
            offs.extend((req.offsets[e0 + 1:e0 + ne + 1] - r0 + offs[-1]).tolist())
        rec = np.concatenate(recs) if recs else np.zeros(0, L.HIT_RECORD_DTYPE)
        if len(rec) > self.rec_cap:
            raise _lib.OrError(_lib.OR_ERR_CAPACITY, f"{len(rec)} records exceed the slot's {self.rec_cap}")
        B = self.bucket(n)
        nrun = B if B is not None else n
        off = np.full(nrun + 1, offs[-1], np.int64)  # padding events have no records
        off[:n + 1] = offs
        rb = rec.view(np.uint8)
        self.h_rec[:rb.size].numpy()[:] = rb
        self.h_off[:nrun + 1].numpy()[:] = off
        with torch.cuda.stream(self.stream):
            self.d_rec[:rb.size].copy_(self.h_rec[:rb.size], non_blocking=True)
            self.d_off[:nrun + 1].copy_(self.h_off[:nrun + 1], non_blocking=True)
            if B is not None:
                self.graphs[B].replay()
            else:
                self._step(n)
            self.h_cnt.copy_(self.d_cnt, non_blocking=True)
            self.h_flags[:n].copy_(self.b.toomany[:n], non_blocking=True)
            self.ev.record(self.stream)
        self.n_used = n
        self.stage = "compute"

    def poll(self):
        """Advance: compute done -> copy the rows back; rows back -> finished.
        Returns True when the slot's pieces are complete."""
        torch = _torch()
        if self.stage is None or not self.ev.query():
            return False
        if self.stage == "compute":
            k = min(int(self.h_cnt.item()), self.out_cap)
            self.k = k
            with torch.cuda.stream(self.stream):
                self.h_out[:k * L.COLLECT_STRIDE].copy_(self.d_out[:k * L.COLLECT_STRIDE], non_blocking=True)
                self.ev.record(self.stream)
            self.stage = "rows"
            return False
        rows = self.h_out[:self.k * L.COLLECT_STRIDE].numpy().reshape(self.k, L.COLLECT_STRIDE).copy()
        flags = self.h_flags[:self.n_used].numpy().copy()
        base = 0
        for req, e0, ne in self.pieces:
            sel = (rows[:, 0] >= base) & (rows[:, 0] < base + ne)
            part = rows[sel]
            part[:, 0] = part[:, 0] - base + e0
            req.rows.append(part)
            req.flags[e0:e0 + ne] = flags[base:base + ne]
            req.pending_pieces -= 1
            base += ne
        self.stage = None
        self.pieces = None
        return True


class Server:
    """Slots + the scheduler.  `max_slots` is an upper bound; the slots
    actually created are those whose buffers fit in the free device memory,
    keeping `reserve_bytes` free."""

    def __init__(self, plane, wire_pos, slot_events=10000, max_slots=4, rec_per_event=400, device=0, scorer=None,
                 graphs=True, reserve_bytes=8 << 30, launch_config=None):
        torch = _torch()
        self.device = device
        wp = torch.from_numpy(np.asarray(wire_pos, np.float32).reshape(-1)).cuda(device)
        self.slots = []
        sms = torch.cuda.get_device_properties(device).multi_processor_count
        per_slot = self.slot_bytes(slot_events, rec_per_event, scorer is not None, sms)
        for _ in range(max_slots):
            free, _total = torch.cuda.mem_get_info(device)
            if free - per_slot < reserve_bytes:
                break
            self.slots.append(Slot(plane, wp, slot_events, slot_events * rec_per_event, device, scorer, graphs))
        if not self.slots:
            raise _lib.OrError(_lib.OR_ERR_NOMEM, "no slot fits in the free device memory")
        for s in self.slots:
            if launch_config is not None:  # autotune.tune() result: shapes before the graphs are captured
                from . import autotune
                autotune.apply(s.rc, launch_config)
            s.capture()
        self.slot_events = slot_events
        self.pending = collections.deque()
        self.requests = []
        self._open = collections.deque()  # submitted, not finished

    @staticmethod
    def slot_bytes(cap, rec_per_event, with_scorer, sm_count=152):
        lb = _lib.lib()
        b = lb.or_hits_view_bytes(cap) + lb.or_tracks_view_bytes(cap)
        b += cap * rec_per_event * 16 + 4 * cap * L.COLLECT_STRIDE * 4  # records, output rows
        b += lb.or_context_bytes(cap, sm_count)  # the slot's context, sized for its batch
        if with_scorer:
            b += 200 * cap * (L.NFEAT * 4 + 4 + 4 + 1)  # rows of either scorer
        return int(b)

    def submit(self, records, offsets, arrival=None):
        req = Request(len(self.requests), records, offsets, time.perf_counter() if arrival is None else arrival)
        self.requests.append(req)
        self.pending.append(req)
        self._open.append(req)
        return req

    def _fill(self, slot):
        """Pieces for a free slot from the pending queue, in arrival order."""
        pieces, room = [], slot.cap
        rec_room = slot.rec_cap
        while self.pending and room > 0:
            req = self.pending[0]
            e0 = req.next_event
            ne = min(room, req.n - e0)
            # keep within the slot's record buffer
            while ne > 0 and req.offsets[e0 + ne] - req.offsets[e0] > rec_room:
                ne //= 2
            if ne == 0:
                break
            pieces.append((req, e0, ne))
            req.next_event += ne
            req.pending_pieces += 1
            room -= ne
            rec_room -= int(req.offsets[e0 + ne] - req.offsets[e0])
            if req.next_event == req.n:
                self.pending.popleft()
        return pieces

    def step(self, now=None):
        """One scheduler pass: finish polled slots, start free ones.  Returns
        True while work is in flight or pending."""
        busy = False
        for s in self.slots:
            if s.stage is not None:
                s.poll()
                busy = busy or s.stage is not None
        for s in self.slots:
            if s.stage is None and self.pending:
                pieces = self._fill(s)
                if pieces:
                    s.launch(pieces)
                    busy = True
        t = time.perf_counter()
        while self._open and self._open[0].done_time is not None:
            self._open.popleft()
        for req in self._open:
            if req.done_time is None and req.next_event == req.n and req.pending_pieces == 0:
                req.done_time = t
        return busy or bool(self.pending)

    def drain(self):
        while self.step():
            time.sleep(0)

    def serve(self, schedule):
        """Run a schedule of (arrival offset s, records, offsets): requests
        are submitted when their time comes, while earlier ones run.
        Returns the requests."""
        t0 = time.perf_counter()
        todo = collections.deque(sorted(schedule, key=lambda x: x[0]))
        out = []
        while True:
            now = time.perf_counter() - t0
            while todo and todo[0][0] <= now:
                a, rec, off = todo.popleft()
                out.append(self.submit(rec, off, arrival=t0 + a))
            busy = self.step()
            if not busy:
                if not todo:
                    break
                time.sleep(max(0.0, min(todo[0][0] - now, 0.001)))
        return out


def latency_stats(requests):
    lat = np.array([r.done_time - r.arrival for r in requests if r.done_time is not None])
    ev = sum(r.n for r in requests)
    t0 = min(r.arrival for r in requests)
    t1 = max(r.done_time for r in requests)
    return {"requests": len(requests), "events": ev, "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "events_per_s": ev / (t1 - t0)}
