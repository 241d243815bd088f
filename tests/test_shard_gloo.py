"""Event sharding across ranks, on CPU with the gloo backend (world size 2).

Each rank takes its contiguous share of one seeded batch, runs the path on it
(the CPU oracle stands in for a rank's GPU here), and the host-side
collectives assemble the per-event results and the max time.  The union must
equal the single-process run: events are independent, so sharding changes
nothing but where an event runs.
"""
import json
import os
import socket

import numpy as np
import pytest


def test_shard_range_partitions_every_event():
    from orgpu import shard
    for n in (0, 1, 7, 64, 1001):
        for world in (1, 2, 3, 8):
            ranges = [shard.shard_range(n, world, r) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.shard_range(10, 2, 2)


def _global_counts(tracks, toomany):
    from orgpu import layout as L
    out = np.zeros(tracks.n, np.int64)
    for e in range(tracks.n):
        if not toomany[e]:
            out[e] = sum(1 for s, k, r in tracks.records(e) if r[L.TRK_STID] == 6)
    return out


def _worker(rank, world, port, out_path):
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (repo, os.path.join(repo, "e1039-gpu_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist
    from oracle import pyoracle as O
    from orgpu import GEOMETRY_E906, layout as L, shard, synth as S

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", world_size=world, rank=rank)
    plane, wp = O.parse_geometry(GEOMETRY_E906)
    geo = S.Geometry(plane, wp)
    rec, off, _ = S.generate(geo, S.config_small(48, 906001))
    rec, off = S.cap_records(rec, off)
    my_rec, my_off, first = shard.shard_records(rec, off, world, rank)
    h = S.pack(my_rec, my_off, geo.wire_pos_f32())
    t, st = L.HostTracks(h.n), O.OracleState(h.n)
    O.run_all(plane, h, t, st, n_threads=1)
    counts = shard.gather_to_rank0(_global_counts(t, st.toomany))
    flags = shard.gather_to_rank0(st.toomany.astype(np.int64))
    tmax = shard.max_over_ranks(float(rank + 1))
    nsum = shard.sum_over_ranks(int(h.n))
    if rank == 0:
        hf = S.pack(rec, off, geo.wire_pos_f32())
        tf, sf = L.HostTracks(hf.n), O.OracleState(hf.n)
        O.run_all(plane, hf, tf, sf, n_threads=1)
        with open(out_path, "w") as f:
            json.dump({"counts": counts.tolist(), "flags": flags.tolist(),
                       "full_counts": _global_counts(tf, sf.toomany).tolist(),
                       "full_flags": sf.toomany.astype(int).tolist(), "tmax": tmax, "nsum": nsum,
                       "first": first}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_union_equals_single_run(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle import pyoracle as O
    O.build()
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "rank0.json")
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    r = json.load(open(out))
    assert r["counts"] == r["full_counts"]
    assert r["flags"] == r["full_flags"]
    assert sum(r["full_counts"]) > 0
    assert r["tmax"] == 2.0
    assert r["nsum"] == 48
