"""Throughput of the online-reconstruction hot path on GB300.

Workload: the uneven batch -- 100,000 seeded synthetic E906 events with 0-3
muons (weights 0.2/0.3/0.4/0.1) and log-normal noise (median 300 hits,
sigma 0.8, clipped at 3000).  One step = the whole plain path over the
batch: device packer (compact hit records -> reference layout), event
reducer, XZ, YZ, back-track cleaning, global tracking.

  value   events/s with the records already in HBM (device-timed, CUDA events)
  e2e     events/s through the C ABI with host buffers: pinned records H2D,
          the path, track collection, count + tracks D2H, every step; the
          record copy is double-buffered (step k+1's records go up on a copy
          stream while step k computes), and the timed region holds one copy
          per step
  roofline / cpu_baseline / clocks / gpu_launches as the JSON keys say.

`--impl reference` times the reference's algorithm on the host cores (the CPU
restatement, all threads) on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "e1039-gpu_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "events/s (plain path: event reducer + XZ/YZ tracklets + cleaning + global tracking)"
UNIT = "events/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--events", type=int, default=100000)
    ap.add_argument("--seed", type=int, default=906002)
    ap.add_argument("--cpu-sample", type=int, default=0, help="events in the CPU-baseline sample (0 = auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-rt", action="store_true", help="skip the R-T calibration packer leg")
    ap.add_argument("--no-config4", action="store_true", help="skip the high-occupancy leg")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="reference arm: skip the reference's own GPU kernels")
    ap.add_argument("--reference-gpu-sample", type=int, default=20000,
                    help="reference arm: events given to the reference's GPU kernels")
    return ap.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def config_json(args, n):
    return {"workload": "uneven batch: %d seeded synthetic E906 events, 0-3 muons (0.2/0.3/0.4/0.1), "
                        "log-normal noise median 300 sigma 0.8 clip 3000" % n,
            "events_per_gpu": n, "seed": args.seed, "geometry": "basic_geometry_e906",
            "step": "pack + event reducer + XZ + YZ + back-track cleaning + global tracking",
            "parallelism": "replicas only (events sharded, no collective)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if r[5 + k] == "Active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def run_cpu(plane, wp, rec, off, n, threads):
    from oracle import pyoracle as O
    from orgpu import layout as L, synth as S
    geo = S.Geometry(plane, wp)
    h = S.pack(rec[:off[n]], off[:n + 1], geo.wire_pos_f32())
    t = L.HostTracks(n)
    st = O.OracleState(n)
    t0 = time.perf_counter()
    O.run_all(plane, h, t, st, n_threads=threads)
    dt = time.perf_counter() - t0
    return dt, (threads if threads > 0 else O.hardware_threads())


def reference_gpu_leg(plane, wp, rec, off, n_sample):
    """The reference's own GPU kernels (oracle/_ref/ref_kernels_fmad1.cubin:
    reconstruction_kernels.cuh compiled unchanged for sm_103a with the flags
    of its Makefile) on the first n_sample events of the workload, chained as
    online_reconstruction.cu:776-933 launches them -- one block per event,
    8 threads for the event reducer, 32 for the others, in chunks of its
    EstnEvtMax = 10,000 events -- each launch timed with CUDA events.  The
    reference XZ kernel is not run (it calls __syncthreads in thread-dependent
    branches, K:684-807): the oracle's XZ, bit-exact with the reference's own
    XZ helpers, fills the tracklets between the reducer and YZ.  Only events
    inside the reference's fixed arrays are given to it (raw chamber hits per
    plane <= 120, windowed hits and pairs <= 100, from the oracle's counted
    run); the rest would write past them."""
    from oracle import pyoracle as O
    from oracle.ref import build_ref, refrun
    from orgpu import layout as L, synth as S
    if not os.path.exists(build_ref.image_path("fmad1")):
        return {"unavailable": "reference images not built (oracle/ref/build_ref.py needs the reference sources)"}
    geo = S.Geometry(plane, wp)
    n = min(n_sample, len(off) - 1)
    hits = S.pack(rec[:off[n]], off[:n + 1], geo.wire_pos_f32())
    h2, t2, st2 = hits.copy(), L.HostTracks(n), O.OracleState(n)
    O.run_all(plane, h2, t2, st2, counted=True)
    counts = st2.counts.reshape(n, O.NCOUNTS)
    raw = hits.nhits_cham.reshape(n, L.NCHAM).max(axis=1)
    idx = np.nonzero((raw <= 120) & (counts[:, 6] <= 100) & (counts[:, 7] <= 100))[0]
    per = (L.NCHAM, L.EVT_CHAM_FLOATS, L.NHODO, L.EVT_HODO_FLOATS, L.NPROP, L.EVT_PROP_FLOATS)
    rk = refrun.RefKernels("fmad1")
    rk.set_plane(plane)
    rk.timing = {}
    tracks_out = 0
    try:
        for a in range(0, len(idx), L.REF_EVTMAX):
            sel = idx[a:a + L.REF_EVTMAX]
            m = len(sel)
            h = L.HostHits(m)
            for dst, src, k in zip(h.arrays(), hits.arrays(), per):
                dst[:] = src.reshape(n, k)[sel].reshape(-1)
            rk.put_hits(h)
            rk.put_flags(np.zeros(m, np.uint8))
            rk.event_reduce(m)
            h_er = rk.get_hits(m)
            st = O.OracleState(m)
            st.toomany[:] = rk.get_flags(m)
            t = L.HostTracks(m)
            O.xz(plane, h_er, t, st)
            rk.put_tracks(t)
            rk.put_flags(st.toomany)
            rk.yz(m)
            rk.back_clean(m)
            rk.global_tracking(m)
            rk.selection(m)
            tracks_out += int(rk.get_tracks(m).ntracks.astype(np.int64).sum())
    finally:
        rk.close()
    tm = dict(rk.timing)
    stage = {"event_reduce": tm.get("er", 0.0), "yz": tm.get("yz", 0.0),
             "back_clean": tm.get("clean", 0.0) + tm.get("clean_x", 0.0), "global": tm.get("global", 0.0),
             "select": tm.get("prop", 0.0) + tm.get("gclean", 0.0) + tm.get("gclean_x", 0.0)}
    chain = sum(stage.values())
    return {"image": "fmad1 (the reference's Makefile flags), device code compiled here from its sources",
            "events_sample": int(n), "events_in_reference_bounds": int(len(idx)),
            "stage_ms": stage, "chain_ms_without_xz": chain,
            "events_per_s_without_xz": len(idx) / (chain / 1000.0) if chain > 0 else None,
            "xz": "oracle (the reference XZ kernel is not runnable)",
            "timing": "CUDA events around each launch, summed over chunks of 10,000 events"}


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    from orgpu import GEOMETRY_E906, layout as L, synth as S
    if args.impl == "reference":
        if rank != 0:
            return
        # the reference arm loads the oracle only (oracle/liborc.so): the
        # geometry is parsed by the oracle's restatement of the reference's
        # reader, and the library is neither built nor loaded
        from oracle import pyoracle as O
        plane, wp = O.parse_geometry(GEOMETRY_E906)
    else:
        import __graft_entry__
        __graft_entry__.build()
        from orgpu import _lib
        plane, wp = _lib.geometry_load(GEOMETRY_E906)
    n = args.events
    from orgpu import shard
    cfg = S.config_uneven(n, shard.rank_seed(args.seed, rank))
    rec, off, truth = S.generate(S.Geometry(plane, wp), cfg)
    rec, off = S.cap_records(rec, off)
    cj = config_json(args, n)
    cj["l2"] = "inputs larger than L2 (hit collections %.1f GB, records %.0f MB per step)" % (
        L.EVT_CHAM_FLOATS * 4 * n / 1e9 * (1 + (L.EVT_HODO_FLOATS + L.EVT_PROP_FLOATS) / L.EVT_CHAM_FLOATS),
        rec.nbytes / 1e6)

    if args.impl == "reference":
        # each step: the CPU restatement on a bounded sample, all host threads
        ns = args.cpu_sample or min(n, 12000)
        times = []
        for i in range(args.warmup + args.steps):
            dt, cores = run_cpu(plane, wp, rec, off, ns, 0)
            if i >= args.warmup:
                times.append(dt)
        v = ns * len(times) / sum(times)
        line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000 * statistics.mean(times), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cj,
                "impl": "reference",
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": "first %d events of the workload per step" % ns},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        if not args.no_reference_gpu:
            try:
                line["reference_gpu_kernels"] = reference_gpu_leg(plane, wp, rec, off, args.reference_gpu_sample)
            except Exception as ex:  # the CPU arm's line stands without it
                line["reference_gpu_kernels"] = {"unavailable": "%s: %s" % (type(ex).__name__, ex)}
        print(json.dumps(line))
        return

    import torch
    from orgpu import pipeline
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    rc = pipeline.Reconstruction(plane, local)
    tuned = None
    if not args.no_autotune:
        # launch shapes for this workload, tuned on a sample of its events
        from orgpu import autotune
        ns = min(n, 16000)
        sample = S.pack(rec[:off[ns]], off[:ns + 1], S.Geometry(plane, wp).wire_pos_f32())
        tuned = autotune.tune(rc, sample, candidates=(1, 2, 4, 8, 16), repeats=2, device=local)
        del sample
    b = pipeline.DeviceBatch(n, local)
    stream = torch.cuda.current_stream(dev)
    d_rec = torch.from_numpy(rec.view(np.uint8)).to(dev)
    d_off = torch.from_numpy(off).to(dev)
    d_wp = torch.from_numpy(wp.astype(np.float32).reshape(-1)).to(dev)
    out_cap = max(1024, int(n * 3))
    d_out = torch.empty(out_cap * L.COLLECT_STRIDE, dtype=torch.float32, device=dev)
    d_cnt = torch.zeros(1, dtype=torch.int64, device=dev)

    stages = ["pack", "event_reduce", "xz", "yz", "back_clean", "global"]

    def step(evs=None):
        if evs is not None:
            evs[0].record(stream)
        rc.pack(b, d_rec, d_off, d_wp)
        calls = [rc.event_reduce, rc.xz_tracking, rc.yz_tracking, rc.back_track_cleaning, rc.global_tracking]
        if evs is not None:
            evs[1].record(stream)
        b.ntracklets.zero_()
        for k, fn in enumerate(calls):
            fn(b)
            if evs is not None:
                evs[2 + k].record(stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident throughput -----------------------------------------
    for _ in range(args.warmup):
        step()
    rc.sync()
    per_stage = {s: [] for s in stages}
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    all_evs = [[torch.cuda.Event(enable_timing=True) for _ in range(len(stages) + 1)] for _ in range(args.steps)]
    t_start.record(stream)
    for i in range(args.steps):
        step(all_evs[i])
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    rc.sync()
    # the YZ work of a step (every step runs the same batch): counted on one
    # more, untimed step, so that the timed ones run without the counters
    rc.set_yz_work_counting(True)
    step()
    rc.sync()
    yz_counts = rc.yz_work_counts()
    rc.set_yz_work_counting(False)
    ms = t_start.elapsed_time(t_end) / args.steps
    for evs in all_evs:
        for k, s in enumerate(stages):
            per_stage[s].append(evs[k].elapsed_time(evs[k + 1]))
    ms = shard.max_over_ranks(ms, device=dev)
    value = world * n / (ms / 1000.0)
    stage_ms = {s: statistics.mean(v) for s, v in per_stage.items()}

    # results of the last step, for the roofline accounting
    toomany = b.toomany.cpu().numpy()
    cnt = {"cham": b.nhits_cham.cpu().numpy(), "hodo": b.nhits_hodo.cpu().numpy(),
           "prop": b.nhits_prop.cpu().numpy()}

    # ---- end to end through the C ABI with host buffers ---------------------
    h_rec = torch.from_numpy(rec.view(np.uint8)).pin_memory()
    h_off = torch.from_numpy(off).pin_memory()
    h_cnt = torch.zeros(1, dtype=torch.int64).pin_memory()
    h_out = torch.empty(out_cap * L.COLLECT_STRIDE, dtype=torch.float32).pin_memory()
    h_flags = torch.empty(n, dtype=torch.uint8).pin_memory()
    d2h_bytes = []

    # Double-buffered inputs: step k+1's records go up on a copy stream while
    # step k computes; each step still copies its own records in and reads
    # its own result back.
    copy_stream = torch.cuda.Stream(dev)
    d_recs = [d_rec, torch.empty_like(d_rec)]
    d_offs = [d_off, torch.empty_like(d_off)]
    copied = [torch.cuda.Event(), torch.cuda.Event()]
    used = [torch.cuda.Event(), torch.cuda.Event()]
    pipe = {"k": 0, "staged": False}

    def stage(i):
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_event(used[i])  # the step that read buffer i has packed it
            d_recs[i].copy_(h_rec, non_blocking=True)
            d_offs[i].copy_(h_off, non_blocking=True)
            copied[i].record(copy_stream)

    def e2e_step():
        i = pipe["k"] % 2
        if not pipe["staged"]:
            stage(i)
        stream.wait_event(copied[i])
        rc.pack(b, d_recs[i], d_offs[i], d_wp)
        used[i].record(stream)
        rc.run_batch(b)
        rc.collect(b, d_out, d_cnt, 6.0)
        stage(1 - i)
        pipe["staged"] = True
        pipe["k"] += 1
        h_cnt.copy_(d_cnt, non_blocking=True)
        h_flags.copy_(b.toomany, non_blocking=True)
        stream.synchronize()
        k = min(int(h_cnt.item()), out_cap)
        h_out[:k * L.COLLECT_STRIDE].copy_(d_out[:k * L.COLLECT_STRIDE], non_blocking=True)
        stream.synchronize()
        d2h_bytes.append(8 + n + k * L.COLLECT_STRIDE * 4)
        return k

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    d2h_bytes.clear()
    e0.record(stream)
    ntrk = 0
    for _ in range(args.steps):
        ntrk = e2e_step()
    stream.wait_event(copied[pipe["k"] % 2])  # the copy staged by the last step is inside the region
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e_ms = shard.max_over_ranks(e2e_ms, device=dev)
    rc.sync()

    if rank != 0:
        return

    # ---- roofline of the dominant stage (YZ) and of the event reducer --------
    peaks = measured_peaks()
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    prof = profile_figures()
    dominant = max(stage_ms, key=stage_ms.get)
    roofline = yz_roofline(yz_counts, stage_ms["yz"], n, clk, dev, prof)
    roofline["dominant_stage"] = "%s (%.2f of %.2f ms per step)" % (dominant, stage_ms[dominant], ms)
    # event reducer: algorithmic bytes = 20 B per raw hit read + 20 B per kept
    # hit written + 48 counts read and written + the flag, per event
    path_det = np.isin(rec["det"], np.array(L.PATH_PLANES))
    raw = int(path_det.sum())
    kept = int(cnt["cham"].reshape(n, L.NCHAM)[:, [d - 1 for d in L.EFF_DETID_CHAMBERS]].sum() +
               cnt["hodo"].sum() + cnt["prop"].sum())
    er_bytes = 20 * raw + 20 * kept + n * (48 * 8 + 1)
    er_gbs = er_bytes / (stage_ms["event_reduce"] / 1000.0) / 1e9
    er_prof = prof.get("kernels", {}).get("er_kernel", {})
    er_traffic = er_prof.get("dram_bytes_per_event")
    roofline_er = {"bound": "hbm", "kernel": "er_kernel (event reducer)", "achieved": er_gbs, "peak": hbm_peak,
                   "unit": "GB/s", "frac": er_gbs / hbm_peak, "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)",
                   "traffic": None if er_traffic is None else er_traffic * n,
                   "traffic_source": prof.get("source"), "algorithmic_bytes_per_launch": er_bytes}

    # ---- CPU baseline ---------------------------------------------------------
    cpu = None
    if not args.no_cpu_baseline:
        ns = args.cpu_sample or min(n, 12000)
        dt, cores = run_cpu(plane, wp, rec, off, ns, 0)
        cpu = {"value": ns / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "first %d events of the workload, one pass, all host threads" % ns}

    rt_res = None if args.no_rt else rt_leg(args, rc, b, plane, rec, d_rec, d_off, d_wp, dev)
    learned_res = None if args.no_learned else learned_leg(args, rc, b, rec, off, d_rec, d_off, d_wp, value, dev)
    config4_res = None if args.no_config4 else config4_leg(args, rc, b, plane, wp, dev, with_learned=not args.no_learned)
    serving_res = None if args.no_serving else serving_leg(plane, wp, tuned)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, no dataset)", "config": cj,
            "e2e": {"value": world * n / (e2e_ms / 1000.0), "unit": UNIT, "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": int(rec.nbytes + off.nbytes),
                    "d2h_bytes_per_step": int(statistics.mean(d2h_bytes)) if d2h_bytes else 0,
                    "copies": "records H2D double-buffered (the next step's during this step's compute), "
                              "result D2H each step after its compute"},
            "roofline": roofline, "roofline_event_reducer": roofline_er, "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": LAUNCHES_PER_STEP * args.steps,
            "stage_ms": stage_ms,
            "events_rejected_frac": float(toomany.mean()), "global_tracks_last_step": ntrk,
            "learned": learned_res, "serving": serving_res, "rt_calibration": rt_res, "config4": config4_res,
            "autotune": None if tuned is None else {"events_per_cta": tuned["best"], "sample_events": tuned["events"],
                                                    "stage_ms_by_shape": tuned["ms"]}}
    print(json.dumps(line))


def opcounts():
    """The frozen per-unit FP32 operation counts (include/or_opcount.h)."""
    import re
    with open(os.path.join(REPO, "include", "or_opcount.h")) as f:
        return {m.group(1): int(m.group(2)) for m in re.finditer(r"#define (OR_OPS_[A-Z0-9_]+) (\d+)", f.read())}


def measured_peaks():
    """MEASURED_PEAKS.json (HBM copy GB/s, cuBLAS bf16 TFLOP/s), or {}."""
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def profile_figures():
    """Per-kernel figures of the committed ncu captures (profiles/traffic.json):
    DRAM bytes per event, issue activity, tensor-pipe activity."""
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def yz_roofline(counts, yz_ms, n, clk, dev, prof, nx=4):
    """The YZ stage (the dominant one) against the FP32 issue peak: the
    algorithmic FP32 operations of its combinations (frozen counts of
    include/or_opcount.h times the device work counters of the step) per
    second.  The stage is bound by instruction issue on the FP32/INT pipes,
    not by HBM or the tensor cores, so the measured issue activity of its
    kernels (ncu) is given beside it."""
    import torch
    ops = opcounts()
    fitted, hitsum, surv = counts
    n_avg = hitsum / fitted if fitted else 0.0
    first = fitted * (ops["OR_OPS_FIT_FIXED"] + ops["OR_OPS_YZ_CUT1"]) + hitsum * (ops["OR_OPS_CALC_Y"] +
                                                                                  ops["OR_OPS_FIT_POINT"])
    per_surv = ((n_avg / 2) * ops["OR_OPS_LR_PAIR"] + n_avg * ops["OR_OPS_LR_SINGLE"] +
                n_avg * ops["OR_OPS_FIT_POINT"] + ops["OR_OPS_FIT_FIXED"] + ops["OR_OPS_YZ_CUT2"] +
                ops["OR_OPS_PROP_MATCH"] + ops["OR_OPS_HODO_MATCH"] + (n_avg + nx) * ops["OR_OPS_CHI2_HIT"])
    total = first + surv * per_surv
    secs = yz_ms / 1000.0
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = clk.get("sm_max_mhz") or 2070.0
    peak = sms * 128 * 2 * mhz * 1e6 / 1e12  # FP32 lanes x (FMA = 2 flops) x clock
    achieved = total / secs / 1e12
    kp = prof.get("kernels", {})
    yz_k = ("yz_plan_kernel", "yz_first_kernel", "yz_second_kernel")
    per_ev = [kp.get(k, {}).get("dram_bytes_per_event") for k in yz_k]
    return {"bound": "issue (FP32/INT pipes; neither HBM nor tensor)",
            "kernel": "YZ stage: yz_tab, yz_plan, yz_first, yz_second, yz_apply kernels",
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "nominal FP32 non-tensor peak: %d SMs x 128 lanes x 2 (FMA) x %.0f MHz" % (sms, mhz),
            "traffic": None if None in per_ev else sum(per_ev) * n,
            "traffic_source": prof.get("source"),
            "algorithmic_flops_per_launch": total,
            "fitted_combinations": fitted, "first_cut_survivors": surv, "mean_uv_hits": n_avg,
            "fitted_combinations_per_s": fitted / secs, "survivors_per_s": surv / secs,
            "flops_per_fitted_combination": (first / fitted) if fitted else None,
            "flops_per_survivor": per_surv, "x_hits_assumed": nx,
            "issue_active_ncu": {k: kp.get(k, {}).get("issue_active") for k in yz_k},
            "op_counts": "include/or_opcount.h"}


# kernels one step launches: pack, event reducer, XZ, YZ fit table / plan /
# first cut / survivors / apply, cleaning, global tracking
LAUNCHES_PER_STEP = 10


def rt_leg(args, rc, b, plane, rec, d_rec, d_off, d_wp, dev):
    """The device packer with the drift distance from the R-T calibration
    (clamped cubic spline per plane, evaluated in double per hit), and the
    same conversion in place on packed hits, against the plain packer, on
    the workload's records; device time per launch (CUDA events)."""
    import torch
    from orgpu import CALIBRATION_E906, _lib, pipeline
    rt, _ = _lib.rt_load(CALIBRATION_E906, plane)
    d_rt = pipeline.rt_to_device(rt, dev.index)
    stream = torch.cuda.current_stream(dev)
    legs = {"pack_ms": lambda: rc.pack(b, d_rec, d_off, d_wp),
            "pack_rt_ms": lambda: rc.pack_rt(b, d_rec, d_off, d_wp, d_rt),
            "rt_apply_ms": lambda: rc.rt_apply(b, d_rt)}
    out = {}
    for name, fn in legs.items():
        for _ in range(args.warmup):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = e0.elapsed_time(e1) / args.steps
    # leave the batch as the plain chain had it
    rc.pack(b, d_rec, d_off, d_wp)
    rc.sync()
    n_rt = int(np.isin(rec["det"], np.r_[1:31, 47:55]).sum())
    out["records"] = int(len(rec))
    out["converted_hits"] = n_rt
    # algorithmic bytes of the packer: 16 B record read + 20 B hit written
    out["pack_rt_gbs"] = 36.0 * len(rec) / (out["pack_rt_ms"] / 1000.0) / 1e9
    return out


def learned_leg(args, rc, b_plain, rec, off, d_rec, d_off, d_wp, plain_value, dev):
    """The learned path on the same batch: the combination scorer (rows =
    live (u3, v3) outer iterations of the queued YZ tracklets, pruned on the
    tensor cores' scores, or_run_batch_scored) when its model is present,
    and the tracklet scorer (or_run_batch_learned) beside it.  Events/s and,
    against the plain run of the last timed step, the recall of global tracks
    and of dimuons (tracks bit for bit), learned tracks absent from the plain
    output, rows kept and uncertain events."""
    import os as _os
    import torch
    from orgpu import learned, pipeline
    n = b_plain.n
    stream = torch.cuda.current_stream(dev)
    bl = pipeline.DeviceBatch(n, dev.index)
    lrn = learned.Learned(rc)

    def timed(step):
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        rc.sync()
        return e0.elapsed_time(e1) / args.steps

    def agreement(ms, sp, path):
        n_ref, n_match, n_new = lrn.agreement(b_plain, bl)
        d_ref, d_rep, d_new, dt_ref, dt_rep = learned.dimuon_agreement(rc, b_plain, bl, dev.index)
        return {"value": n / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms, "plain_value": plain_value,
                "ratio_vs_plain": (n / (ms / 1000.0)) / plain_value,
                "recall": n_match / n_ref if n_ref else 1.0, "plain_global_tracks": n_ref,
                "reproduced": n_match, "learned_global_tracks": n_new,
                "learned_tracks_not_in_plain": n_new - n_match,
                "dimuon_recall": d_rep / d_ref if d_ref else 1.0, "plain_dimuons": d_ref,
                "dimuons_reproduced": d_rep, "learned_dimuons": d_new,
                "dimuon_track_recall": dt_rep / dt_ref if dt_ref else 1.0,
                "model": path, "t_keep": sp.t_keep, "t_unc": sp.t_unc}

    out = None
    if _os.path.exists(learned.MODEL_COMBO_E906):
        sp = learned.ScorerParams.load(learned.MODEL_COMBO_E906)
        cs = learned.ComboScorer(rc)
        model = learned.DeviceModel(sp, dev.index)
        orows = learned.OuterRows(n, device=dev.index)

        def step_combo():
            rc.pack(bl, d_rec, d_off, d_wp)
            cs.run_batch(bl, orows, model, sp.t_keep, sp.t_unc)

        ms = timed(step_combo)
        nr = orows.n_rows()
        out = agreement(ms, sp, "e1039-gpu_gb300/data/combo_scorer_e906.npz")
        out.update({"scorer": "combination scorer: (u3, v3) outer iterations of queued YZ tracklets",
                    "rows": nr, "rows_kept": float((orows.scores[:nr] >= sp.t_keep).float().mean().item()) if nr
                    else 1.0, "uncertain_events": int(orows.uncertain[:n].sum().item()),
                    "mlp": mlp_figures(lrn, model, orows.features, nr, orows.scores, stream)})
        del orows
    sp = learned.ScorerParams.load()
    model = learned.DeviceModel(sp, dev.index)
    r = learned.TrackletRows(n, device=dev.index)

    def step_tracklet():
        rc.pack(bl, d_rec, d_off, d_wp)
        lrn.run_batch(bl, r, model, sp.t_keep, sp.t_unc)

    ms = timed(step_tracklet)
    nr = r.n_rows()
    tk = agreement(ms, sp, "e1039-gpu_gb300/data/scorer_e906.npz")
    tk.update({"scorer": "tracklet scorer: XZ tracklets",
               "kept_share": float(r.keep[:nr].float().mean().item()) if nr else 1.0})
    if out is None:
        return tk
    out["tracklet_scorer"] = tk
    return out


def mlp_figures(lrn, model, features, nr, scores, stream, reps=10):
    """The scoring MLP (mlp_score_kernel, 16-64-64-1 in BF16 on the tensor
    cores) over the step's nr combination rows, timed alone with CUDA events:
    achieved BF16 FLOP/s against the measured cuBLAS bf16 peak, and the rows'
    bytes (16 f32 features in, one f32 score out) against the HBM peak -- at
    10,368 FLOP per 68 bytes the kernel is bound by memory, not by the
    tensor pipe; the ncu tensor-pipe activity is given beside it."""
    import torch
    if nr <= 0:
        return None
    for _ in range(3):
        lrn.score(model, features, nr, scores)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        lrn.score(model, features, nr, scores)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    flops_row = 2 * (16 * 64 + 64 * 64 + 64 * 1)
    bytes_row = 16 * 4 + 4
    peaks = measured_peaks()
    bf16 = float(peaks.get("bf16_tflops", 1900.0))
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    tflops = nr * flops_row / (ms / 1000.0) / 1e12
    gbs = nr * bytes_row / (ms / 1000.0) / 1e9
    prof = profile_figures().get("kernels", {}).get("mlp_score_kernel", {})
    return {"kernel": "mlp_score_kernel", "rows": nr, "ms": ms, "flops_per_row": flops_row, "bytes_per_row": bytes_row,
            "achieved_tflops": tflops, "bf16_peak_tflops": bf16, "frac_of_bf16_peak": tflops / bf16,
            "achieved_gbs": gbs, "hbm_peak_gbs": hbm, "frac_of_hbm_peak": gbs / hbm, "bound": "hbm",
            "peak_source": "measured (MEASURED_PEAKS.json)" if peaks else "fallback",
            "tensor_pipe_active_ncu": prof.get("tensor_pipe_active")}


def config4_leg(args, rc, b, plane, wp, dev, with_learned=True, chunks=5, seed=906004):
    """High occupancy: 5 x the batch size (500,000 events at the default
    100,000) with two muons, Poisson(1000) noise uniform over the (plane,
    element) pairs of the 48 planes the path reads, and after-pulse
    duplicates of 10 % of the hits (same element, tdc + U(50, 200) ns).
    Generated in chunks of one batch (other seeds per chunk) by a spawned
    process pool; each chunk is packed and reconstructed on the device with
    its records already in HBM (CUDA events around pack + the plain chain,
    and around pack + the learned chain).  The event reducer's station
    limits (210/120/90/90 reduced chamber hits) reject every event of this
    workload, as the reference's would; the rejection rate is reported."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import torch
    from orgpu import learned, synth as S
    n = b.n
    jobs = [(bytes(plane.to_bytes()), wp, S.config_high_occupancy(n, seed + i)) for i in range(chunks)]
    with cf.ProcessPoolExecutor(max_workers=min(chunks, os.cpu_count() or 1),
                                mp_context=mp.get_context("spawn")) as ex:
        parts = list(ex.map(S.generate_capped, jobs))
    stream = torch.cuda.current_stream(dev)
    d_wp = torch.from_numpy(wp.astype(np.float32).reshape(-1)).to(dev)
    lrn = sp = model = r = bl = None
    if with_learned:
        combo = os.path.exists(learned.MODEL_COMBO_E906)
        sp = learned.ScorerParams.load(learned.MODEL_COMBO_E906 if combo else learned.MODEL_E906)
        lrn = learned.ComboScorer(rc) if combo else learned.Learned(rc)
        model = learned.DeviceModel(sp, dev.index)
        r = learned.OuterRows(n, device=dev.index) if combo else learned.TrackletRows(n, device=dev.index)
        bl = pipeline_batch(n, dev)
        agree_lrn = learned.Learned(rc)
    ms_plain, ms_learned, rejected, records, tracks = 0.0, 0.0, 0, 0, 0
    agree = [0, 0, 0]
    for rec4, off4 in parts:
        d_rec = torch.from_numpy(rec4.view(np.uint8)).to(dev)
        d_off = torch.from_numpy(off4).to(dev)
        records += len(rec4)
        legs = [("plain", lambda: (rc.pack(b, d_rec, d_off, d_wp), b.ntracklets.zero_(), rc.run_batch(b)))]
        if with_learned:
            legs.append(("learned", lambda: (rc.pack(bl, d_rec, d_off, d_wp),
                                             lrn.run_batch(bl, r, model, sp.t_keep, sp.t_unc))))
        for name, fn in legs:
            fn()  # warm-up on this chunk
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            if name == "plain":
                ms_plain += e0.elapsed_time(e1)
            else:
                ms_learned += e0.elapsed_time(e1)
        rc.sync()
        rejected += int(b.toomany.sum().item())
        if with_learned:
            a = agree_lrn.agreement(b, bl)
            agree = [x + y for x, y in zip(agree, a)]
        del d_rec, d_off
    total = n * len(parts)
    out = {"events": total, "chunks": len(parts), "records": records,
           "workload": ("two muons, Poisson(1000) noise uniform over the (plane, element) pairs of the 48 path "
                        "planes, after-pulses on 10 percent of hits; seeds %d..%d" % (seed, seed + len(parts) - 1)),
           "value": total / (ms_plain / 1000.0), "unit": UNIT, "ms_total": ms_plain,
           "rejected_frac": rejected / total,
           "rejection_rule": "reduced chamber hits per station above 210/120/90/90 (D0/D2/D3p/D3m)"}
    if with_learned:
        out["learned"] = {"value": total / (ms_learned / 1000.0), "unit": UNIT, "ms_total": ms_learned,
                          "ratio_vs_plain": ms_plain / ms_learned, "plain_global_tracks": agree[0],
                          "reproduced": agree[1], "learned_global_tracks": agree[2],
                          "recall": (agree[1] / agree[0]) if agree[0] else None}
    return out


def _os_rel(path):
    return os.path.relpath(path, REPO)


def pipeline_batch(n, dev):
    from orgpu import pipeline
    return pipeline.DeviceBatch(n, dev.index)


def serving_leg(plane, wp, tuned=None, pool_events=40000, burst_s=4.0, seed=906005):
    """Spill-structured Poisson arrivals of batches of U(1, 10000) one-dimuon
    events (the learned-scorer / small-batch distribution) at three offered
    loads, through the continuous-batching server: p50/p99 latency and
    sustained events/s per load.  Each 4 s burst starts on an idle server:
    the 56 s gap between spills is the drain.  The same schedules run again
    on a server whose slots take the learned path (scorer + pruned YZ, plain
    fallback for uncertain events)."""
    import gc
    import torch
    from orgpu import learned, serving, synth as S
    geo = S.Geometry(plane, wp)
    rec, off, _ = S.generate(geo, S.config_small(pool_events, seed))
    rec, off = S.cap_records(rec, off)
    rng = np.random.default_rng(seed)

    def take(n):
        e0 = int(rng.integers(0, pool_events - n + 1))
        r0 = off[e0]
        return rec[r0:off[e0 + n]], (off[e0:e0 + n + 1] - r0).astype(np.int64)

    srv = serving.Server(plane, wp, slot_events=10000, max_slots=4, rec_per_event=400, launch_config=tuned)
    # capacity: a saturating queue of full-size batches
    cal = srv.serve([(0.0,) + take(10000) for _ in range(12)])
    cap = serving.latency_stats(cal)["events_per_s"]
    schedules = {}
    for frac in (0.5, 0.8, 1.1):
        rate = frac * cap / 5000.5  # batches per second (mean batch 5000.5 events)
        sched, t = [], 0.0
        while True:
            t += float(rng.exponential(1.0 / rate))
            if t > burst_s:
                break
            sched.append((t,) + take(int(rng.integers(1, 10001))))
        schedules["%.1fx" % frac] = (frac, sched)

    def run_loads(server):
        loads = {}
        for key, (frac, sched) in schedules.items():
            done = server.serve(sched)
            st = serving.latency_stats(done) if done else {}
            st["offered_events_per_s"] = frac * cap
            loads[key] = st
        return loads

    loads = run_loads(srv)
    nslots = len(srv.slots)
    del srv
    gc.collect()
    torch.cuda.empty_cache()
    model_path = learned.MODEL_COMBO_E906 if os.path.exists(learned.MODEL_COMBO_E906) else learned.MODEL_E906
    lsrv = serving.Server(plane, wp, slot_events=10000, max_slots=4, rec_per_event=400, launch_config=tuned,
                          scorer=learned.ScorerParams.load(model_path))
    lcal = lsrv.serve([(0.0,) + take(10000) for _ in range(12)])
    learned_res = {"slots": len(lsrv.slots), "capacity_events_per_s": serving.latency_stats(lcal)["events_per_s"],
                   "model": _os_rel(model_path), "loads": run_loads(lsrv)}
    del lsrv
    gc.collect()
    torch.cuda.empty_cache()
    return {"slots": nslots, "slot_events": 10000, "graphs": True, "burst_s": burst_s,
            "capacity_events_per_s": cap, "workload": "one dimuon + Poisson(150) noise per event", "loads": loads,
            "learned": learned_res}


if __name__ == "__main__":
    main()
