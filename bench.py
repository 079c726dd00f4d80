#!/usr/bin/env python
"""Benchmark: overlap-search reads/s (and suffix-sort Msuffix/s) of PASQUAL's hot path.

Workload (default): 50 Mbp synthetic genome, GC 41 %, 10 % repeat copies of 1-5 kbp segments at
1 % divergence; 100 bp reads at 30x from both strands with 0.5 % substitution errors; t = 63;
32-bit index.  Reads are de-duplicated (equal or reverse-complement reads dropped) before use.

A step is one overlap search (find_intervals + transitive reduction + edge CSR) over every read,
on indexes already resident in HBM.  ``value`` = reads searched / time, whole job.

``e2e`` runs the public API end to end each step: host reads (pinned) -> GPU suffix sorts and
FM-indexes -> overlap search -> edges back to host, into host arrays allocated by the untimed
first step and reused (as the pinned input buffer is).

``--impl reference`` times the reference's CPU algorithm for the same metric: the C restatement
of the reference (oracle/), OpenMP over all host cores, on a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import signal
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "overlap-search reads/s + sort Msuffix/s, learned vs plain GPU, bit-exact"
WORKLOAD = "50Mbp_L100_30x_t63"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--scale", type=float, default=1.0, help="genome-size scale (1.0 = full)")
    ap.add_argument("--cpu-scale", type=float, default=0.1,
                    help="genome-size scale of the CPU-baseline sample")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-modes", action="store_true", help="skip the plain/learned comparison")
    ap.add_argument("--batched-scale", type=float, default=0.25,
                    help="genome scale of the queued-search workload (0 = skip)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _group_size() -> int:
    import torch.distributed as dist
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def rank_barrier() -> None:
    """Barrier over the replicas (the default process group); nothing with one rank."""
    if _group_size() > 1:
        import torch.distributed as dist
        dist.barrier()


def rank_max(x: float, device="cpu") -> float:
    """Maximum of x over the replicas (x itself with one rank).  `device` is where the reduction
    tensor lives: the rank's GPU under NCCL, the CPU under gloo."""
    if _group_size() == 1:
        return x
    import torch
    import torch.distributed as dist
    tt = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def replica_throughput(reads_per_rank: int, world: int, slowest_ms: float) -> float:
    """Whole-job reads/s of `world` replicas that each searched reads_per_rank reads, the slowest
    in slowest_ms per step (weak scaling: every rank searches its own full read set)."""
    return reads_per_rank * world / (slowest_ms * 1e-3)


def workload_reads(name: str, scale: float):
    from pasqual_gb300 import synth
    _, rd, L, t = synth.make_workload(name, scale=scale)
    return synth.dedup(rd), L, t


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_figure(key: str):
    """A figure recorded in the committed ncu summary of the search kernel ("key = value")."""
    p = os.path.join(ROOT, "profiles", "k_search_lean.md")
    try:
        txt = open(p).read()
    except OSError:
        return None
    m = re.search(re.escape(key) + r"\s*=\s*([0-9.]+)", txt)
    return float(m.group(1)) if m else None


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        """Start sampling and wait (up to 10 s) for the first sample, so that the sampler's own
        start-up stays out of the timed region."""
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        t0 = time.time()
        while time.time() - t0 < 10.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.05)

    def stop(self):
        if not self.proc:
            return None
        self.proc.send_signal(signal.SIGTERM)
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(workload: str, scale: float, seconds: float, threads: int | None = None):
    """The C restatement of the reference's overlap search on the host cores (OpenMP), timed on a
    bounded sample: index of a genome scaled by `scale`, search over as many reads as fit in
    about `seconds` seconds."""
    from oracle import port
    port.build()
    rd, L, t = workload_reads(workload, scale)
    threads = threads or os.cpu_count() or 1
    P = port.Port(32)
    ix = P.build_index(rd, t, threads=threads, seed_k=min(12, t))
    seeds = (ix["seed0"], ix["seed1"])
    nr = rd.shape[0]
    probe = min(nr, 20000)
    t0 = time.perf_counter()
    P.overlaps(ix, 0, probe, threads=threads, seeds=seeds)
    dt = time.perf_counter() - t0
    count = int(min(nr, max(probe, probe * seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    g = P.overlaps(ix, 0, count, threads=threads, seeds=seeds)
    dt = time.perf_counter() - t0
    return {"value": count / dt, "unit": "reads/s", "cores": threads, "kind": "port",
            "sample": "%d of %d reads of the %s workload at genome scale %g (%d bp reads, t=%d), "
                      "forward/backward seeds at depth 12 as the reference's sort records them; "
                      "%.1f s" % (count, nr, workload, scale, L, t, dt),
            "probes_per_read": g.probes / max(count, 1)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cb = cpu_baseline(args.workload, args.cpu_scale, args.cpu_seconds)
    vals = [cb["value"]]
    for _ in range(max(0, args.steps - 1)):
        vals.append(cpu_baseline(args.workload, args.cpu_scale, args.cpu_seconds / 2)["value"])
    v = statistics.median(vals)
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "reads/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int32-index", "data": "synthetic",
           "config": {"workload": args.workload, "index": "U32", "sample_scale": args.cpu_scale},
           "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
           "e2e": {"value": v, "unit": "reads/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    out["cpu_baseline"]["value"] = v
    print(json.dumps(out), flush=True)


def seed_modes(P, nr: int, steps: int):
    """Plain backward search (mode 0), interval scan with the k-mer table (1) and with the learned
    index (2) on the same index: search reads/s (whole pq_overlaps, CSR included), kernel time and
    probes per read of each, plus the learned model's build figures."""
    out = {}
    ref = None
    P.learned_build(0, 400)
    P.learned_build(1, 400)
    for name, mode in (("plain", 0), ("scan", 1), ("learned", 2)):
        P.set_seed_mode(mode)
        P.overlaps()
        search, kern = [], []
        for _ in range(steps):
            P.overlaps()
            search.append(P.stage_ms()[2])
            kern.append(P.kernel_stats()[0])
        g = P.graph()
        same = ref is None or (np.array_equal(g.dest, ref[0]) and np.array_equal(g.edge_off, ref[1]))
        if ref is None:
            ref = (g.dest.copy(), g.edge_off.copy())
        out[name] = {"reads_per_s": nr / (statistics.median(search) * 1e-3),
                     "search_ms": statistics.median(search), "kernel_ms": statistics.median(kern),
                     "probes_per_read": g.probes / max(nr, 1), "edges_identical_to_plain": bool(same)}
    lx = [P.learned_info(d) for d in (0, 1)]
    out["learned_model"] = {
        "segments": lx[0]["segments"], "hidden": lx[0]["hidden"], "train_steps": lx[0]["steps"],
        "distinct_keys": [x["num_keys"] for x in lx],
        "build_ms": sum(x["keys_ms"] + x["train_ms"] + x["eval_ms"] for x in lx),
        "train_ms": sum(x["train_ms"] for x in lx),
        "mean_window_rows": [x["mean_window"] for x in lx],
        "mean_window_rows_root_only": [x["mean_window_root"] for x in lx],
        "window_misses": lx[0]["misses"], "window_queries": lx[0]["queries"]}
    out["learned_vs_plain"] = out["learned"]["reads_per_s"] / out["plain"]["reads_per_s"]
    out["scan_vs_plain"] = out["scan"]["reads_per_s"] / out["plain"]["reads_per_s"]
    P.set_seed_mode(1)
    return out


def batched(scale: float, steps: int, device: int, stream):
    """Queued search: several read sets (own L and t each) in one persistent kernel from a device
    work queue, replayed from a CUDA graph with the autotuned plan, against one search launch per
    read set."""
    import torch
    import pasqual_gb300 as pq
    from pasqual_gb300 import synth
    name = "100Mbp_L75-250_25x_batched"
    sets = synth.make_batches(name, scale=scale)
    ctxs = []
    for rd, L, t in sets:
        P = pq.Pasqual(32, device=device, stream=stream.cuda_stream)
        P.set_reads(rd, t)
        P.build_index()
        ctxs.append(P)
    total = sum(rd.shape[0] for rd, _, _ in sets)

    def timed(fn):
        fn()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(device)
        return e0.elapsed_time(e1) / steps

    seq_ms = timed(lambda: [P.overlaps() for P in ctxs])
    ref = [(P.graph().dest.copy()) for P in ctxs]
    tune_ms = pq.autotune_batched(ctxs, graph=True)
    q_ms = timed(lambda: pq.overlaps_batched(ctxs, graph=True))
    same = all(np.array_equal(P.graph().dest, r) for P, r in zip(ctxs, ref))
    st = ctxs[0].batch_stats()
    for P in ctxs:
        P.close()
    return {"workload": name, "genome_scale": scale,
            "read_sets": [{"reads": int(rd.shape[0]), "read_len": L, "t": t} for rd, L, t in sets],
            "reads": int(total), "sequential_reads_per_s": total / (seq_ms * 1e-3),
            "queued_graph_reads_per_s": total / (q_ms * 1e-3), "queued_vs_sequential": seq_ms / q_ms,
            "queued_kernel_ms": st["kernel_ms"], "autotuned_kernel_ms": tune_ms,
            "plan": {k: st[k] for k in ("ctas_per_sm", "groups_per_item", "edge_slots")},
            "graph": bool(st["graph_used"]), "edges_identical_to_sequential": bool(same)}


def run_ours(args):
    import torch
    import pasqual_gb300 as pq

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    rd, L, t = workload_reads(args.workload, args.scale)
    nr = rd.shape[0]
    n = nr * L
    width = 32 if n < (1 << 32) else 64          # the reference's U32/U64 split by index size
    from pasqual_gb300 import synth
    width = max(width, synth.WORKLOADS[args.workload].get("index", 32))
    stream = torch.cuda.Stream(device=dev)
    P = pq.Pasqual(width, device=local, stream=stream.cuda_stream)

    def barrier():
        rank_barrier()

    def max_over_ranks(x: float) -> float:
        return rank_max(x, dev)

    # ---- index build (setup) and suffix-sort throughput
    P.set_reads(rd, t)
    P.build_index()                       # warm-up build
    sort_ms = []
    for _ in range(max(1, min(args.steps, 3))):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        P.sort(0)
        P.sort(1)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        sort_ms.append(e0.elapsed_time(e1))
    P.build_index()                       # index for the search; sort scratch given back
    sort_ms_med = statistics.median(sort_ms)

    # ---- overlap search: warm-up, then K timed steps (clock sampling runs through both)
    clocks = Clocks(local)
    clocks.start()
    for _ in range(args.warmup):
        P.overlaps()
    _, l0 = P.kernel_stats()
    kern_ms = []
    barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        P.overlaps()
        kern_ms.append(P.kernel_stats()[0])
    e1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    ck = clocks.stop()
    _, l1 = P.kernel_stats()
    step_ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    g = P.graph()
    probes = g.probes
    wide = g.wide_reads
    ne = len(g.dest)

    # ---- end to end through the public API with host buffers
    pinned = torch.empty((nr, L), dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = rd
    e2e_ms = []
    parts = []
    h2d = nr * L
    d2h = 0
    gg = None                              # host output arrays, reused from step to step
    for s in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        P.set_reads(pinned.numpy(), t)
        t1 = time.perf_counter()
        P.build_index()
        t2 = time.perf_counter()
        P.overlaps()
        t3 = time.perf_counter()
        gg = P.graph(out=gg)
        t3g = time.perf_counter()
        if s == 0:                         # page-locked host arrays of the graph's sizes, reused
            gg = pq.Graph(**{f: torch.empty(max(getattr(gg, f).nbytes, 1), dtype=torch.uint8, pin_memory=True)
                             .numpy()[:getattr(gg, f).nbytes].view(getattr(gg, f).dtype)
                             for f in ("num_B", "num_F", "olp_B", "olp_F", "edge_off", "dest", "length",
                                       "etype", "trans")})
        d2h = sum(a.nbytes for a in (gg.num_B, gg.num_F, gg.olp_B, gg.olp_F, gg.edge_off, gg.dest,
                                      gg.length, gg.etype, gg.trans))
        torch.cuda.synchronize(dev)
        t4 = time.perf_counter()
        if s > 0:                          # first pass is a warm-up
            e2e_ms.append((t4 - t0) * 1e3)
            sm, fm, _ = P.stage_ms()
            parts.append({"set_reads_ms": (t1 - t0) * 1e3, "build_index_ms": (t2 - t1) * 1e3,
                          "sort_ms": sm, "fm_ms": fm, "search_ms": (t3 - t2) * 1e3,
                          "graph_d2h_ms": (t4 - t3) * 1e3, "graph_call_ms": (t3g - t3) * 1e3})
    e2e_ms_med = max_over_ranks(statistics.median(e2e_ms)) if e2e_ms else None

    if rank != 0:
        return
    peak, peak_kind = measured_peak_hbm()
    kms = statistics.median(kern_ms)
    cb = None
    if world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(args.workload, args.cpu_scale, args.cpu_seconds)
    # Algorithmic bytes: 32 B for every rank probe the reference's method takes on this workload
    # shape (counted by the C restatement on the CPU sample, or the figure recorded beside the ncu
    # summary), whatever the GPU kernels skip.
    oracle_ppr = cb["probes_per_read"] if cb else profile_figure("oracle_probes_per_read")
    alg_bytes = 32.0 * oracle_ppr * nr if oracle_ppr else 32.0 * probes
    achieved = alg_bytes / (kms * 1e-3) / 1e9
    tpr = profile_figure("dram_bytes_per_read")
    out = {
        "metric": METRIC, "value": replica_throughput(nr, world, step_ms), "unit": "reads/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int%d-index" % width, "data": "synthetic",
        "config": {"workload": args.workload, "genome_scale": args.scale, "reads": nr,
                   "read_len": L, "t": t, "index": "U%d" % width, "suffixes_per_index": n,
                   "edges": ne, "wide_tier_reads": wide, "seed_k": min(12, t),
                   "l2": "inputs larger than L2 (two FM-indexes %.2f GB + reads %.2f GB)"
                         % (2 * (n // 64 + 1) * 32 / 1e9, n / 1e9),
                   "parallelism": "replica per GPU" if world > 1 else "single GPU"},
        "sort": {"value": 2 * n / (sort_ms_med * 1e-3) / 1e6, "unit": "Msuffix/s",
                 "ms_fw_plus_bw": sort_ms_med},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "kernel": "k_search_lean (+ k_search_fast over handed-over reads)",
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "reference_probes_per_read": oracle_ppr,
                     "probes_per_read": probes / max(nr, 1), "kernel_ms": kms,
                     "traffic": (tpr * nr) if tpr else None},
        "gpu_launches": int(l1 - l0),
        "e2e": ({"value": replica_throughput(nr, world, e2e_ms_med), "unit": "reads/s",
                 "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                 "ms_per_step": e2e_ms_med, "parts_last_step": parts[-1]} if e2e_ms_med else None),
    }
    if ck:
        out["clocks"] = ck
    if not args.no_modes:
        out["seed_modes"] = seed_modes(P, nr, max(1, min(args.steps, 3)))
    if args.batched_scale > 0:
        out["batched"] = batched(args.batched_scale, max(1, min(args.steps, 3)), local, stream)
    if cb:
        out["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(out), flush=True)
    P.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
