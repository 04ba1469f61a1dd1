#!/usr/bin/env python3
"""Benchmark of the random-walk hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--config c2|c2s|c1|c0|c3|c3s|c4]

Workloads (synthetic RMAT graphs, a=.57 b=.19 c=.19 d=.05, seed 1, isolated
vertices removed, stand in for the reference's datasets, which are absent):
  c2 (default): out-of-core PPR -- RMAT(2^30 vertices, 2^33 edges), 32 MiB
      partitions in pinned host memory, -p 256 (the graph gets 256 x 32 MiB =
      8 GiB of device memory, the vertex index included), walker pool 2^28
      (-b), W = 2|V| walks from source 0, stop probability 0.15.  One step =
      one full run from a cold device cache, through the public API
      (lt_run_ppr with a host count buffer): every partition load, zero-copy
      read and walker spill is inside the timed region.  `value` is the
      learned scheduler (wave runs, cache slots by predicted visits); beside
      it under "variants": the plain (reference) scheduler, the plain
      scheduler at the wave runs' calibrated zero-copy threshold (plain_x8),
      the batched / frequency ablations, and learned / plain with the
      reference's slot layout (host index).  Every run of every variant must
      give the first run's counts bit for bit, and the cpu_baseline sample
      must equal the same walkers run through the product.  The line also
      carries serving latency at 1 000 queries/s (learned and plain).
  c2s: the c2 setup scaled down for profiler captures -- RMAT(2^24, 2^28),
      16 of its 32 MiB partitions cached, walker pool 2^22.
  c1: walk-based PageRank on RMAT(2^23, 2^27) resident in HBM (32 MiB
      partitions all cached), 2|V| walkers one per vertex, l = 10, teleport
      when U > 0.85; `value` times lt_walk_device_compact passes (u32 row
      offsets and counters, the layout the engine uses while E and a call's
      counter updates fit 32 bits) on device buffers, with lt_walk_device
      (u64 layout) timed beside it under "u64_layout"; `e2e` is the public
      API with the graph re-copied from pinned host memory.
  c0: PPR on RMAT(2^20, 2^24) resident in HBM, source 0, W = 2|V|.
  c3: batched multi-source PPR on RMAT(2^26, 2^30) resident in HBM: 4096
      sources drawn Zipf(s = 1.1) over the out-degree rank, walks per source
      lognormal (median 1e4, sigma 1.5 -- values the workload description
      leaves open) clipped to [1e3, 1e6], stop probability 0.15, per-source
      u32 sparse counts; `value` times lt_ppr_batch_device (the captured
      batch pipeline) on device buffers after the autotuner, `e2e` lt_ppr_batch
      with host buffers.
  c3s: c3 scaled down for profiler captures -- RMAT(2^22, 2^26), 256 sources.
  c4: serving PPR on the c2 graph and cache: Poisson arrivals at 100, 1 000
      and 10 000 queries/s, uniform random sources, lognormal walk counts
      (median 1e4, sigma 1.0 -- left open by the workload) clipped to
      [1e3, 1e5]; continuous batching through lt_serve_*; p50 / p99 latency
      and steps/s per rate for the learned and the plain scheduler, and for
      wave steps with least-recently-used slots (batched, ablation).
Steps per run: hops taken (PPR, the reference's 2|V|/0.15 estimate counted
exactly) or updates (PageRank, W * l).
--impl reference times the CPU restatement of the reference walk semantics
(oracle/, OpenMP over all host cores; its update rules pinned to the
reference's own App::update code) on a bounded sample of the same workload
per step (SAMPLES); its input graph comes from the oracle's CPU generator,
so that arm uses neither the GPU nor this repository's library.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "c2": dict(workload="ppr-rmat30-e33-outofcore-p256-b2^28", app=0, scale=30, edges=1 << 33, length=0,
               start=0, prob=0.15, part_mb=32, partitions=256, batch=1 << 28),
    "c2s": dict(workload="ppr-rmat24-e28-outofcore-p16-b2^22", app=0, scale=24, edges=1 << 28, length=0,
                start=0, prob=0.15, part_mb=32, partitions=16, batch=1 << 22),
    "c1": dict(workload="pagerank-rmat23-e27-resident", app=1, scale=23, edges=1 << 27, length=10,
               start=2, prob=0.85, part_mb=32),
    "c0": dict(workload="ppr-rmat20-e24-resident", app=0, scale=20, edges=1 << 24, length=0,
               start=0, prob=0.15, part_mb=32),
    "c4": dict(workload="serve-ppr-rmat30-e33-outofcore-p256", app=0, scale=30, edges=1 << 33, length=0,
               start=0, prob=0.15, part_mb=32, partitions=256, batch=1 << 28, serving=True,
               rates=(100, 1000, 10000), seconds=(4.0, 2.0, 1.0), walk_median=1e4, walk_sigma=1.0,
               walk_min=1e3, walk_max=1e5),
    "c3": dict(workload="ppr-batch4096-zipf1.1-lognormal-rmat26-e30", app=0, scale=26, edges=1 << 30, length=0,
               start=0, prob=0.15, part_mb=32, queries=4096, zipf=1.1, walk_median=1e4, walk_sigma=1.5,
               walk_min=1e3, walk_max=1e6, batch_queries=True),
    "c3s": dict(workload="ppr-batch256-zipf1.1-lognormal-rmat22-e26", app=0, scale=22, edges=1 << 26, length=0,
                start=0, prob=0.15, part_mb=32, queries=256, zipf=1.1, walk_median=1e4, walk_sigma=1.5,
                walk_min=1e3, walk_max=1e6, batch_queries=True),
}
SEED_GRAPH = 1
SEED_WALK = 1


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--config", default="c2", choices=sorted(CONFIGS))
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="target CPU time of the cpu_baseline sample")
    p.add_argument("--no-autotune", action="store_true",
                   help="out-of-core configs: run with the default knobs instead of the autotuner's")
    p.add_argument("--variants", default="",
                   help="out-of-core configs: comma-separated subset of the variants to run (profiler "
                        "captures; the line then carries no comparisons and no serving)")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


# ------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, line in self.lines:
            if t < t0 or t > t1:
                continue
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak(key, fallback):
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)[key]), "measured"
    return fallback, "fallback"


def profiled_traffic(workload):
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f).get(workload)
    return None


# ---------------------------------------------------------- CPU oracle

# Oracle sample of each workload: the same bounded piece of the workload for
# the reference arm (one sample per step) and the cpu_baseline leg (repeated
# samples, median), so the two CPU figures measure identical work.
#   walkers: the first n walkers of the run; queries: the first n queries.
SAMPLES = {"c2": dict(walkers=1 << 22), "c2s": dict(walkers=1 << 20), "c4": dict(walkers=1 << 22),
           "c1": dict(walkers=None), "c0": dict(walkers=None), "c3": dict(queries=64), "c3s": dict(queries=64)}


def cpu_sample(name, cfg, rp, col, threads):
    """One oracle run over the workload's sample.  Returns (steps, seconds,
    outputs, description): PPR / PageRank counts of the first n walkers, or
    the per-query counts of the first n queries."""
    import oracle
    V = len(rp) - 1
    W = 2 * V
    smp = SAMPLES[name]
    t = time.perf_counter()
    if cfg.get("batch_queries"):
        sources, walkers, seeds = c3_queries(cfg, rp)
        q = min(smp["queries"], len(sources))
        outs, hops = [], 0
        for i in range(q):
            c, _, st = oracle.ppr(rp, col, int(sources[i]), int(walkers[i]), prob=cfg["prob"], seed=int(seeds[i]),
                                  threads=threads)
            nz = np.nonzero(c)[0]
            outs.append((nz, c[nz]))
            hops += int(st[1])
        dt = time.perf_counter() - t
        return hops, dt, outs, f"first {q} of {len(sources)} queries ({hops} hops)"
    n = min(W, smp["walkers"] or W)
    if cfg["app"] == 1:
        c, st = oracle.pagerank(rp, col, n, length=cfg["length"], alpha=cfg["prob"], seed=SEED_WALK,
                                start_mode=cfg["start"], threads=threads)
        steps = int(st[0])
    else:
        c, _, st = oracle.ppr(rp, col, 0, n, prob=cfg["prob"], seed=SEED_WALK, threads=threads)
        steps = int(st[1])
    dt = time.perf_counter() - t
    return steps, dt, c, f"first {n} of {W} walkers ({steps} steps)"


def cpu_baseline_leg(name, cfg, rp, col, seconds):
    """cpu_baseline: the oracle sample repeated until about `seconds` of CPU
    work (at least 3 samples), median rate; also returns the sample's
    outputs for the parity check against the product.

    The sample runs in a child process that has no CUDA context, as the
    reference arm's process has none: on the GB300's Grace host a CUDA
    context in the process slows the oracle's random reads of the graph by
    about 38 % (the c2 sample: 31 -> 19 M steps/s on the same arrays before
    and after the context was created).  The graph reaches the child through
    an in-memory file (memfd); the outputs come back pickled."""
    import mmap
    import pickle
    rp = np.ascontiguousarray(rp, dtype=np.uint64)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    nbytes = rp.nbytes + col.nbytes
    fd = os.memfd_create("lt_cpu_leg")
    try:
        os.ftruncate(fd, nbytes)
        m = mmap.mmap(fd, nbytes)
        np.frombuffer(m, dtype=np.uint64, count=len(rp))[:] = rp
        np.frombuffer(m, dtype=np.uint32, count=len(col), offset=rp.nbytes)[:] = col
        m.close()
        out = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-leg-child", str(fd), str(len(rp)),
                              str(len(col)), name, repr(seconds)], pass_fds=(fd,), stdout=subprocess.PIPE,
                             check=True).stdout
    finally:
        os.close(fd)
    cpu, res = pickle.loads(out)
    if isinstance(res, tuple) and res and res[0] == "sparse":
        _, n, nz, vals = res
        res = np.zeros(n, dtype=vals.dtype)
        res[nz] = vals
    return cpu, res


def cpu_leg_child(argv):
    """Child side of cpu_baseline_leg (no CUDA, no library of this
    repository): maps the graph, runs the sample, pickles the result."""
    import mmap
    import pickle
    fd, nrp, ncol, name, seconds = int(argv[0]), int(argv[1]), int(argv[2]), argv[3], float(argv[4])
    m = mmap.mmap(fd, 8 * nrp + 4 * ncol, prot=mmap.PROT_READ)
    rp = np.frombuffer(m, dtype=np.uint64, count=nrp)
    col = np.frombuffer(m, dtype=np.uint32, count=ncol, offset=8 * nrp)
    cpu, res = _cpu_baseline_here(name, CONFIGS[name], rp, col, seconds)
    if isinstance(res, np.ndarray):
        nz = np.nonzero(res)[0]
        res = ("sparse", len(res), nz, res[nz])
    sys.stdout.buffer.write(pickle.dumps((cpu, res), protocol=pickle.HIGHEST_PROTOCOL))
    sys.stdout.flush()
    return 0


def _cpu_baseline_here(name, cfg, rp, col, seconds):
    """The sample loop of cpu_baseline_leg, in this process."""
    threads = os.cpu_count() or 1
    rates, out, desc, total = [], None, "", 0.0
    while len(rates) < 3 or (total < seconds and len(rates) < 20):
        steps, dt, out, desc = cpu_sample(name, cfg, rp, col, threads)
        rates.append(steps / dt)
        total += dt
    value = statistics.median(rates)
    return ({"value": value, "unit": "steps/s", "cores": threads, "kind": "port",
             "sample": f"{desc}; median of {len(rates)} samples, {total:.1f} s of CPU work"}, out)


def workload_config(name, cfg, V, E, P):
    """The workload the line is measured on (identical in both arms)."""
    c = {"workload": cfg["workload"], "V": V, "E": E, "partitions": P, "partition_mb": cfg["part_mb"]}
    if "partitions" in cfg:
        c.update({"cached_partitions": cfg["partitions"],
                  "device_graph_bytes": cfg["partitions"] * (cfg["part_mb"] << 20),
                  "walker_pool": cfg["batch"], "walkers": 2 * V, "source": 0, "prob": cfg["prob"],
                  "l2": "graph (%d GiB) in host memory, far larger than L2; device cache dropped before every step"
                        % ((8 * (V + 1) + 4 * E) >> 30)})
    elif cfg.get("batch_queries"):
        c.update({"queries": cfg["queries"], "zipf": cfg["zipf"],
                  "walks": "lognormal median %g sigma %g in [%g, %g]" % (cfg["walk_median"], cfg["walk_sigma"],
                                                                         cfg["walk_min"], cfg["walk_max"]),
                  "prob": cfg["prob"], "l2": "graph (%d MiB) larger than L2, no flush" % ((8 * (V + 1) + 4 * E) >> 20)})
    else:
        gb = 8 * (V + 1) + 4 * E
        c.update({"walkers": 2 * V, "length": cfg["length"], "prob": cfg["prob"], "start": cfg["start"],
                  "l2": ("inputs larger than L2 (graph %d MiB > 129 MB L2), no flush" % (gb >> 20)) if gb > 129e6
                  else "graph (%d MiB) fits in L2 and is not flushed: a parity case, not a bench line" % (gb >> 20)})
    return c


def reference_arm(args, cfg):
    """The CPU restatement of the reference's walk semantics (oracle/, its
    App::update pinned to the reference's own code) on the host cores, over
    a bounded sample of the same workload per step.  The input graph is made
    by the oracle's CPU generator (bit-identical to the GPU generator): no
    GPU and no library of this repository is used in this arm."""
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    import oracle
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    rp, col = oracle.rmat(cfg["scale"], cfg["edges"], seed=SEED_GRAPH)
    node_off, _ = oracle.partition(rp, cfg["part_mb"] << 20)
    setup_s = time.perf_counter() - t0
    V, E, P = len(rp) - 1, len(col), len(node_off) - 1
    rates, desc, total = [], "", 0.0
    for i in range(args.warmup + args.steps):
        steps, dt, _, desc = cpu_sample(args.config, cfg, rp, col, threads)
        if i >= args.warmup:
            rates.append(steps / dt)
            total += dt
    value = statistics.median(rates)
    line = {
        "impl": "reference", "metric": "walk steps/s", "value": value, "unit": "steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / len(rates) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic RMAT (seeded), stand-in for the reference datasets",
        "config": workload_config(args.config, cfg, V, E, P),
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": threads, "kind": "port",
                         "sample": f"{desc} per step; median of {len(rates)} steps"},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup": {"graph_generation_s": setup_s, "generator": "oracle (CPU, OpenMP)"},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------ GB300 arm

def init_dist():
    """One process per GPU (replicas): the process group exists only for the
    barrier around the timed region and the max over ranks of its time."""
    import torch
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    return ws, rank, local, dist


def max_over_ranks(dist, local, x):
    if not dist:
        return x
    import torch
    dev = f"cuda:{local}" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def link_bytes(s):
    return s["h2d_graph_bytes"] + s["h2d_walker_bytes"] + s["d2h_walker_bytes"] + s["zerocopy_bytes"]


def serve_rate(lt, e, cfg, V, rate, seconds, seed):
    """Serve a Poisson trace at `rate` queries/s on engine e (continuous
    batching through lt_serve_*); p50 / p99 latency from arrival to result."""
    srv = lt.Server(e, max_active=4096, table_slots=1 << 27, prob=cfg["prob"])
    t, src, w, seeds = serve_trace(cfg, V, rate, seconds, seed)
    n = len(t)
    lat = []
    nxt = 0
    t0 = lt.Server.now_ms()
    while len(lat) < n:
        now = lt.Server.now_ms() - t0
        while nxt < n and t[nxt] <= now:
            srv.submit(int(src[nxt]), int(w[nxt]), int(seeds[nxt]), arrival_ms=t0 + float(t[nxt]))
            nxt += 1
        c, a, p = srv.step()
        if c:
            for tk in srv.finished():
                lat.append(srv.latency_ms(tk))
                srv.result(tk)
        if a == 0 and p == 0 and nxt < n:
            time.sleep(max(0.0, (t[nxt] - (lt.Server.now_ms() - t0)) / 1e3))
    span_s = (lt.Server.now_ms() - t0) / 1e3
    srv.close()
    st = e.stats()
    lat = np.array(lat)
    return {"queries": n, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "span_s": span_s, "walkers": int(w.sum()), "steps": st["moves"], "steps_per_s": st["moves"] / span_s,
            "bytes_per_step": link_bytes(st) / max(1, st["moves"]), "iterations": st["iterations"],
            "partition_loads": st["partition_loads"]}


def spread(xs):
    return {"min": min(xs), "median": statistics.median(xs), "max": max(xs),
            "stdev": statistics.stdev(xs) if len(xs) > 1 else 0.0}


def gb300_ooc(args, cfg):
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        # torch only for the barrier and the max over ranks of a replica run
        ws, rank, local, dist = init_dist()
    import lighttraffic_gb300 as lt

    g = lt.Graph.rmat(cfg["scale"], cfg["edges"], seed=SEED_GRAPH, part_bytes=cfg["part_mb"] << 20, device=local)
    V, E, P = g.num_nodes, g.num_edges, g.num_partitions
    W = 2 * V
    # the CPU leg first, before the GPU has worked (the host cores share the
    # module's power with the GPU: measured after the timed runs, the same
    # sample ran 36 % slower than in the reference arm's fresh process)
    cpu, sample_counts = None, None
    if not args.no_cpu_baseline and ws == 1:
        rp, col = g.csr_views()
        cpu, sample_counts = cpu_baseline_leg(args.config, cfg, rp, col, args.cpu_seconds)
        del rp, col
    link_peak = lt.host_link_gbs(local)
    gather_peak = lt.host_gather_gbs(local)
    counts = lt.pinned_empty(V, np.uint64)   # host count buffer in page-locked memory
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    thr_ref = (cfg["part_mb"] << 20) // 128 // 2   # src/Scheduler.h:295
    # learned = the headline; plain = the reference policy (one partition per
    # iteration, its zero-copy threshold, load / compute overlap on);
    # plain_x8 = the same at the threshold the wave runs use (x8: 32 B per
    # zero-copy hop measured, against the 256 B the reference's rule
    # assumes); batched / frequency = wave runs without predictions / with a
    # moving average; *_host_index = the reference's slot layout (rowptr
    # slices travel with the partitions).  The default layout keeps the
    # vertex index on the device inside the -p budget (fewer slots).
    variants = {"learned": dict(sched=lt.SCHED_LEARNED), "plain": dict(sched=lt.SCHED_PLAIN),
                "plain_x8": dict(sched=lt.SCHED_PLAIN, zerocopy_threshold=8 * thr_ref),
                "batched": dict(sched=lt.SCHED_BATCHED), "frequency": dict(sched=lt.SCHED_FREQUENCY),
                "learned_host_index": dict(sched=lt.SCHED_LEARNED, resident_index=False),
                "plain_host_index": dict(sched=lt.SCHED_PLAIN, resident_index=False),
                "learned_tier50": dict(sched=lt.SCHED_LEARNED, hot_tier=50)}
    # named only through --variants: wave runs that read every uncached
    # partition zero-copy in each kernel (no bounded groups), bounded groups
    # of other footprints, no prefill, every bucketing pass planned by the
    # host, 2048-walker bucketing tiles (two CTAs per SM), and hot-vertex
    # tiers of 25-75 % of the graph budget
    extra = {"learned_sweep": dict(sched=lt.SCHED_LEARNED, zc_group_bytes=1 << 62, sweep_walkers=1 << 62),
             "learned_zc2g": dict(sched=lt.SCHED_LEARNED, zc_group_bytes=2 << 30),
             "learned_zc8g": dict(sched=lt.SCHED_LEARNED, zc_group_bytes=8 << 30),
             "learned_noprefill": dict(sched=lt.SCHED_LEARNED, prefill=False),
             "frequency_noprefill": dict(sched=lt.SCHED_FREQUENCY, prefill=False),
             "learned_hostplan": dict(sched=lt.SCHED_LEARNED, host_plan=True),
             "learned_tile2k": dict(sched=lt.SCHED_LEARNED, bucket_items=8),
             "learned_nosplit": dict(sched=lt.SCHED_LEARNED, split=False),
             "learned_nosweep": dict(sched=lt.SCHED_LEARNED, sweep_walkers=1),
             "learned_zc256m": dict(sched=lt.SCHED_LEARNED, zc_group_bytes=256 << 20),
             "learned_zc1g": dict(sched=lt.SCHED_LEARNED, zc_group_bytes=1 << 30),
             "learned_lf4": dict(sched=lt.SCHED_LEARNED, load_factor=4),
             "learned_lf16": dict(sched=lt.SCHED_LEARNED, load_factor=16),
             "learned_sweep2m": dict(sched=lt.SCHED_LEARNED, sweep_walkers=1 << 21),
             "learned_tier25": dict(sched=lt.SCHED_LEARNED, hot_tier=25),
             "learned_tier75": dict(sched=lt.SCHED_LEARNED, hot_tier=75),
             "frequency_tier50": dict(sched=lt.SCHED_FREQUENCY, hot_tier=50)}
    if args.variants:
        keep = args.variants.split(",")
        variants = {k: v for k, v in {**variants, **extra}.items() if k in keep}
        assert variants, f"no variant among {keep}"
    K = args.steps
    n_timed = {"learned": K, "batched": K, "frequency": K, "plain": min(K, 5), "plain_x8": min(K, 5),
               "learned_host_index": min(K, 3), "plain_host_index": min(K, 3), "learned_tier50": min(K, 5)}
    n_timed.update({k: K for k in extra})
    engines = {}
    ref_counts = [None]
    checked = [0]
    first_run = {}       # the process's first run (for a profiler capture of exactly its step kernels)

    def one_run(name):
        # one engine per variant for the whole benchmark (its pinned host
        # spill slabs and the prefetcher's training persist); the device
        # cache is emptied before every run, so each run starts cold
        if name not in engines:
            engines[name] = lt.Engine(g, partitions=cfg["partitions"], batch=cfg["batch"], seed=SEED_WALK,
                                      device=local, **variants[name])
        e = engines[name]
        e.drop_cache()
        t0 = time.perf_counter()
        e.ppr(0, W, cfg["prob"], out=counts)
        t1 = time.perf_counter()
        # every run of every variant must give the first run's counts, bit
        # for bit (outside the timed interval)
        if ref_counts[0] is None:
            assert int(counts.sum()) == W, "PPR invariant (one count per walk) violated"
            ref_counts[0] = counts.copy()
        else:
            assert np.array_equal(counts, ref_counts[0]), f"{name}: counts differ from the first run"
        checked[0] += 1
        st = e.stats()
        if not first_run:
            first_run.update(sched=name, step_launches=st["computing_calls"] + st["zerocopy_calls"],
                             zero_copy_bytes=st["zerocopy_bytes"])
        return (t1 - t0, st, e.policy_stats())

    # the out-of-core autotuner on the headline engine; the ablations get the
    # same wave knobs and every variant the same grid and bucketing tile, so
    # the comparisons differ only in the policy
    tune = None
    if "learned" in variants and not args.no_autotune:
        engines["learned"] = lt.Engine(g, partitions=cfg["partitions"], batch=cfg["batch"], seed=SEED_WALK,
                                       device=local, **variants["learned"])
        tune = engines["learned"].autotune()
        shared = dict(ctas_per_sm=tune["ctas_per_sm"], bucket_items=tune["bucket_items"])
        wave = dict(zc_group_bytes=tune["zc_group_bytes"], load_factor=tune["load_factor"])
        for name in variants:
            if name == "learned":
                continue
            # a variant's own knobs (e.g. learned_zc2g's group size) win
            variants[name] = {**shared,
                              **(wave if name.split("_")[0] in ("batched", "frequency", "learned")
                                 and "host_index" not in name else {}),
                              **variants[name]}
    for i in range(args.warmup):
        for name in variants:
            if i == 0 or name == "learned":
                one_run(name)
    if dist:
        dist.barrier()
    wall0 = time.time()
    times = {name: [] for name in variants}
    stats, pstats = {}, {}
    order = list(variants)
    for k in range(K):
        for name in (order if k % 2 == 0 else order[::-1]):
            if k < n_timed[name]:
                dt, st, ps = one_run(name)
                times[name].append(dt)
                stats[name], pstats[name] = st, ps
    wall1 = time.time()
    # host-link bandwidth again after the timed runs: on these shared hosts it
    # can drop during a call (contention outside this process)
    link_after = lt.host_link_gbs(local)
    res = {}
    for name in variants:
        st = stats[name]
        el = max_over_ranks(dist, local, sum(times[name]))
        res[name] = {"value": st["moves"] * len(times[name]) * ws / el,
                     "bytes_per_step": link_bytes(st) / st["moves"],
                     "ms_per_step": el / len(times[name]) * 1e3, "runs": len(times[name]),
                     "iterations": st["iterations"], "partition_loads": st["partition_loads"],
                     "refill_loads": st["refill_loads"], "prefill_loads": st["prefill_loads"],
                     "zerocopy_groups": st["zerocopy_groups"], "zerocopy_sweeps": st["zerocopy_sweeps"],
                     "overlap_computes": st["overlap_computes"], "device_plans": st["device_plans"],
                     "hot_vertices": st["hot_vertices"], "split_launches": st["split_launches"],
                     "cache_slots": st["cache_slots"],
                     "index_on_device": bool(st["index_on_device"]), "step_s": spread(times[name]),
                     # where one run's time goes (last run): CUDA-event time of
                     # the step kernels on cached queues / zero-copy sets, of
                     # the bucketing kernels and of the partition copies; host
                     # time blocked on each iteration's step kernel; wall time
                     "run_ms": {"computing": st["computing_ms"], "zero_copy": st["zerocopy_ms"],
                                "bucketing": st["bucket_ms"], "graph_loading": st["graph_loading_ms"],
                                "host_wait": st["host_wait_ms"], "running": st["running_ms"]},
                     # host time outside waits, by phase (last run)
                     "host_ms": {"sched": st["host_sched_ms"], "submit": st["host_submit_ms"],
                                 "replay": st["host_replay_ms"], "observe": st["host_observe_ms"]}}
        if pstats[name]["name"] in ("learned", "frequency"):
            res[name]["policy"] = pstats[name]
        ps = engines[name].partition_stats()
        vis, cvis = ps["visits"].astype(np.float64), ps["cached_visits"].astype(np.float64)
        top = np.sort(vis)[::-1][: st["cache_slots"]].sum()
        # share of partition entries that found their partition cached, and
        # what the best fixed set of cache_slots partitions would have caught
        res[name]["cache"] = {"entries": int(vis.sum()), "cached_share": float(cvis.sum() / max(1.0, vis.sum())),
                              "best_fixed_set_share": float(top / max(1.0, vis.sum()))}

    # serving latency on the same graph and cache (the c4 workload at 1 000
    # queries/s), learned against the reference loop
    serving = {}
    c4 = CONFIGS["c4"]
    for name in ("learned", "plain"):
        if name in engines:
            serving[name] = serve_rate(lt, engines[name], c4, V, 1000, 2.0, SEED_WALK + 1000)
    clocks.stop()
    clk = clocks.summary(wall0 - 0.5, wall1)
    if args.variants:
        print(json.dumps({"profile_run": True, "config": workload_config(args.config, cfg, V, E, P),
                          "variants": res, "autotune": tune, "first_run": first_run}), flush=True)
        for e in engines.values():
            e.close()
        return 0

    # the oracle sample of the cpu_baseline leg, and the same walkers through
    # the product: identical counts
    parity = {"cross_variant_runs_identical": checked[0]}
    if sample_counts is not None:
        n = SAMPLES[args.config]["walkers"] or W
        got = engines["learned"].ppr(0, min(n, W), cfg["prob"])
        assert np.array_equal(got, sample_counts), "product and oracle differ on the sample"
        parity["oracle_sample_identical"] = {"walkers": min(n, W), "identical": True}
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    L, Pn, P8 = res["learned"], res["plain"], res["plain_x8"]
    s = stats["learned"]
    value = L["value"]
    el_learned = L["ms_per_step"] / 1e3
    launches = s["computing_calls"] + s["zerocopy_calls"]
    # step kernel, HBM side: 20 B per hop (rowptr pair + col), 16 B per count
    # (one per walk), 48 B per hand-off (walker read + staged write + scatter
    # read + queue write, 12 B each)
    alg = 20 * s["moves"] + 16 * W + 48 * s["handoffs"]
    kern_s = max(s["step_kernel_ms"], 1e-6) / 1e3
    hbm_peak, peak_src = measured_peak("hbm_gbs", 6800.0)
    run_link = link_bytes(s)
    stronger = Pn if Pn["value"] >= P8["value"] else P8
    line = {
        "metric": "walk steps/s", "value": value, "unit": "steps/s", "n_gpus": ws, "steps": K,
        "warmup": args.warmup, "ms_per_step": L["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic RMAT (seeded), stand-in for the reference datasets",
        "config": workload_config(args.config, cfg, V, E, P),
        "scheduler": "learned (wave runs, cache slots by the online-trained network's predicted visits)",
        "layout": "compact vertex index on the device (u32 offsets within each partition, %d MiB) inside "
                  "the %d MiB graph budget: %d partition slots"
                  % ((4 * (V + 1)) >> 20, cfg["partitions"] * cfg["part_mb"], s["cache_slots"]),
        # The dominant kernel of an out-of-core run is the step kernel on
        # zero-copy sets: each zero-copy hop reads one 4-byte column entry
        # from pinned host memory, and the link moves its 32-byte sector
        # (31.9 B per hop, ncu).  Its roofline is the GPU's random-sector
        # read rate from host memory, measured in this run; the whole run's
        # host-link bytes (loads + zero-copy + spills) over its time against
        # the copy engine's pinned H2D rate is under "run".
        "roofline": {"bound": "host_link", "kernel": "walk_part_kernel, zero-copy launches",
                     "achieved": s["zerocopy_bytes"] / max(s["zerocopy_ms"], 1e-6) * 1e3 / 1e9,
                     "peak": gather_peak, "unit": "GB/s",
                     "frac": s["zerocopy_bytes"] / max(s["zerocopy_ms"], 1e-6) * 1e3 / 1e9 / gather_peak,
                     "traffic": s["zerocopy_bytes"] / max(1, s["zerocopy_calls"]),
                     "traffic_is": "host-link bytes per zero-copy launch: 32 B sector per zero-copy hop (ncu)",
                     "alg_bytes_per_launch": 4 * s["zerocopy_bytes"] / 32 / max(1, s["zerocopy_calls"]),
                     "mean_launch_ms": s["zerocopy_ms"] / max(1, s["zerocopy_calls"]),
                     "launches": s["zerocopy_calls"],
                     "peak_source": "random 32 B sector reads from mapped pinned host memory, measured in this "
                                    "run (lt_host_gather_gbs)",
                     "run": {"achieved": run_link / el_learned / 1e9, "peak": link_peak, "unit": "GB/s",
                             "frac": run_link / el_learned / 1e9 / link_peak, "bytes_per_run": run_link,
                             "is": "graph H2D + zero-copy + walker spill bytes over the run time, against the "
                                   "pinned H2D copy rate measured in this run"},
                     "hbm": {"kernel": "walk_part_kernel", "achieved": alg / kern_s / 1e9, "peak": hbm_peak,
                             "unit": "GB/s", "frac": alg / kern_s / 1e9 / hbm_peak,
                             "alg_bytes_per_launch": alg / max(1, launches),
                             "mean_launch_ms": s["step_kernel_ms"] / max(1, launches), "launches": launches,
                             "traffic": profiled_traffic(cfg["workload"]), "peak_source": peak_src}},
        "host_link": {"bytes_per_step": run_link / s["moves"], "achieved_gbs": run_link / el_learned / 1e9,
                      "peak_gbs": link_peak, "gather_peak_gbs": gather_peak,
                      "peak_gbs_after_timed_runs": link_after,
                      "bytes_by_kind": {"graph_loads": s["h2d_graph_bytes"], "zero_copy": s["zerocopy_bytes"],
                                        "walker_spill": s["h2d_walker_bytes"] + s["d2h_walker_bytes"]},
                      "first_run": first_run,
                      "zerocopy_bytes": "32 B per zero-copy hop with the vertex index on the device (62 B "
                                        "without), measured with ncu"},
        "variants": res,
        "autotune": tune,
        "learned_over_plain": {
            "vs_plain": {"steps_per_s": value / Pn["value"], "bytes_per_step": L["bytes_per_step"] / Pn["bytes_per_step"]},
            "vs_plain_x8": {"steps_per_s": value / P8["value"], "bytes_per_step": L["bytes_per_step"] / P8["bytes_per_step"]},
            "vs_stronger_plain": {"which": "plain" if stronger is Pn else "plain_x8",
                                  "steps_per_s": value / stronger["value"],
                                  "bytes_per_step": L["bytes_per_step"] / stronger["bytes_per_step"]},
            "host_index_layout": {
                "steps_per_s": res["learned_host_index"]["value"] / res["plain_host_index"]["value"],
                "bytes_per_step": res["learned_host_index"]["bytes_per_step"] / res["plain_host_index"]["bytes_per_step"]}},
        "learned_over_ablations": {n: {"steps_per_s": value / res[n]["value"],
                                       "bytes_per_step": L["bytes_per_step"] / res[n]["bytes_per_step"]}
                                   for n in ("batched", "frequency")},
        # half the graph budget as a hot-vertex tier (built from the first
        # run's counts): fewer host-link bytes per step, at this cost in steps/s
        "hot_tier_50": {"steps_per_s": res["learned_tier50"]["value"] / value,
                        "bytes_per_step": res["learned_tier50"]["bytes_per_step"] / L["bytes_per_step"],
                        "hot_vertices": res["learned_tier50"]["hot_vertices"]},
        "serving_1000qps": serving,
        "parity": parity,
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": s["h2d_graph_bytes"] + s["h2d_walker_bytes"],
                "d2h_bytes_per_step": 8 * V + s["d2h_walker_bytes"],
                "note": "each step is a full run through lt_run_ppr from a cold cache with host output buffers"},
        "gpu_launches": s["kernel_launches"] * K,
        "clocks": clk,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    for e in engines.values():
        e.close()
    if dist:
        dist.destroy_process_group()
    return 0


def gb300_resident(args, cfg):
    import torch
    ws, rank, local, dist = init_dist()
    import lighttraffic_gb300 as lt

    g = lt.Graph.rmat(cfg["scale"], cfg["edges"], seed=SEED_GRAPH, part_bytes=cfg["part_mb"] << 20, device=local)
    rp, col = g.csr()
    V, E = g.num_nodes, g.num_edges
    W = 2 * V
    dev = f"cuda:{local}"
    d_rp = torch.from_numpy(rp.view(np.int64)).to(dev)
    d_col = torch.from_numpy(col.view(np.int32)).to(dev)
    d_cnt = torch.zeros(V, dtype=torch.int64, device=dev)
    d_scr = torch.zeros(max(1, lt.lib.lt_walk_scratch_bytes() // 8), dtype=torch.int64, device=dev)
    d_st = torch.zeros(3, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()
    app, start, length, prob = cfg["app"], cfg["start"], cfg["length"], cfg["prob"]
    # compact layout (u32 row offsets and counters), what the engine runs when
    # E and the pass's counter updates fit 32 bits; the u64 layout beside it
    compact_ok = E < (1 << 32) and (W * max(1, length) if app == 1 else W) < (1 << 32)
    d_rp32 = torch.zeros(V + 1, dtype=torch.int32, device=dev)
    d_cnt32 = torch.zeros(V, dtype=torch.int32, device=dev)
    if compact_ok:
        lt.check(lt.lib.lt_rowptr_narrow(d_rp.data_ptr(), d_rp32.data_ptr(), V, stream.cuda_stream))

    def launch_std():
        d_cnt.zero_()
        lt.check(lt.lib.lt_walk_device(app, start, d_rp.data_ptr(), d_col.data_ptr(), V, 0, W, length,
                                       ctypes.c_float(prob), 0, SEED_WALK, d_cnt.data_ptr(), None, None,
                                       d_scr.data_ptr(), d_st.data_ptr(), stream.cuda_stream))

    # packed layout: row offset and counter of a vertex side by side
    d_rows = torch.zeros(2 * (V + 1), dtype=torch.int32, device=dev)

    def launch_packed():
        lt.check(lt.lib.lt_rows_pack(d_rp.data_ptr(), d_rows.data_ptr(), V, stream.cuda_stream))
        lt.check(lt.lib.lt_walk_device_packed(app, start, d_rows.data_ptr(), d_col.data_ptr(), V, 0, W, length,
                                              ctypes.c_float(prob), 0, SEED_WALK, None, None, d_scr.data_ptr(),
                                              d_st.data_ptr(), stream.cuda_stream))

    def launch_compact():
        d_cnt32.zero_()
        lt.check(lt.lib.lt_walk_device_compact(app, start, d_rp32.data_ptr(), d_col.data_ptr(), V, 0, W, length,
                                               ctypes.c_float(prob), 0, SEED_WALK, d_cnt32.data_ptr(), None, None,
                                               d_scr.data_ptr(), d_st.data_ptr(), stream.cuda_stream))

    def timed(launch):
        for _ in range(args.warmup):
            launch()
        torch.cuda.synchronize()
        d_st.zero_()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0.record()
        for i in range(args.steps):
            starts[i].record()
            launch()
            ends[i].record()
        t1.record()
        torch.cuda.synchronize()
        el = max_over_ranks(dist, local, t0.elapsed_time(t1))
        st = d_st.cpu().numpy().astype(np.uint64) // np.uint64(args.steps)
        return el, [x.elapsed_time(y) for x, y in zip(starts, ends)], st

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    wall0 = time.time()
    std_ms, std_kern, std_st = timed(launch_std)
    std_total = int(d_cnt.sum().item())
    packed = None
    if compact_ok:
        elapsed_ms, kern_ms, st = timed(launch_compact)
        total = int(d_cnt32.to(torch.int64).sum().item())
        assert (std_st == st).all(), "compact and u64 layouts took different steps"
        p_ms, p_kern, p_st = timed(launch_packed)
        assert (p_st == st).all(), "packed and compact layouts took different steps"
        assert torch.equal(d_rows[1::2][:V].to(torch.int64), d_cnt32.to(torch.int64)), "packed counts differ"
        packed = {"value": (int(p_st[0]) if app == 1 else int(p_st[1])) * args.steps * ws / (p_ms / 1e3),
                  "ms_per_step": p_ms / args.steps, "mean_launch_ms": statistics.mean(p_kern),
                  "note": "lt_walk_device_packed: rows[2v] first edge, rows[2v+1] counter (the pack kernel is "
                          "inside each timed step: it also clears the counters)"}
    else:
        elapsed_ms, kern_ms, st, total = std_ms, std_kern, std_st, std_total
    updates, moves, tele = (int(x) for x in st)
    steps_per_pass = updates if app == 1 else moves
    assert total == (W * length if app == 1 else W) == std_total, "invariant violated in the timed pass"
    value = steps_per_pass * args.steps * ws / (elapsed_ms / 1e3)
    counter_updates = updates if app == 1 else W
    # algorithmic bytes: row-offset pair + column entry per hop, counter
    # read-modify-write per update, at the width of the layout timed
    ob, cb = (4, 4) if compact_ok else (8, 8)
    alg_bytes = (2 * ob + 4) * moves + 2 * cb * counter_updates
    mean_kern_s = statistics.mean(kern_ms) / 1e3
    peak, peak_src = measured_peak("hbm_gbs", 6800.0)
    achieved = alg_bytes / mean_kern_s / 1e9

    eng = lt.Engine(g, seed=SEED_WALK, device=local)
    host_counts = torch.empty(V, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    e2e_times, h2d = [], 0
    for i in range(args.warmup + max(3, min(args.steps, 10))):
        eng.drop_cache()
        t0 = time.perf_counter()
        if app == 1:
            eng.pagerank(W, length=length, start=start, alpha=prob, out=host_counts)
        else:
            eng.ppr(0, W, prob, out=host_counts)
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append(t1 - t0)
            h2d = eng.stats()["h2d_graph_bytes"]
    e2e_s = statistics.mean(e2e_times)
    clocks.stop()
    clk = clocks.summary(wall0 - 0.5, time.time())
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    line = {
        "metric": "walk steps/s", "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic RMAT (seeded), stand-in for the reference datasets",
        "config": workload_config(args.config, cfg, V, E, g.num_partitions),
        "steps_per_pass": steps_per_pass, "parallelism": "replicas" if ws > 1 else "1 GPU",
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": profiled_traffic(cfg["workload"] + ("-compact" if compact_ok else "")),
                     "kernel": "walk_whole_kernel" + (" (compact layout)" if compact_ok else ""),
                     "alg_bytes_per_launch": alg_bytes, "mean_launch_ms": mean_kern_s * 1e3,
                     "peak_source": peak_src},
        "layout": "compact (u32 row offsets and counters)" if compact_ok else "u64 row offsets and counters",
        "u64_layout": {"value": steps_per_pass * args.steps * ws / (std_ms / 1e3), "ms_per_step": std_ms / args.steps,
                       "mean_launch_ms": statistics.mean(std_kern)},
        "packed_layout": packed,
        "e2e": {"value": steps_per_pass * ws / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 8 * V, "ms_per_step": e2e_s * 1e3},
        "gpu_launches": args.steps,
        "clocks": clk,
        "stats_per_pass": {"updates": updates, "moves": moves, "teleports": tele},
    }
    if not args.no_cpu_baseline and ws == 1:
        # the sample is the whole pass: the oracle's counts equal the product's
        line["cpu_baseline"], want = cpu_baseline_leg(args.config, cfg, rp, col, args.cpu_seconds)
        assert np.array_equal(host_counts, want), "product and oracle counts differ"
        line["parity"] = {"oracle_identical": {"walkers": W, "identical": True}}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def c3_queries(cfg, rp):
    """Zipf(s) sources over the out-degree rank, lognormal walk counts."""
    V = len(rp) - 1
    deg = np.diff(rp.astype(np.int64))
    order = np.argsort(-deg, kind="stable")
    rng = np.random.default_rng(SEED_WALK)
    n = cfg["queries"]
    ranks = np.arange(1, V + 1, dtype=np.float64)
    pz = ranks ** -cfg["zipf"]
    pz /= pz.sum()
    r = rng.choice(V, size=n, p=pz)
    sources = order[r].astype(np.uint32)
    w = np.exp(rng.normal(np.log(cfg["walk_median"]), cfg["walk_sigma"], n))
    walkers = np.clip(np.round(w), cfg["walk_min"], cfg["walk_max"]).astype(np.uint64)
    seeds = (np.arange(n, dtype=np.uint64) + np.uint64(1)).astype(np.uint64)
    return sources, walkers, seeds


def gb300_batch(args, cfg):
    import torch
    ws, rank, local, dist = init_dist()
    import lighttraffic_gb300 as lt

    g = lt.Graph.rmat(cfg["scale"], cfg["edges"], seed=SEED_GRAPH, part_bytes=cfg["part_mb"] << 20, device=local)
    V, E = g.num_nodes, g.num_edges
    rp, col = g.csr_views()
    sources, walkers, seeds = c3_queries(cfg, rp)
    n, Wt = len(sources), int(walkers.sum())
    e = lt.Engine(g, seed=SEED_WALK, device=local)
    tune = e.autotune()
    dev = f"cuda:{local}"
    d_src = torch.from_numpy(sources.view(np.int32)).to(dev)
    d_w = torch.from_numpy(walkers.view(np.int64)).to(dev)
    d_seed = torch.from_numpy(seeds.view(np.int64)).to(dev)
    d_off = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    d_v = torch.zeros(Wt, dtype=torch.int32, device=dev)
    d_c = torch.zeros(Wt, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()

    def launch():
        lt.check(lt.lib.lt_ppr_batch_device(e._h, n, d_src.data_ptr(), d_w.data_ptr(), d_seed.data_ptr(),
                                            ctypes.c_float(cfg["prob"]), d_off.data_ptr(), d_v.data_ptr(),
                                            d_c.data_ptr(), Wt, stream.cuda_stream))

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    for _ in range(args.warmup):
        launch()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    wall0 = time.time()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.steps):
        launch()
    b.record()
    torch.cuda.synchronize()
    elapsed_ms = max_over_ranks(dist, local, a.elapsed_time(b))
    # one more batch through the public host API: stats (hops) and e2e time
    e2e = []
    pinned_out = (lt.pinned_empty(n + 1, np.uint64), lt.pinned_empty(Wt, np.uint32), lt.pinned_empty(Wt, np.uint32))
    for _ in range(3):
        t0 = time.perf_counter()
        off, v, c = e.ppr_batch(sources, walkers, seeds, cfg["prob"], out=pinned_out)
        e2e.append(time.perf_counter() - t0)
    e2e = e2e[1:]
    st = e.stats()
    assert int(c.astype(np.uint64).sum()) == Wt, "PPR invariant (one count per walk) violated"
    moves = st["moves"]
    clocks.stop()
    clk = clocks.summary(wall0 - 0.5, time.time())
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    value = moves * args.steps * ws / (elapsed_ms / 1e3)
    pairs = int(off[-1])
    tslots = sum(1 << max(5, int(np.ceil(np.log2(max(2, int(x) << tune["load_shift"]))))) for x in walkers)
    # 20 B per hop, 8 B per endpoint (table slot read + count RMW), 8 B per
    # table slot cleared and 8 B per slot scanned twice, 8 B per output pair
    alg = 20 * moves + 8 * Wt + 24 * tslots + 8 * pairs
    peak, peak_src = measured_peak("hbm_gbs", 6800.0)
    kern_s = st["step_kernel_ms"] / 1e3
    achieved = alg / kern_s / 1e9
    line = {
        "metric": "walk steps/s", "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic RMAT (seeded) and synthetic Zipf / lognormal queries",
        "config": workload_config(args.config, cfg, V, E, g.num_partitions),
        "walkers": Wt, "sparse_pairs": pairs, "autotune": tune, "parallelism": "replicas" if ws > 1 else "1 GPU",
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": profiled_traffic(cfg["workload"]), "kernel": "batch pipeline (walk + tables)",
                     "alg_bytes_per_launch": alg, "mean_launch_ms": st["step_kernel_ms"], "peak_source": peak_src},
        "e2e": {"value": moves * ws / statistics.mean(e2e), "unit": "steps/s",
                "h2d_bytes_per_step": 20 * n, "d2h_bytes_per_step": 8 * (n + 1) + 8 * pairs,
                "ms_per_step": statistics.mean(e2e) * 1e3},
        "gpu_launches": 6 * args.steps,
        "clocks": clk,
    }
    if not args.no_cpu_baseline and ws == 1:
        line["cpu_baseline"], want = cpu_baseline_leg(args.config, cfg, rp, col, args.cpu_seconds)
        for q, (vs, cs) in enumerate(want):
            a, b = int(off[q]), int(off[q + 1])
            order = np.argsort(v[a:b], kind="stable")
            assert np.array_equal(v[a:b][order], vs) and np.array_equal(c[a:b][order], cs), f"query {q} differs"
        line["parity"] = {"oracle_identical": {"queries": len(want), "identical": True}}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def serve_trace(cfg, V, rate, seconds, seed):
    rng = np.random.default_rng(seed)
    n = max(1, int(rate * seconds))
    gaps = rng.exponential(1.0 / rate, n)
    t = np.cumsum(gaps) * 1e3
    src = rng.integers(0, V, n).astype(np.uint32)
    w = np.clip(np.round(np.exp(rng.normal(np.log(cfg["walk_median"]), cfg["walk_sigma"], n))),
                cfg["walk_min"], cfg["walk_max"]).astype(np.uint64)
    seeds = rng.integers(1, 1 << 62, n, dtype=np.uint64)
    return t, src, w, seeds


def gb300_serve(args, cfg):
    ws, rank, local = dist_env()
    if ws > 1:
        ws, rank, local, _ = init_dist()
    import lighttraffic_gb300 as lt

    g = lt.Graph.rmat(cfg["scale"], cfg["edges"], seed=SEED_GRAPH, part_bytes=cfg["part_mb"] << 20, device=local)
    V = g.num_nodes
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    wall0 = time.time()
    out = {}
    for name, sched in [("learned", lt.SCHED_LEARNED), ("plain", lt.SCHED_PLAIN), ("batched", lt.SCHED_BATCHED),
                        ("frequency", lt.SCHED_FREQUENCY)]:
        e = lt.Engine(g, partitions=cfg["partitions"], batch=cfg["batch"], seed=SEED_WALK, sched=sched, device=local)
        per_rate = {}
        for rate, seconds in zip(cfg["rates"], cfg["seconds"]):
            per_rate[str(rate)] = serve_rate(lt, e, cfg, V, rate, seconds, SEED_WALK + rate)
        out[name] = per_rate
        e.close()
    clocks.stop()
    clk = clocks.summary(wall0 - 0.5, time.time())
    if rank != 0:
        return 0
    mid = str(cfg["rates"][1])
    line = {
        "metric": "PPR p99 latency ms", "value": out["learned"][mid]["p99_ms"], "unit": "ms", "n_gpus": ws,
        "steps": 1, "warmup": 0, "ms_per_step": None, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic RMAT graph, synthetic Poisson query trace",
        "config": {"workload": cfg["workload"], "V": V, "rates_qps": list(cfg["rates"]),
                   "walks": "lognormal median %g sigma %g in [%g, %g]" % (cfg["walk_median"], cfg["walk_sigma"],
                                                                          cfg["walk_min"], cfg["walk_max"]),
                   "value_is": f"learned scheduler p99 at {mid} qps"},
        "serving": out, "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--cpu-leg-child":
        return cpu_leg_child(sys.argv[2:])
    args = parse()
    cfg = CONFIGS[args.config]
    if cfg.get("serving") and args.impl != "reference":
        return gb300_serve(args, cfg)
    if args.impl == "reference":
        return reference_arm(args, cfg)
    if "partitions" in cfg:
        return gb300_ooc(args, cfg)
    if cfg.get("batch_queries"):
        return gb300_batch(args, cfg)
    return gb300_resident(args, cfg)


if __name__ == "__main__":
    sys.exit(main())
