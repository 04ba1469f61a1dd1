#!/usr/bin/env python3
"""Benchmark of the random-walk hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--config c1|c0]

One "step" is one full pass of the app over its workload:
  c1 (default): walk-based PageRank on RMAT(2^23 vertices, 2^27 edges, a/b/c/d =
      .57/.19/.19/.05, seed 1, isolated vertices removed), 32 MiB partitions all
      cached in HBM, W = 2|V| walkers starting one per vertex (walker i at vertex
      i mod V), l = 10, teleport when U > 0.85 -> W * l walk steps per pass.
  c0: PPR on RMAT(2^20, 2^24), source 0, W = 2|V|, stop probability 0.15; steps
      are the hops taken (the reference's 2|V|/0.15 estimate, counted exactly).
Synthetic inputs stand in for the reference's datasets (absent, no network).

value  : device-resident passes through lt_walk_device (graph already in HBM,
         counters zeroed inside each pass), CUDA events on the launching stream.
e2e    : the public API call lt_run_pagerank / lt_run_ppr with host buffers; each
         step drops the device cache first, so the timed region holds the H2D
         copy of every partition (pinned host memory) and the D2H of the counts.
Graph inputs (576 MiB for c1) exceed the 129 MB L2, so no flush is needed
between passes.
--impl reference times the CPU restatement of the reference walk semantics
(oracle/, OpenMP over all host cores) on a bounded sample of the same workload.
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
    "c1": dict(workload="pagerank-rmat23-e27-resident", app=1, scale=23, edges=1 << 27, length=10,
               start=2, prob=0.85, part_mb=32),
    "c0": dict(workload="ppr-rmat20-e24-resident", app=0, scale=20, edges=1 << 24, length=0,
               start=0, prob=0.15, part_mb=32),
}
SEED_GRAPH = 1
SEED_WALK = 1


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--config", default="c1", choices=sorted(CONFIGS))
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="target CPU time of the cpu_baseline sample")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


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

    def summary(self, t0=None, t1=None):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, line in self.lines:
            if t0 is not None and (t < t0 or t > t1):
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
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------- reference arm

def cpu_rate(cfg, rp, col, seconds, threads):
    """Oracle (CPU restatement of the reference semantics) on a bounded sample;
    returns (steps/s, sample description, threads)."""
    import oracle
    V = len(rp) - 1
    W = 2 * V

    def run(n):
        t = time.perf_counter()
        if cfg["app"] == 1:
            _, st = oracle.pagerank(rp, col, n, length=cfg["length"], seed=SEED_WALK,
                                    start_mode=cfg["start"], threads=threads)
            steps = int(st[0])
        else:
            _, _, st = oracle.ppr(rp, col, 0, n, prob=cfg["prob"], seed=SEED_WALK, threads=threads)
            steps = int(st[1])
        return steps, time.perf_counter() - t

    n = min(W, 1 << 17)
    steps, dt = run(n)
    n2 = int(min(W, max(n, n * seconds / max(dt, 1e-3))))
    if n2 > n:
        steps, dt = run(n2)
        n = n2
    return steps / dt, f"first {n} of {W} walkers ({steps} steps, {dt:.1f} s)", threads


def host_graph(cfg):
    """The same RMAT graph on the host, from the oracle's generator (identical bytes)."""
    import oracle
    return oracle.rmat(cfg["scale"], cfg["edges"], seed=SEED_GRAPH)


def reference_arm(args, cfg):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    rp, col = host_graph(cfg)
    threads = os.cpu_count() or 1
    per_step = max(1.0, min(6.0, 150.0 / max(1, args.steps + args.warmup)))
    rates = []
    desc = ""
    for i in range(args.warmup + args.steps):
        r, desc, _ = cpu_rate(cfg, rp, col, per_step, threads)
        if i >= args.warmup:
            rates.append(r)
    value = statistics.median(rates)
    line = {
        "impl": "reference", "metric": "walk steps/s", "value": value, "unit": "steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": "synthetic RMAT (seeded), stand-in for the reference datasets",
        "config": {"workload": cfg["workload"], "V": len(rp) - 1, "E": len(col),
                   "walkers": 2 * (len(rp) - 1), "length": cfg["length"]},
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": threads, "kind": "port",
                         "sample": desc},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------ GB300 arm

def gb300_arm(args, cfg):
    import torch
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import lighttraffic_gb300 as lt

    g = lt.Graph.rmat(cfg["scale"], cfg["edges"], seed=SEED_GRAPH, part_bytes=cfg["part_mb"] << 20,
                      device=local)
    rp, col = g.csr()
    V, E = g.num_nodes, g.num_edges
    W = 2 * V
    d_rp = torch.from_numpy(rp.view(np.int64)).to(f"cuda:{local}")
    d_col = torch.from_numpy(col.view(np.int32)).to(f"cuda:{local}")
    d_cnt = torch.zeros(V, dtype=torch.int64, device=f"cuda:{local}")
    d_scr = torch.zeros(max(1, lt.lib.lt_walk_scratch_bytes() // 8), dtype=torch.int64,
                        device=f"cuda:{local}")
    d_st = torch.zeros(3, dtype=torch.int64, device=f"cuda:{local}")
    stream = torch.cuda.current_stream()
    app, start, length, prob = cfg["app"], cfg["start"], cfg["length"], cfg["prob"]

    def one_pass():
        d_cnt.zero_()
        lt.check(lt.lib.lt_walk_device(app, start, d_rp.data_ptr(), d_col.data_ptr(), V, 0, W, length,
                                       ctypes.c_float(prob), 0, SEED_WALK, d_cnt.data_ptr(), None, None,
                                       d_scr.data_ptr(), d_st.data_ptr(), stream.cuda_stream))

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    for _ in range(args.warmup):
        one_pass()
    torch.cuda.synchronize()
    d_st.zero_()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    t_all0, t_all1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    wall0 = time.time()
    t_all0.record()
    for i in range(args.steps):
        d_cnt.zero_()
        starts[i].record()
        lt.check(lt.lib.lt_walk_device(app, start, d_rp.data_ptr(), d_col.data_ptr(), V, 0, W, length,
                                       ctypes.c_float(prob), 0, SEED_WALK, d_cnt.data_ptr(), None, None,
                                       d_scr.data_ptr(), d_st.data_ptr(), stream.cuda_stream))
        ends[i].record()
    t_all1.record()
    torch.cuda.synchronize()
    wall1 = time.time()
    if dist:
        dist.barrier()
    elapsed_ms = t_all0.elapsed_time(t_all1)
    kern_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    st = d_st.cpu().numpy().astype(np.uint64) // np.uint64(args.steps)
    updates, moves, tele = (int(x) for x in st)
    steps_per_pass = updates if app == 1 else moves
    # correctness of the timed passes: Σ counts is the reference's invariant
    total = int(d_cnt.sum().item())
    assert total == (W * length if app == 1 else W), "invariant violated in the timed pass"
    if dist:
        t = torch.tensor([elapsed_ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    value = steps_per_pass * args.steps * ws / (elapsed_ms / 1e3)

    # roofline of the step kernel: algorithmic bytes per launch / mean launch time
    # 20 B per graph hop (rowptr[c], rowptr[c+1], col[e]) + 16 B per counter update
    # (u64 read + write); PageRank counts every update, PPR once per walk.
    counter_updates = updates if app == 1 else W
    alg_bytes = 20 * moves + 16 * counter_updates
    mean_kern_s = statistics.mean(kern_ms) / 1e3
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
        peak_src = "measured"
    achieved = alg_bytes / mean_kern_s / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get(cfg["workload"])

    # e2e through the public API with host buffers
    eng = lt.Engine(g, seed=SEED_WALK, device=local)
    host_counts = torch.empty(V, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    e2e_times = []
    h2d = 0
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
    e2e_value = steps_per_pass * ws / e2e_s
    clocks.stop()
    clk = clocks.summary(wall0 - 0.5, time.time())

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    line = {
        "metric": "walk steps/s", "value": value, "unit": "steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic RMAT (seeded), stand-in for the reference datasets",
        "config": {"workload": cfg["workload"], "V": V, "E": E, "partitions": g.num_partitions,
                   "walkers": W, "length": length, "steps_per_pass": steps_per_pass,
                   "l2": "inputs larger than L2 (graph %d MiB > 129 MB L2), no flush" % ((8 * (V + 1) + 4 * E) >> 20),
                   "parallelism": "replicas" if ws > 1 else "1 GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "walk_whole_kernel", "alg_bytes_per_launch": alg_bytes,
                     "mean_launch_ms": mean_kern_s * 1e3, "peak_source": peak_src},
        "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 8 * V, "ms_per_step": e2e_s * 1e3},
        "gpu_launches": args.steps,
        "clocks": clk,
        "stats_per_pass": {"updates": updates, "moves": moves, "teleports": tele},
    }
    if not args.no_cpu_baseline and ws == 1:
        r, desc, threads = cpu_rate(cfg, rp, col, args.cpu_seconds, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": r, "unit": "steps/s", "cores": threads, "kind": "port",
                                "sample": desc}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    cfg = CONFIGS[args.config]
    if args.impl == "reference":
        return reference_arm(args, cfg)
    return gb300_arm(args, cfg)


if __name__ == "__main__":
    sys.exit(main())
