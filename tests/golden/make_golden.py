"""Generate the golden fixtures under tests/golden/.

Run in a checkout that has the reference sources (it builds
``oracle/_ref/ref_partition`` from them with ``make -C oracle ref``):

    python tests/golden/make_golden.py

Fixtures
  graphs/<name>.bcsr                 small graphs (hand-made and RMAT)
  graphs/<name>.<bytes>.part         .part written by the reference's own
                                     EqualSizeStrategy + materialize
  partitions.json                    per (graph, max_bytes): the reference's
                                     node/edge offsets, or its error message
  walks.json                         oracle outputs (sha256 of the count /
                                     endpoint / path arrays) for small seeded
                                     walks: regression vectors of the oracle
                                     itself, not reference outputs (the
                                     reference's walks are not reproducible:
                                     cuRAND seeded from an uninitialised value)
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

GRAPHS = os.path.join(HERE, "graphs")


def hand_graphs():
    g = {}
    # path 0->1->2->3 with a dangling end
    g["path4"] = (np.array([0, 1, 2, 3, 3], np.uint64), np.array([1, 2, 3], np.uint32))
    # a hub with 40 out-edges, then a ring of 9 vertices
    rp = [0, 40] + [40 + i + 1 for i in range(9)]
    col = [1 + (i % 9) for i in range(40)] + [2 + i if i < 8 else 1 for i in range(9)]
    g["hub10"] = (np.array(rp, np.uint64), np.array(col, np.uint32))
    # vertices with zero out-degree in the middle and at the end
    g["gaps8"] = (np.array([0, 3, 3, 5, 5, 5, 9, 10, 10], np.uint64),
                  np.array([1, 2, 7, 0, 6, 0, 1, 2, 3, 5], np.uint32))
    return g


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    if os.path.isdir(GRAPHS):
        shutil.rmtree(GRAPHS)
    os.makedirs(GRAPHS)
    graphs = hand_graphs()
    graphs["rmat10"] = oracle.rmat(10, 1 << 13, seed=7)
    graphs["rmat12"] = oracle.rmat(12, 1 << 15, seed=3)
    sizes = {
        "path4": [24, 28, 32, 40, 1 << 20],
        "hub10": [100, 175, 176, 200, 256, 1 << 20],
        "gaps8": [20, 28, 36, 48, 1 << 20],
        "rmat10": [2048, 4096, 9000, 1 << 20],
        "rmat12": [4096, 16384, 65536, 1 << 20],
    }
    parts = {}
    for name, (rp, col) in graphs.items():
        path = os.path.join(GRAPHS, f"{name}.bcsr")
        oracle.write_bcsr(path, rp, col)
        for sz in sizes[name]:
            key = f"{name}:{sz}"
            try:
                no, eo = oracle.ref_partition(path, sz)
                shutil.move(path + ".part", os.path.join(GRAPHS, f"{name}.{sz}.part"))
                parts[key] = {"node_off": no.tolist(), "edge_off": eo.tolist()}
            except ValueError as e:
                parts[key] = {"error": str(e)}
    with open(os.path.join(HERE, "partitions.json"), "w") as f:
        json.dump(parts, f, indent=1, sort_keys=True)

    def h(a):
        return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()

    walks = {}
    for name in ["hub10", "gaps8", "rmat10", "rmat12"]:
        rp, col = graphs[name]
        V = len(rp) - 1
        c, ep, st = oracle.ppr(rp, col, 0, 5000, prob=0.15, seed=11, endpoints=True)
        walks[f"{name}:ppr"] = {"counts": h(c), "endpoints": h(ep), "sum": int(c.sum()),
                                "moves": int(st[1])}
        c, st = oracle.pagerank(rp, col, 2 * V, length=10, runs=2, seed=12,
                                start_mode=oracle.START_PER_VERTEX)
        walks[f"{name}:pagerank"] = {"counts": h(c), "sum": int(c.sum()), "teleports": int(st[2])}
        ep, pa, st = oracle.generic_walk(rp, col, 3 * V, length=6, seed=13, paths=True,
                                         start_mode=oracle.START_UNIFORM)
        walks[f"{name}:walk"] = {"endpoints": h(ep), "paths": h(pa), "moves": int(st[1])}
    with open(os.path.join(HERE, "walks.json"), "w") as f:
        json.dump(walks, f, indent=1, sort_keys=True)
    print(f"wrote {len(parts)} partition cases and {len(walks)} walk cases")


if __name__ == "__main__":
    main()
