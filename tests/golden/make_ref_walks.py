"""Generate tests/golden/ref_walks.json: walk outputs of the reference's own
App::update code.

Run in a checkout that has the reference sources (the reference tree is
$LT_REF_ROOT, else a directory named "reference" beside this repository):

    python tests/golden/make_ref_walks.py

It builds oracle/_ref/ref_apps with ``make -C oracle ref`` -- app/ppr.cu,
app/pagerank.cu and app/genericwalk.cu compiled in place with g++ against the
host stand-ins of oracle/ref_shim/, driven partition by partition with the
keyed Philox stream (see oracle/ref_apps_main.cpp) -- and records, for every
case below, the SHA-256 and the sum of the output arrays (PPR / PageRank
visit counts u64[V]; generic-walk endpoints u32[W] and paths
u32[W (length + 1)]).  tests/test_ref_pin.py holds the oracle to these
vectors and tests/test_gpu_walk.py the CUDA engine.

PageRank runs only on graphs in which every vertex has out-edges: at a vertex
without them the reference computes `% 0` (app/pagerank.cu:42).  The graph
rmat12ring is rmat12 with one out-edge added to each such vertex, written to
graphs/rmat12ring.bcsr.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

GRAPHS = os.path.join(HERE, "graphs")
EXE = os.path.join(ROOT, "oracle", "_ref", "ref_apps")

# (app, graph, parts, start, source, walkers, length, prob, runs, run0, seed)
CASES = []
for _g in ("path4", "hub10", "gaps8", "rmat10", "rmat12"):
    for _seed in (1, 0xDEADBEEF12345):
        for _prob in (0.15, 0.5, 1.0):
            CASES.append(("ppr", _g, 3, 0, 0, 6000, 0, _prob, 1, 0, _seed))
        CASES.append(("ppr", _g, 2, 0, 1, 3001, 0, 0.15, 2, 0, _seed))
        for _start in (1, 2):
            CASES.append(("walk", _g, 3, _start, 0, 5000, 7, 0.0, 1, 2, _seed))
for _g in ("hub10", "rmat12ring"):
    for _seed in (1, 0xDEADBEEF12345):
        for _start in (1, 2):
            CASES.append(("pagerank", _g, 3, _start, 0, 4099, 9, 0.85, 2, 0, _seed))


def ring_graph():
    """rmat12 with one out-edge (to (7 v + 1) mod V, never v itself) added to
    every vertex without out-edges."""
    rp, col = oracle.read_bcsr(os.path.join(GRAPHS, "rmat12.bcsr"))
    V = len(rp) - 1
    deg = np.diff(rp.astype(np.int64))
    rows = [col[int(rp[v]):int(rp[v + 1])] if deg[v] else
            np.array([(7 * v + 1) % V if (7 * v + 1) % V != v else (v + 1) % V], np.uint32) for v in range(V)]
    newdeg = np.array([len(r) for r in rows], np.uint64)
    nrp = np.concatenate([[0], np.cumsum(newdeg)]).astype(np.uint64)
    return nrp, np.concatenate(rows).astype(np.uint32)


def outputs(app, raw, V, W, length):
    if app == "walk":
        return [np.frombuffer(raw, np.uint32, W), np.frombuffer(raw, np.uint32, W * (length + 1), 4 * W)]
    return [np.frombuffer(raw, np.uint64, V)]


def digest(arrays):
    return [{"sha256": hashlib.sha256(a.tobytes()).hexdigest(), "sum": int(a.astype(np.uint64).sum())}
            for a in arrays]


def run_case(case, tmp):
    app, g, parts, start, source, W, length, prob, runs, run0, seed = case
    path = os.path.join(GRAPHS, g + ".bcsr")
    V = int(np.fromfile(path, np.uint32, 1)[0])
    out = os.path.join(tmp, "out.bin")
    subprocess.run([EXE, app, path, str(min(parts, V)), str(start), str(source), str(W), str(length),
                    repr(float(np.float32(prob))), str(runs), str(run0), str(seed), out], check=True)
    return outputs(app, open(out, "rb").read(), V, W, length)


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    rp, col = ring_graph()
    oracle.write_bcsr(os.path.join(GRAPHS, "rmat12ring.bcsr"), rp, col)
    rows = []
    with tempfile.TemporaryDirectory() as tmp:
        for case in CASES:
            keys = ("app", "graph", "parts", "start", "source", "walkers", "length", "prob", "runs", "run0", "seed")
            rows.append({**dict(zip(keys, case)), "outputs": digest(run_case(case, tmp))})
    with open(os.path.join(HERE, "ref_walks.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_ref_walks.py", "harness": "oracle/ref_apps_main.cpp",
                   "cases": rows}, f, indent=1)
    print(f"{len(rows)} cases written")


if __name__ == "__main__":
    main()
