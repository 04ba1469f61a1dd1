"""The oracle against the reference's own App::update code.

tests/golden/ref_walks.json holds outputs of oracle/ref_apps_main.cpp: the
reference's app/ppr.cu, app/pagerank.cu and app/genericwalk.cu compiled in
place with g++ and driven partition by partition the way its step kernel
drives them (src/WalkManager.h:229-246), with the keyed Philox stream in
place of cuRAND (tests/golden/make_ref_walks.py made the file).  The oracle
must reproduce every vector bit for bit: this pins its restatement of the
three apps' update rules to the reference's code.  Where the harness is built
(a checkout with the reference sources), further seeded cases run it live.
"""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, ROOT

with open(os.path.join(GOLDEN, "ref_walks.json")) as _f:
    REF = json.load(_f)["cases"]
EXE = os.path.join(ROOT, "oracle", "_ref", "ref_apps")


def _graph(name):
    return oracle.read_bcsr(os.path.join(GOLDEN, "graphs", f"{name}.bcsr"))


def oracle_outputs(case):
    rp, col = _graph(case["graph"])
    app, W, L, prob, seed = case["app"], case["walkers"], case["length"], case["prob"], case["seed"]
    if app == "walk":
        ep, pa, _ = oracle.generic_walk(rp, col, W, length=L, start_mode=case["start"], run=case["run0"],
                                        seed=seed, paths=True)
        return [ep, pa]
    counts = np.zeros(len(rp) - 1, np.uint64)
    for r in range(case["run0"], case["run0"] + case["runs"]):
        oracle.walk_batch(oracle.APP_PPR if app == "ppr" else oracle.APP_PAGERANK, rp, col,
                          start_mode=case["start"], source=case["source"], walkers=W, length=L, prob=prob,
                          run=r, seed=seed, counts=counts)
    return [counts]


def _digest(arrays):
    return [{"sha256": hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest(),
             "sum": int(a.astype(np.uint64).sum())} for a in arrays]


def _id(c):
    return f"{c['app']}-{c['graph']}-s{c['start']}-p{c['prob']}-r{c['runs']}-{c['seed']:x}"


@pytest.mark.parametrize("case", REF, ids=[_id(c) for c in REF])
def test_oracle_matches_reference_update(case):
    assert _digest(oracle_outputs(case)) == case["outputs"]


def test_vectors_cover_every_app_and_start():
    seen = {(c["app"], c["start"]) for c in REF}
    assert {("ppr", 0), ("walk", 1), ("walk", 2), ("pagerank", 1), ("pagerank", 2)} <= seen
    assert any(c["prob"] == 1.0 for c in REF) and any(c["runs"] > 1 for c in REF)


def _live(app, graph, parts, start, source, W, L, prob, runs, run0, seed, tmp_path):
    path = os.path.join(GOLDEN, "graphs", f"{graph}.bcsr")
    out = str(tmp_path / "o.bin")
    subprocess.run([EXE, app, path, str(parts), str(start), str(source), str(W), str(L),
                    repr(float(np.float32(prob))), str(runs), str(run0), str(seed), out], check=True)
    raw = open(out, "rb").read()
    V = len(_graph(graph)[0]) - 1
    if app == "walk":
        return [np.frombuffer(raw, np.uint32, W), np.frombuffer(raw, np.uint32, W * (L + 1), 4 * W)]
    return [np.frombuffer(raw, np.uint64, V)]


@pytest.mark.skipif(not os.path.exists(EXE), reason="reference harness not built (no reference sources)")
@pytest.mark.parametrize("seed", [3, 77, 2**40 + 5])
def test_live_reference_harness(seed, tmp_path):
    """More seeds, probabilities, sources and partition counts than the
    vectors hold, straight against the harness."""
    rng = np.random.default_rng(seed)
    for graph in ("rmat10", "rmat12", "gaps8"):
        V = len(_graph(graph)[0]) - 1
        prob = float(rng.choice([0.05, 0.15, 0.3, 0.9]))
        src = int(rng.integers(0, V))
        parts = int(rng.integers(1, min(V, 9) + 1))
        case = dict(app="ppr", graph=graph, start=0, source=src, walkers=4000, length=0, prob=prob, runs=1,
                    run0=int(rng.integers(0, 3)), seed=seed)
        got = _live("ppr", graph, parts, 0, src, 4000, 0, prob, 1, case["run0"], seed, tmp_path)
        assert all((a == b).all() for a, b in zip(got, oracle_outputs(case))), case
        L = int(rng.integers(1, 12))
        case = dict(app="walk", graph=graph, start=int(rng.integers(1, 3)), source=0, walkers=3000, length=L,
                    prob=0.0, runs=1, run0=int(rng.integers(0, 3)), seed=seed)
        got = _live("walk", graph, parts, case["start"], 0, 3000, L, 0.0, 1, case["run0"], seed, tmp_path)
        assert all((a == b).all() for a, b in zip(got, oracle_outputs(case))), case
    case = dict(app="pagerank", graph="rmat12ring", start=1, source=0, walkers=5000, length=6, prob=0.85, runs=3,
                run0=0, seed=seed)
    got = _live("pagerank", "rmat12ring", 5, 1, 0, 5000, 6, 0.85, 3, 0, seed, tmp_path)
    assert all((a == b).all() for a, b in zip(got, oracle_outputs(case)))
