"""The CPU oracle against known answers, the reference's invariants and its
own golden regression vectors (tests/golden/walks.json)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

# Known-answer vectors of Philox4x32-10 published with Random123 (Salmon et
# al., SC'11, kat_vectors): counter, key -> output.
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,want", PHILOX_KAT)
def test_philox_kat(ctr, key, want):
    assert oracle.philox(ctr, key).tolist() == want


def test_threshold53_exact():
    assert oracle.threshold53(1.0) == 1 << 53
    assert oracle.threshold53(0.5) == 1 << 52
    # 0.15f widened to double, times 2^53, floored
    want = int(np.float64(np.float32(0.15)) * 2.0 ** 53)
    assert oracle.threshold53(0.15) == want


def _hash(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _golden_graph(name):
    return oracle.read_bcsr(os.path.join(GOLDEN, "graphs", f"{name}.bcsr"))


def test_ppr_path_graph_is_deterministic():
    # 0->1->2->3, 3 has no out-edges: a walk of length L from 0 ends at
    # min(L-1, 3) (app/ppr.cu:22-42: L-1 hops, or the dangling vertex reached)
    rp, col = _golden_graph("path4")
    c, ep, st = oracle.ppr(rp, col, 0, 4000, prob=0.3, seed=5, endpoints=True)
    L = np.array([oracle.ppr_length(5, 0, i, 0.3) for i in range(4000)])
    assert (ep == np.minimum(L - 1, 3)).all()
    assert c.sum() == 4000
    assert np.bincount(ep, minlength=4).tolist() == c.tolist()


def test_ppr_length_distribution():
    # P(L = 2 + k) = p (1-p)^k  (src/walk/SingleSource.h:11-18)
    L = np.array([oracle.ppr_length(9, 0, i, 0.25) for i in range(20000)])
    assert L.min() == 2
    assert abs(L.mean() - (2 + 0.75 / 0.25)) < 0.08


@pytest.mark.parametrize("name", ["hub10", "gaps8", "rmat10", "rmat12"])
def test_reference_sum_invariants(name):
    rp, col = _golden_graph(name)
    V = len(rp) - 1
    c, _, _ = oracle.ppr(rp, col, 0, 3000, seed=2)
    assert c.sum() == 3000                       # app/ppr.cu:77-85
    c, _ = oracle.pagerank(rp, col, 2 * V, length=7, runs=3, seed=2)
    assert c.sum() == 2 * V * 7 * 3               # app/pagerank.cu:202-210


def test_generic_walk_paths_consistent():
    rp, col = _golden_graph("gaps8")
    ep, pa, _ = oracle.generic_walk(rp, col, 200, length=5, seed=4, paths=True)
    pa = pa.reshape(200, 6)
    for w in range(200):
        row = pa[w]
        valid = row[row != oracle.INVALID_NODE]
        assert (row[: len(valid)] == valid).all()        # padding only at the end
        assert valid[-1] == ep[w]
        for a, b in zip(valid[:-1], valid[1:]):            # every hop is an edge
            assert b in col[rp[a]:rp[a + 1]]
        if len(valid) < 6:                                 # stopped early => dangling
            assert rp[valid[-1] + 1] == rp[valid[-1]]


def test_walks_schedule_independent_of_threads():
    rp, col = _golden_graph("rmat12")
    a, _ = oracle.pagerank(rp, col, 5000, length=10, seed=3, threads=1)
    b, _ = oracle.pagerank(rp, col, 5000, length=10, seed=3, threads=4)
    assert (a == b).all()


def test_walk_golden_vectors():
    with open(os.path.join(GOLDEN, "walks.json")) as f:
        gold = json.load(f)
    for name in ["hub10", "gaps8", "rmat10", "rmat12"]:
        rp, col = _golden_graph(name)
        V = len(rp) - 1
        c, ep, st = oracle.ppr(rp, col, 0, 5000, prob=0.15, seed=11, endpoints=True)
        g = gold[f"{name}:ppr"]
        assert (_hash(c), _hash(ep), int(c.sum()), int(st[1])) == (g["counts"], g["endpoints"], g["sum"], g["moves"])
        c, st = oracle.pagerank(rp, col, 2 * V, length=10, runs=2, seed=12, start_mode=oracle.START_PER_VERTEX)
        g = gold[f"{name}:pagerank"]
        assert (_hash(c), int(c.sum()), int(st[2])) == (g["counts"], g["sum"], g["teleports"])
        ep, pa, st = oracle.generic_walk(rp, col, 3 * V, length=6, seed=13, paths=True)
        g = gold[f"{name}:walk"]
        assert (_hash(ep), _hash(pa), int(st[1])) == (g["endpoints"], g["paths"], g["moves"])


def test_rmat_properties():
    rp, col = oracle.rmat(12, 1 << 15, seed=3)
    V = len(rp) - 1
    assert rp[0] == 0 and rp[-1] == 1 << 15 and (np.diff(rp.astype(np.int64)) >= 0).all()
    assert col.max() < V
    deg = np.diff(rp.astype(np.int64))
    present = deg > 0
    present[col] = True
    assert present.all()                                   # isolated vertices removed
    # RMAT skew: vertex 0 (all-zero bits) has the largest expected out-degree
    assert deg[0] == deg.max()
    rp2, col2 = oracle.rmat(12, 1 << 15, seed=3, threads=1)
    assert (rp == rp2).all() and (col == col2).all()
