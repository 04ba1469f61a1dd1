"""Batched multi-source PPR: every query's sparse counts equal the oracle's
PPR with that query's seed, alone or in any batch, before and after tuning."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graph16():
    return oracle.rmat(16, 1 << 20, seed=21)


def _as_dict(off, v, c, q):
    a, b = int(off[q]), int(off[q + 1])
    return dict(zip(v[a:b].tolist(), c[a:b].tolist()))


def _oracle_dict(rp, col, src, w, seed):
    counts, _, _ = oracle.ppr(rp, col, src, w, prob=0.15, seed=seed)
    nz = np.nonzero(counts)[0]
    return dict(zip(nz.tolist(), counts[nz].astype(np.uint32).tolist()))


def test_batch_matches_oracle(lt, require_gpu, graph16):
    rp, col = graph16
    V = len(rp) - 1
    g = lt.Graph.from_csr(rp, col, 1 << 30)
    e = lt.Engine(g, seed=5)
    rng = np.random.default_rng(3)
    n = 60
    src = rng.integers(0, V, n).astype(np.uint32)
    src[:5] = 0                                   # repeated sources are distinct queries
    w = rng.integers(1, 20000, n).astype(np.uint64)
    w[7] = 1
    seeds = rng.integers(1, 1 << 62, n, dtype=np.uint64)
    off, v, c = e.ppr_batch(src, w, seeds)
    assert off[0] == 0 and len(off) == n + 1
    for q in range(n):
        got = _as_dict(off, v, c, q)
        assert sum(got.values()) == int(w[q])
        assert got == _oracle_dict(rp, col, int(src[q]), int(w[q]), int(seeds[q])), q


def test_alone_equals_in_mix_and_single_run(lt, require_gpu, graph16):
    rp, col = graph16
    V = len(rp) - 1
    g = lt.Graph.from_csr(rp, col, 1 << 30)
    e = lt.Engine(g, seed=77)
    src = np.array([3, 11, 3, 900, 4000], np.uint32)
    w = np.array([5000, 300, 7000, 1, 20000], np.uint64)
    seeds = np.array([77, 8, 9, 10, 11], np.uint64)
    off, v, c = e.ppr_batch(src, w, seeds)
    for q in range(len(src)):
        o1, v1, c1 = e.ppr_batch(src[q:q + 1], w[q:q + 1], seeds[q:q + 1])
        assert _as_dict(o1, v1, c1, 0) == _as_dict(off, v, c, q)
    # query 0 uses the engine seed: equals the single-source run
    dense = e.ppr(3, 5000, 0.15)
    nz = np.nonzero(dense)[0]
    assert _as_dict(off, v, c, 0) == dict(zip(nz.tolist(), dense[nz].astype(np.uint32).tolist()))


def test_autotune_and_replay(lt, require_gpu, graph16):
    rp, col = graph16
    V = len(rp) - 1
    g = lt.Graph.from_csr(rp, col, 1 << 30)
    e = lt.Engine(g, seed=1)
    src = (np.arange(200, dtype=np.uint64) * 97 % V).astype(np.uint32)
    w = (np.arange(200, dtype=np.uint64) % 13 + 1) * 500
    seeds = np.arange(200, dtype=np.uint64) + 1000
    before = e.ppr_batch(src, w, seeds)
    t = e.autotune()
    assert t["tuned"] and t["block"] in (128, 256, 512) and t["load_shift"] in (1, 2)
    after = e.ppr_batch(src, w, seeds)
    for q in range(0, 200, 17):
        assert _as_dict(*before, q) == _as_dict(*after, q)
    # replays with other batch sizes reuse the captured graph
    for n in (1, 37, 200):
        o, v, c = e.ppr_batch(src[:n], w[:n], seeds[:n])
        for q in range(0, n, 11):
            assert _as_dict(o, v, c, q) == _as_dict(*before, q)


def test_batch_needs_resident_graph(lt, require_gpu, graph16):
    rp, col = graph16
    g = lt.Graph.from_csr(rp, col, 256 << 10)
    e = lt.Engine(g, partitions=2)
    with pytest.raises(lt.LTError):
        e.ppr_batch([0], [10])


def test_batch_into_pinned_outputs(lt, require_gpu):
    """ppr_batch(out=...) with page-locked arrays from pinned_empty gives the
    same pairs as fresh arrays, twice in a row (buffers reused)."""
    g = lt.Graph.rmat(14, 1 << 18, seed=3, part_bytes=1 << 30)
    e = lt.Engine(g, seed=5)
    src = np.array([0, 3, 3, 17], np.uint32)
    w = np.array([5000, 1200, 800, 3000], np.uint64)
    seeds = np.array([1, 2, 3, 4], np.uint64)
    ref = e.ppr_batch(src, w, seeds)
    out = (lt.pinned_empty(len(src) + 1, np.uint64), lt.pinned_empty(int(w.sum()), np.uint32),
           lt.pinned_empty(int(w.sum()), np.uint32))
    for _ in range(2):
        off, v, c = e.ppr_batch(src, w, seeds, out=out)
        assert (off == ref[0]).all()
        for q in range(len(src)):
            a, b = int(off[q]), int(off[q + 1])
            got = sorted(zip(v[a:b].tolist(), c[a:b].tolist()))
            want = sorted(zip(ref[1][a:b].tolist(), ref[2][a:b].tolist()))
            assert got == want


def test_c3s_zipf_batch_matches_oracle(lt, require_gpu):
    """The c3 batch workload scaled down (RMAT 2^22 / 2^26, 256 sources drawn
    Zipf(1.1) by out-degree rank, lognormal walks clipped to [1e3, 1e6]):
    every query's sparse counts equal the oracle's PPR with its seed."""
    import bench
    g = lt.Graph.rmat(22, 1 << 26, seed=1, part_bytes=32 << 20)
    rp, col = g.csr_views()
    sources, walkers, seeds = bench.c3_queries(bench.CONFIGS["c3s"], rp)
    e = lt.Engine(g, seed=1)
    off, v, c = e.ppr_batch(sources, walkers, seeds, 0.15)
    for q in range(len(sources)):
        got = _as_dict(off, v, c, q)
        assert got == _oracle_dict(rp, col, int(sources[q]), int(walkers[q]), int(seeds[q])), q
    e.autotune()
    off2, v2, c2 = e.ppr_batch(sources, walkers, seeds, 0.15)
    for q in (0, 1, len(sources) // 2, len(sources) - 1):
        assert _as_dict(off2, v2, c2, q) == _as_dict(off, v, c, q)
