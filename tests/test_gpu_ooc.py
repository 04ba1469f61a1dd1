"""GPU parity of the out-of-core path (device cache smaller than the graph).

The partition cache size (-p), walker budget (-b, forcing host spills),
zero-copy threshold and scheduling policy change the schedule, never the
result: counts, endpoints and paths must equal the oracle's bit for bit.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g16():
    rp, col = oracle.rmat(16, 1 << 20, seed=21)
    return rp, col


def _index_share(rp, part_bytes):
    """Partitions' worth of the -p budget the device-resident vertex index
    takes (at most 8 (V+1) bytes; 4 (V+1) in the compact layout)."""
    return -(-8 * len(rp) // part_bytes)


def _eng(lt, rp, col, part_bytes, **kw):
    """-p is a byte budget: with the vertex index on the device (the
    default) its share is added, so that at least the asked-for number of
    slots remains."""
    g = lt.Graph.from_csr(rp, col, part_bytes)
    if kw.get("resident_index", True) and kw.get("partitions"):
        kw["partitions"] += _index_share(rp, part_bytes)
    return g, lt.Engine(g, **kw)


CASES = [
    # (partitions cached, walker budget, zero-copy threshold, scheduler)
    (4, 0, 0, 0),            # plain, no zero-copy
    (1, 0, 0, 0),            # a single slot
    (4, 0, 1 << 40, 0),      # every cold partition read zero-copy
    (4, 0, None, 0),         # default threshold partitionSize/128/2
    (3, 20000, 0, 0),        # tiny walker pool: host spills
    (5, 0, 0, 1),            # FIFO policy
    (4, 0, None, 2),         # learned (wave runs): cache by predicted visits
    (2, 20000, None, 3),     # frequency ablation, host spills
    (4, 0, None, 4),         # batched: wave runs, least recently used slots
    (1, 0, 0, 4),            # wave runs through a single slot, no zero-copy
    (3, 20000, 0, 2),        # learned, tiny walker pool, no zero-copy
    (4, 0, 1 << 40, 4),      # wave runs with every cold partition read zero-copy
]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("index", [True, False])
def test_ppr_ooc(lt, require_gpu, g16, case, index):
    """index: vertex index resident on the device (default) or rowptr slices
    in the slots and read zero-copy from the host (the reference's layout)."""
    K, B, zc, sched = case
    rp, col = g16
    extra = _index_share(rp, 256 << 10) if index else 0
    g, e = _eng(lt, rp, col, 256 << 10, partitions=K, batch=B, zerocopy_threshold=zc, sched=sched, seed=9,
                resident_index=index)
    assert g.num_partitions > K
    W = 300000
    got = e.ppr(0, W, 0.15)
    want, _, st = oracle.ppr(rp, col, 0, W, prob=0.15, seed=9)
    assert (got == want).all()
    s = e.stats()
    assert s["moves"] == st[1]
    assert s["iterations"] >= 1
    if zc == 0:
        assert s["h2d_graph_bytes"] > 0 and s["zerocopy_calls"] == 0
    if zc == 1 << 40:
        assert s["zerocopy_calls"] > 0
    if index:
        # the vertex index is paid from the (K + extra) x partition-size budget
        assert s["index_on_device"] == 1 and K <= s["cache_slots"] <= K + extra
    else:
        assert s["cache_slots"] == K and s["index_on_device"] == 0
    if B and sched < 2 and not index:
        assert s["d2h_walker_bytes"] > 0 and s["h2d_walker_bytes"] > 0


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("start", [1, 2])
def test_pagerank_ooc(lt, require_gpu, g16, case, start):
    K, B, zc, sched = case
    rp, col = g16
    V = len(rp) - 1
    g, e = _eng(lt, rp, col, 256 << 10, partitions=K, batch=B, zerocopy_threshold=zc, sched=sched, seed=4)
    got = e.pagerank(2 * V, length=8, runs=2, start=start)
    want, st = oracle.pagerank(rp, col, 2 * V, length=8, runs=2, seed=4, start_mode=start)
    assert (got == want).all()
    s = e.stats()
    assert (s["updates"], s["moves"], s["teleports"]) == tuple(int(x) for x in st)


@pytest.mark.parametrize("case", CASES[:3] + CASES[4:5] + [(4, 0, None, 4), (3, 20000, 0, 2), (4, 0, 1 << 40, 4)])
@pytest.mark.parametrize("index", [True, False])
def test_walk_ooc(lt, require_gpu, g16, case, index):
    K, B, zc, sched = case
    rp, col = g16
    V = len(rp) - 1
    g, e = _eng(lt, rp, col, 256 << 10, partitions=K, batch=B, zerocopy_threshold=zc, sched=sched, seed=6,
                resident_index=index)
    for start in (1, 2):
        ep, pa, _ = oracle.generic_walk(rp, col, V + 77, length=6, start_mode=start, run=1, seed=6, paths=True)
        gep, gpa = e.walk(V + 77, length=6, run=1, start=start, paths=True)
        assert (gep == ep).all() and (gpa == pa).all()


@pytest.mark.parametrize("sched", [0, 4])
def test_resident_index_loads_only_edges(lt, require_gpu, g16, sched):
    """With the vertex index on the device a load copies only the col slice:
    same counts as the reference layout, fewer graph bytes per load, each
    load at most the largest partition's col bytes."""
    rp, col = g16
    res = {}
    for index in (True, False):
        g, e = _eng(lt, rp, col, 256 << 10, partitions=3, zerocopy_threshold=0, sched=sched, seed=5,
                    resident_index=index)
        res[index] = (e.ppr(0, 200000, 0.15), e.stats(), g)
    (c1, s1, g1), (c0, s0, _) = res[True], res[False]
    assert (c1 == c0).all()
    assert s1["partition_loads"] > 0 and s0["partition_loads"] > 0
    assert s1["h2d_graph_bytes"] / s1["partition_loads"] < s0["h2d_graph_bytes"] / s0["partition_loads"]
    eo = g1.partitions()[1].astype(np.int64)
    assert s1["h2d_graph_bytes"] <= s1["partition_loads"] * 4 * int(np.diff(eo).max())


def test_resident_and_ooc_agree(lt, require_gpu, g16):
    rp, col = g16
    V = len(rp) - 1
    g = lt.Graph.from_csr(rp, col, 128 << 10)
    full = lt.Engine(g, seed=3)
    part = lt.Engine(g, partitions=2, seed=3)
    assert (full.ppr(7, 200000, 0.2) == part.ppr(7, 200000, 0.2)).all()
    assert (full.pagerank(3 * V, 10, start=2) == part.pagerank(3 * V, 10, start=2)).all()


@pytest.mark.parametrize("sched", [0, 2, 4])
def test_repeated_runs_and_drop_cache(lt, require_gpu, g16, sched):
    rp, col = g16
    g, e = _eng(lt, rp, col, 256 << 10, partitions=3, seed=12, sched=sched)
    a = e.ppr(0, 100000, 0.15)
    b = e.ppr(0, 100000, 0.15)                 # warm cache
    e.drop_cache()
    c = e.ppr(0, 100000, 0.15)                 # cold again
    assert (a == b).all() and (a == c).all()


def test_c0_ooc_full_size(lt, require_gpu):
    """c0 graph with one 32 MiB slot for its 3+ partitions."""
    g = lt.Graph.rmat(20, 1 << 24, seed=1, part_bytes=32 << 20)
    rp, col = g.csr()
    V = g.num_nodes
    e = lt.Engine(g, partitions=1, seed=1)
    got = e.ppr(0, 2 * V, 0.15)
    want, _, _ = oracle.ppr(rp, col, 0, 2 * V, prob=0.15, seed=1)
    assert (got == want).all()
    s = e.stats()
    assert s["partition_loads"] >= 2


def test_wave_runs_take_fewer_iterations(lt, require_gpu, g16):
    """A wave drains every cached queue per kernel: far fewer iterations than
    the one-partition-per-iteration reference loop, same counts."""
    rp, col = g16
    res = {}
    for sched in (0, 4):
        g, e = _eng(lt, rp, col, 256 << 10, partitions=4, sched=sched, seed=9)
        res[sched] = (e.ppr(0, 300000, 0.15), e.stats())
    assert (res[0][0] == res[4][0]).all()
    assert res[4][1]["iterations"] < res[0][1]["iterations"]


def test_wave_runs_without_pipelining(lt, require_gpu, g16):
    """--no-pipeline: loads finish before the kernel of their iteration;
    results identical, same loads."""
    rp, col = g16
    out = {}
    for pipe in (True, False):
        g, e = _eng(lt, rp, col, 256 << 10, partitions=4, sched=4, seed=9, pipeline=pipe, zerocopy_threshold=0)
        out[pipe] = (e.ppr(0, 300000, 0.15), e.stats())
    assert (out[True][0] == out[False][0]).all()
    want, _, _ = oracle.ppr(rp, col, 0, 300000, prob=0.15, seed=9)
    assert (out[False][0] == want).all()


@pytest.fixture(scope="module")
def c2s(lt):
    """The c2 out-of-core workload scaled down: RMAT 2^24 / 2^28 (1.1 GiB in
    pinned host memory, 32 MiB partitions), W = 2|V| PPR walks from vertex 0,
    against the oracle on the same arrays."""
    g = lt.Graph.rmat(24, 1 << 28, seed=1, part_bytes=32 << 20)
    rp, col = g.csr_views()
    W = 2 * g.num_nodes
    want, _, st = oracle.ppr(rp, col, 0, W, prob=0.15, seed=1)
    return g, W, want, st


@pytest.mark.parametrize("sched,pipeline,host_plan,split", [(2, True, False, True), (2, True, True, True),
                                                            (2, True, False, False), (4, True, False, True),
                                                            (3, True, False, True), (0, True, False, True),
                                                            (0, False, False, True), (1, True, False, True)])
def test_c2s_scale_ooc(lt, require_gpu, c2s, sched, pipeline, host_plan, split):
    """16 of the graph's partitions cached, walker pool 2^22: every scheduler,
    with and without the load/compute overlap, gives the oracle's counts bit
    for bit, and wave runs read bounded zero-copy groups (the path that takes
    most of a c2 run).  The plain loop finds no cached partition to compute
    while a load is in flight: its step kernel walks every walker through all
    cached partitions, so none keeps a queue (the reference stops walkers at
    each partition border, src/WalkManager.h:239, and computes the queues
    that builds up during loads).  Bucketing passes are planned by a device
    kernel behind the step kernel, or (host_plan) by the host; wave runs
    step the cached walkers and the zero-copy group in two concurrent
    kernels (split) or in one."""
    g, W, want, st = c2s
    assert g.num_partitions > 16
    e = lt.Engine(g, partitions=16, batch=1 << 22, seed=1, sched=sched, pipeline=pipeline, host_plan=host_plan,
                  split=split)
    got = e.ppr(0, W, 0.15)
    assert (got == want).all()
    s = e.stats()
    assert s["moves"] == st[1]
    if sched in (2, 3, 4):
        assert s["zerocopy_groups"] > 0
    if not pipeline:
        assert s["overlap_computes"] == 0
    if host_plan:
        assert s["device_plans"] == 0
    else:
        assert s["device_plans"] > 0
    if sched in (2, 3, 4):
        assert (s["split_launches"] > 0) == split
    else:
        assert s["split_launches"] == 0
    e.close()


@pytest.mark.parametrize("sched", [0, 2, 4])
@pytest.mark.parametrize("host_plan", [False, True])
@pytest.mark.parametrize("B", [0, 20000])
def test_bucket_plan_device_or_host(lt, require_gpu, g16, sched, host_plan, B):
    """A bucketing pass is planned by a device kernel right behind the step
    kernel (default, whenever the free chunks provably hold every arrival) or
    by the host after reading the histogram (which may spill walkers first):
    the queues, and so the counts, are the same.  With a tiny walker pool (B)
    the two kinds of pass alternate within one run."""
    rp, col = g16
    W = 300000
    want, _, _ = oracle.ppr(rp, col, 0, W, prob=0.15, seed=9)
    g, e = _eng(lt, rp, col, 256 << 10, partitions=4, batch=B, sched=sched, seed=9, host_plan=host_plan)
    assert (e.ppr(0, W, 0.15) == want).all()
    s = e.stats()
    if host_plan:
        assert s["device_plans"] == 0
    elif B == 0:
        assert s["device_plans"] > 0


@pytest.mark.parametrize("sched", [0, 2])
def test_ooc_autotune_keeps_results(lt, require_gpu, g16, sched):
    """The out-of-core autotuner changes only the schedule: after tuning, and
    with either bucketing tile and a capped step-kernel grid, the counts are
    the oracle's."""
    rp, col = g16
    want, _, _ = oracle.ppr(rp, col, 0, 200000, prob=0.15, seed=3)
    g, e = _eng(lt, rp, col, 256 << 10, partitions=4, sched=sched, seed=3)
    t = e.autotune()
    assert t["tuned"] == 1 and t["trial_walkers"] > 0 and t["bucket_items"] in (0, 8, 16)
    assert t["tuned_ms"] <= t["default_ms"]
    assert (e.ppr(0, 200000, 0.15) == want).all()
    for items, ctas in ((8, 1), (16, 2)):
        g, e = _eng(lt, rp, col, 256 << 10, partitions=4, sched=sched, seed=3, bucket_items=items, ctas_per_sm=ctas,
                    load_factor=2, zc_group_bytes=1 << 20)
        assert (e.ppr(0, 200000, 0.15) == want).all()


@pytest.mark.parametrize("sched", [2, 3, 4])
def test_hot_tier_keeps_results(lt, require_gpu, g16, sched):
    """The hot-vertex tier (built after the first run of a walk from its
    counts, copied in and marked in the vertex index at every later run's
    start, unmarked when the cache is dropped) changes where column entries
    are read, never the result -- and, holding graph data, serves any walk."""
    rp, col = g16
    V = len(rp) - 1
    g, e = _eng(lt, rp, col, 256 << 10, partitions=6, sched=sched, seed=9, hot_tier=50)
    W = 300000
    want, _, st = oracle.ppr(rp, col, 0, W, prob=0.15, seed=9)
    for r in range(3):
        assert (e.ppr(0, W, 0.15) == want).all()
        s = e.stats()
        assert s["moves"] == st[1]
        if r == 0:
            assert s["hot_vertices"] == 0 and s["tier_build_ms"] > 0
        else:
            assert s["hot_vertices"] > 0
        if r == 1:
            e.drop_cache()
    pr_want, _ = oracle.pagerank(rp, col, 2 * V, length=8, runs=2, seed=9, start_mode=1)
    assert (e.pagerank(2 * V, length=8, runs=2, start=1) == pr_want).all()
    assert e.stats()["hot_vertices"] > 0


def test_hot_tier_c2s(lt, require_gpu, c2s):
    """c2s with a tier of half the budget: the second run reads hot vertices
    from the tier and still gives the oracle's counts, with fewer zero-copy
    bytes than the first."""
    g, W, want, st = c2s
    e = lt.Engine(g, partitions=16, batch=1 << 22, seed=1, sched=2, hot_tier=50)
    first = e.ppr(0, W, 0.15)
    s1 = e.stats()
    e.drop_cache()
    second = e.ppr(0, W, 0.15)
    s2 = e.stats()
    assert (first == want).all() and (second == want).all()
    assert s1["hot_vertices"] == 0 and s2["hot_vertices"] > 0
    assert s2["zerocopy_bytes"] < s1["zerocopy_bytes"]
    e.close()
