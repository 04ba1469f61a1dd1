"""GPU parity: the CUDA step kernels against the CPU oracle, bit-exact.

Every comparison is on the same seeded inputs; the RNG is keyed by walker and
step, so visit counts, endpoints and paths must match exactly -- across
graphs, apps, start modes, runs and launch shapes.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _golden(name):
    return oracle.read_bcsr(os.path.join(GOLDEN, "graphs", f"{name}.bcsr"))


SMALL = ["path4", "hub10", "gaps8", "rmat10", "rmat12"]


@pytest.fixture(scope="module")
def rmat16():
    return oracle.rmat(16, 1 << 20, seed=21)


def _engine(lt, rp, col, **kw):
    g = lt.Graph.from_csr(rp, col, 1 << 30)
    return g, lt.Engine(g, **kw)


@pytest.mark.parametrize("name", SMALL)
@pytest.mark.parametrize("seed", [1, 0xDEADBEEF12345])
def test_ppr_small(lt, require_gpu, name, seed):
    rp, col = _golden(name)
    g, e = _engine(lt, rp, col, seed=seed)
    for prob in (0.15, 0.5, 1.0):
        want, _, st = oracle.ppr(rp, col, 0, 7777, prob=prob, seed=seed)
        got = e.ppr(0, 7777, prob)
        assert (got == want).all(), (name, prob)
        s = e.stats()
        assert s["moves"] == st[1]


@pytest.mark.parametrize("name", SMALL)
@pytest.mark.parametrize("start", [1, 2])
def test_pagerank_small(lt, require_gpu, name, start):
    rp, col = _golden(name)
    V = len(rp) - 1
    g, e = _engine(lt, rp, col, seed=77)
    want, st = oracle.pagerank(rp, col, 3 * V + 5, length=9, runs=3, seed=77, start_mode=start)
    got = e.pagerank(3 * V + 5, length=9, runs=3, start=start)
    assert (got == want).all()
    s = e.stats()
    assert (s["updates"], s["moves"], s["teleports"]) == tuple(int(x) for x in st)


@pytest.mark.parametrize("name", SMALL)
@pytest.mark.parametrize("start", [1, 2])
def test_walk_small(lt, require_gpu, name, start):
    rp, col = _golden(name)
    V = len(rp) - 1
    g, e = _engine(lt, rp, col, seed=5)
    for run in (0, 3):
        ep, pa, _ = oracle.generic_walk(rp, col, 4 * V + 3, length=7, start_mode=start, run=run, seed=5,
                                        paths=True)
        gep, gpa = e.walk(4 * V + 3, length=7, run=run, start=start, paths=True)
        assert (gep == ep).all() and (gpa == pa).all()


def test_launch_shape_does_not_change_results(lt, require_gpu, rmat16):
    rp, col = rmat16
    V = len(rp) - 1
    ref = None
    for ctas in (1, 2, 0):
        g, e = _engine(lt, rp, col, seed=3, ctas_per_sm=ctas)
        c = e.pagerank(2 * V, length=10, start=2)
        p = e.ppr(5, 100000, 0.15)
        if ref is None:
            ref = (c, p)
        assert (c == ref[0]).all() and (p == ref[1]).all()
    want, _ = oracle.pagerank(rp, col, 2 * V, length=10, seed=3, start_mode=2)
    assert (ref[0] == want).all()
    wp, _, _ = oracle.ppr(rp, col, 5, 100000, prob=0.15, seed=3)
    assert (ref[1] == wp).all()


def test_ppr_sources_and_zero_walkers(lt, require_gpu, rmat16):
    rp, col = rmat16
    V = len(rp) - 1
    g, e = _engine(lt, rp, col, seed=8)
    for src in (0, 1, V // 2, V - 1):
        want, _, _ = oracle.ppr(rp, col, src, 20000, prob=0.2, seed=8)
        assert (e.ppr(src, 20000, 0.2) == want).all()
    assert e.ppr(0, 0, 0.15).sum() == 0
    with pytest.raises(lt.LTError):
        e.ppr(V, 10, 0.15)                  # source out of range
    with pytest.raises(lt.LTError):
        e.ppr(0, 10, 0.0)                   # would never terminate


def test_gpu_rmat_matches_oracle(lt, require_gpu):
    for scale, edges, seed in [(10, 1 << 13, 7), (12, 1 << 15, 3), (16, 1 << 20, 21)]:
        g = lt.Graph.rmat(scale, edges, seed=seed, part_bytes=1 << 30)
        rp, col = g.csr()
        wr, wc = oracle.rmat(scale, edges, seed=seed)
        assert (rp == wr).all() and (col == wc).all(), scale


def test_c0_ppr_full_size(lt, require_gpu):
    """c0: RMAT(2^20, 2^24), 32 MB partitions all cached, PPR from 0, W = 2V, p = 0.15."""
    g = lt.Graph.rmat(20, 1 << 24, seed=1, part_bytes=32 << 20)
    rp, col = g.csr()
    V = g.num_nodes
    assert g.num_partitions >= 3
    e = lt.Engine(g, seed=1)
    got = e.ppr(0, 2 * V, 0.15)
    want, _, st = oracle.ppr(rp, col, 0, 2 * V, prob=0.15, seed=1)
    assert (got == want).all()
    assert got.sum() == 2 * V
    assert e.stats()["moves"] == st[1]


def test_c1_pagerank_and_walk_full_size(lt, require_gpu):
    """c1: RMAT(2^23, 2^27), 2V walkers one per vertex, PageRank l=10 teleport 0.15,
    generic walk l=10 -- bit-exact against the oracle."""
    g = lt.Graph.rmat(23, 1 << 27, seed=1, part_bytes=32 << 20)
    rp, col = g.csr()
    V = g.num_nodes
    assert g.num_partitions >= 18
    e = lt.Engine(g, seed=1)
    got = e.pagerank(2 * V, length=10, start=2)
    assert got.sum() == 2 * V * 10
    want, _ = oracle.pagerank(rp, col, 2 * V, length=10, seed=1, start_mode=2)
    assert (got == want).all()
    gep, _ = e.walk(2 * V, length=10, start=2)
    wep, _, _ = oracle.generic_walk(rp, col, 2 * V, length=10, start_mode=2, seed=1)
    assert (gep == wep).all()


def test_device_entry_point(lt, require_gpu, rmat16):
    """lt_walk_device on caller device buffers (torch allocations as plumbing)."""
    import ctypes
    import torch
    rp, col = rmat16
    V = len(rp) - 1
    d_rp = torch.from_numpy(rp.view(np.int64)).cuda()
    d_col = torch.from_numpy(col.view(np.int32)).cuda()
    d_cnt = torch.zeros(V, dtype=torch.int64, device="cuda")
    d_scr = torch.zeros(lt.lib.lt_walk_scratch_bytes() // 8, dtype=torch.int64, device="cuda")
    d_st = torch.zeros(3, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    for rep in range(2):
        d_cnt.zero_()
        lt.check(lt.lib.lt_walk_device(0, 0, d_rp.data_ptr(), d_col.data_ptr(), V, 3, 50000, 0,
                                       ctypes.c_float(0.15), 0, 99, d_cnt.data_ptr(), None, None,
                                       d_scr.data_ptr(), d_st.data_ptr(), stream.cuda_stream))
        torch.cuda.synchronize()
        want, _, _ = oracle.ppr(rp, col, 3, 50000, prob=0.15, seed=99)
        assert (d_cnt.cpu().numpy().view(np.uint64) == want).all()


@pytest.mark.parametrize("app,start,length", [(0, 0, 0), (1, 1, 7), (1, 2, 10), (2, 1, 6)])
def test_compact_entry_point(lt, require_gpu, rmat16, app, start, length):
    """lt_walk_device_compact (u32 row offsets from lt_rowptr_narrow, u32
    counters) gives the oracle's counts, endpoints and paths bit for bit."""
    import ctypes
    import torch
    rp, col = rmat16
    V = len(rp) - 1
    W = 2 * V + 13
    d_rp = torch.from_numpy(rp.view(np.int64)).cuda()
    d_rp32 = torch.zeros(V + 1, dtype=torch.int32, device="cuda")
    d_col = torch.from_numpy(col.view(np.int32)).cuda()
    d_cnt = torch.zeros(V, dtype=torch.int32, device="cuda")
    d_ep = torch.zeros(W, dtype=torch.int32, device="cuda")
    d_pa = torch.zeros(W * (length + 1) if app == 2 else 1, dtype=torch.int32, device="cuda")
    d_scr = torch.zeros(lt.lib.lt_walk_scratch_bytes() // 8, dtype=torch.int64, device="cuda")
    d_st = torch.zeros(3, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    lt.check(lt.lib.lt_rowptr_narrow(d_rp.data_ptr(), d_rp32.data_ptr(), V, s))
    for rep in range(2):
        d_cnt.zero_()
        d_st.zero_()
        lt.check(lt.lib.lt_walk_device_compact(app, start, d_rp32.data_ptr(), d_col.data_ptr(), V, 5, W, length,
                                               ctypes.c_float(0.15 if app == 0 else 0.85), 3, 77,
                                               d_cnt.data_ptr() if app != 2 else None, d_ep.data_ptr(),
                                               d_pa.data_ptr() if app == 2 else None, d_scr.data_ptr(),
                                               d_st.data_ptr(), s))
        torch.cuda.synchronize()
        ep = d_ep.cpu().numpy().view(np.uint32)
        if app != 2:
            want, wep, _, st = oracle.walk_batch(app, rp, col, start_mode=start, source=5, walkers=W, length=length,
                                                 prob=0.15 if app == 0 else 0.85, run=3, seed=77, endpoints=True)
            assert (d_cnt.cpu().numpy().view(np.uint32).astype(np.uint64) == want).all()
            assert (ep == wep).all()
            assert tuple(int(x) for x in d_st.cpu().numpy()) == tuple(int(x) for x in st)
        else:
            wep, wpa, _ = oracle.generic_walk(rp, col, W, length=length, start_mode=start, run=3, seed=77,
                                              paths=True)
            assert (ep == wep).all()
            assert (d_pa.cpu().numpy().view(np.uint32) == wpa.ravel()).all()


def test_device_remainder_matches_native(lt, require_gpu):
    """The device build of the integer remainder (no 64-bit division): the
    three-remainder path below 2^16 and the single-precision estimate with
    integer correction from 2^16 to 2^32, against native %."""
    import torch
    rng = np.random.default_rng(3)
    n = 4_000_000
    x = rng.integers(0, np.iinfo(np.uint64).max, n, dtype=np.uint64, endpoint=True)
    d = np.concatenate([
        rng.integers(1, 1 << 16, n // 4, dtype=np.uint64),
        rng.integers(1 << 16, 1 << 32, n // 4, dtype=np.uint64),
        (np.uint64(1) << rng.integers(16, 32, n // 4, dtype=np.uint64)) - rng.integers(0, 3, n // 4, dtype=np.uint64),
        (np.uint64(1) << rng.integers(16, 32, n // 4, dtype=np.uint64)) + rng.integers(0, 3, n // 4, dtype=np.uint64)])
    d = np.minimum(d, np.uint64(0xFFFFFFFF))
    edge_x = np.array([0, 1, 2**32 - 1, 2**32, 2**63, 2**64 - 1, 2**64 - 2] * 9, dtype=np.uint64)
    edge_d = np.array([1, 2, 3, 65535, 65536, 65537, 2**31, 2**32 - 1, 2**32 - 2] * 7, dtype=np.uint64)
    x = np.concatenate([x, edge_x])
    d = np.concatenate([d, edge_d])
    dev = torch.device("cuda:0")
    tx = torch.from_numpy(x.view(np.int64)).to(dev)
    td = torch.from_numpy(d.view(np.int64)).to(dev)
    to = torch.empty_like(tx)
    lt.check(lt.lib.lt_mod_check_device(len(x), tx.data_ptr(), td.data_ptr(), to.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    got = to.cpu().numpy().view(np.uint64)
    assert (got == x % d).all()


def test_hub_degrees_above_2_16(lt, require_gpu):
    """Walks through hubs whose degrees need the large-divisor remainder
    (65 536 .. 1 048 583 out-edges): counts, endpoints and paths bit-exact."""
    degs = [1 << 16, (1 << 16) + 1, 100003, (1 << 20) + 7]
    leaves = 1 << 12
    H = len(degs)
    V = H + leaves
    rows, cols = [], []
    rng = np.random.default_rng(5)
    for h, dg in enumerate(degs):
        rows.append(np.full(dg, h, np.uint32))
        cols.append((H + rng.integers(0, leaves, dg)).astype(np.uint32))
    for v in range(H, V):   # every leaf links back to two hubs
        rows.append(np.full(2, v, np.uint32))
        cols.append(rng.integers(0, H, 2).astype(np.uint32))
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    order = np.argsort(r, kind="stable")
    r, c = r[order], c[order]
    rp = np.zeros(V + 1, np.uint64)
    np.add.at(rp, r.astype(np.int64) + 1, 1)
    rp = np.cumsum(rp).astype(np.uint64)
    g, e = _engine(lt, rp, c, seed=17)
    want, _, _ = oracle.ppr(rp, c, 3, 200000, prob=0.15, seed=17)
    assert (e.ppr(3, 200000, 0.15) == want).all()
    ep, pa, _ = oracle.generic_walk(rp, c, 50000, length=12, start_mode=1, seed=17, paths=True)
    gep, gpa = e.walk(50000, length=12, start=1, paths=True)
    assert (gep == ep).all() and (gpa == pa).all()


def _ref_cases():
    import json
    with open(os.path.join(GOLDEN, "ref_walks.json")) as f:
        return [c for c in json.load(f)["cases"] if not (c["app"] == "ppr" and c["runs"] > 1)]


@pytest.mark.parametrize("case", _ref_cases(), ids=lambda c: f"{c['app']}-{c['graph']}-s{c['start']}-{c['seed']:x}")
def test_engine_matches_reference_update_vectors(lt, require_gpu, case):
    """The CUDA engine against the outputs of the reference's own App::update
    code (tests/golden/ref_walks.json), resident and out of core."""
    import hashlib
    rp, col = _golden(case["graph"])
    W, L = case["walkers"], case["length"]

    def digest(arrays):
        return [{"sha256": hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest(),
                 "sum": int(a.astype(np.uint64).sum())} for a in arrays]

    V = len(rp) - 1
    fit = 24 + 4 * int(np.diff(rp.astype(np.int64)).max())   # the largest vertex's rowptr pair and edges
    for part_bytes, kw in ((1 << 30, {}), (max(fit, (8 * (V + 1) + 4 * len(col)) // 3), dict(partitions=1))):
        g = lt.Graph.from_csr(rp, col, part_bytes)
        if kw and g.num_partitions < 2:
            continue
        e = lt.Engine(g, seed=case["seed"], **kw)
        if case["app"] == "ppr":
            got = [e.ppr(case["source"], W, case["prob"])]
        elif case["app"] == "pagerank":
            got = [e.pagerank(W, length=L, runs=case["runs"], start=case["start"], alpha=case["prob"])]
        else:
            got = list(e.walk(W, length=L, run=case["run0"], start=case["start"], paths=True))
        assert digest(got) == case["outputs"], kw


@pytest.mark.parametrize("app,start", [(0, 0), (1, 1), (1, 2), (2, 1)])
def test_packed_layout_matches_oracle(lt, require_gpu, rmat16, app, start):
    """lt_walk_device_packed (row offset and counter of a vertex side by side)
    against the oracle: counts, endpoints and paths bit-exact."""
    import ctypes
    import torch
    rp, col = rmat16
    V = len(rp) - 1
    dev = torch.device("cuda:0")
    d_rp = torch.from_numpy(rp.view(np.int64)).to(dev)
    d_col = torch.from_numpy(col.view(np.int32)).to(dev)
    d_rows = torch.empty(2 * (V + 1), dtype=torch.int32, device=dev)
    d_scr = torch.zeros(lt.lib.lt_walk_scratch_bytes() // 8, dtype=torch.int64, device=dev)
    d_st = torch.zeros(3, dtype=torch.int64, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    W, L = 3 * V + 11, 7
    paths = app == 2
    d_ep = torch.zeros(W, dtype=torch.int32, device=dev)
    d_pa = torch.zeros(W * (L + 1), dtype=torch.int32, device=dev) if paths else None
    lt.check(lt.lib.lt_rows_pack(d_rp.data_ptr(), d_rows.data_ptr(), V, st))
    lt.check(lt.lib.lt_walk_device_packed(app, start, d_rows.data_ptr(), d_col.data_ptr(), V, 5, W, L if app else 0,
                                          ctypes.c_float(0.15 if app == 0 else 0.85), 3, 41, d_ep.data_ptr(),
                                          d_pa.data_ptr() if paths else None, d_scr.data_ptr(), d_st.data_ptr(), st))
    d_cnt = torch.zeros(V, dtype=torch.int64, device=dev)
    lt.check(lt.lib.lt_rows_counts(d_rows.data_ptr(), d_cnt.data_ptr(), V, st))
    torch.cuda.synchronize()
    got_ep = d_ep.cpu().numpy().view(np.uint32)
    if app == 0:
        want, ep, _ = oracle.walk_batch(oracle.APP_PPR, rp, col, start_mode=0, source=5, walkers=W, prob=0.15, run=3,
                                        seed=41, endpoints=True)[:3]
    elif app == 1:
        want, ep, _, _ = oracle.walk_batch(oracle.APP_PAGERANK, rp, col, start_mode=start, walkers=W, length=L,
                                           prob=0.85, run=3, seed=41, endpoints=True)
    else:
        _, ep, pa, _ = oracle.walk_batch(oracle.APP_WALK, rp, col, start_mode=start, walkers=W, length=L, run=3,
                                         seed=41, endpoints=True, paths=True)
        assert (d_pa.cpu().numpy().view(np.uint32) == pa).all()
    assert (got_ep == ep).all()
    if app != 2:
        assert (d_cnt.cpu().numpy().view(np.uint64) == want).all()
    # the row offsets are untouched by the walk
    assert (d_rows.cpu().numpy().view(np.uint32)[0::2] == rp.astype(np.uint32)).all()
