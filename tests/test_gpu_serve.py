"""Serving: continuous batching of PPR queries on the out-of-core engine.

Each query's counts must equal the oracle's PPR with its seed, whether it
runs alone or while other queries arrive, run and finish around it (the
tolerance is zero: counts are integers)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graph16():
    return oracle.rmat(16, 1 << 20, seed=21)


def _oracle(rp, col, src, w, seed):
    counts, _, _ = oracle.ppr(rp, col, src, w, prob=0.15, seed=seed)
    nz = np.nonzero(counts)[0]
    return dict(zip(nz.tolist(), counts[nz].astype(np.uint32).tolist()))


def _drain(srv, tickets, max_steps=200000):
    out = {}
    for _ in range(max_steps):
        srv.step()
        for t in tickets:
            if t not in out:
                r = srv.result(t)
                if r is not None:
                    out[t] = r
        if len(out) == len(tickets):
            return out
    raise AssertionError("queries did not finish")


@pytest.mark.parametrize("sched", [0, 2, 4])
def test_serve_alone_and_in_mix(lt, require_gpu, graph16, sched):
    rp, col = graph16
    V = len(rp) - 1
    g = lt.Graph.from_csr(rp, col, 256 << 10)
    e = lt.Engine(g, partitions=4, batch=1 << 20, seed=1, sched=sched)
    srv = lt.Server(e, max_active=16, table_slots=1 << 22)
    probe = (17, 20000, 0xABCDEF)
    t = srv.submit(*probe)
    alone = _drain(srv, [t])[t][0]
    assert alone == _oracle(rp, col, *probe)
    # the same query while 40 others with different sources arrive over time
    rng = np.random.default_rng(8)
    tickets, specs = [], []
    for i in range(40):
        spec = (int(rng.integers(0, V)), int(rng.integers(1000, 30000)), int(rng.integers(1, 1 << 60)))
        specs.append(spec)
        tickets.append(srv.submit(*spec))
        if i == 20:
            tp = srv.submit(*probe)
        srv.step()
    res = _drain(srv, tickets + [tp])
    assert res[tp][0] == alone
    for t, spec in list(zip(tickets, specs))[::7]:
        assert res[t][0] == _oracle(rp, col, *spec)
    assert all(r[1] >= 0 for r in res.values())
    srv.close()
    # the engine runs regular calls again after serving (cache state intact)
    got = e.ppr(3, 40000, 0.15)
    want, _, _ = oracle.ppr(rp, col, 3, 40000, prob=0.15, seed=1)
    assert (got == want).all()


def test_serve_admission_limits(lt, require_gpu, graph16):
    rp, col = graph16
    g = lt.Graph.from_csr(rp, col, 256 << 10)
    e = lt.Engine(g, partitions=4, batch=1 << 20, seed=1)
    srv = lt.Server(e, max_active=2, table_slots=1 << 16)
    ts = [srv.submit(5 + i, 5000, 100 + i) for i in range(6)]
    c, a, p = srv.step()
    assert a <= 2 and p >= 4                    # slots and table room bound admission
    res = _drain(srv, ts)
    for i, t in enumerate(ts):
        assert res[t][0] == _oracle(rp, col, 5 + i, 5000, 100 + i)
    srv.close()
