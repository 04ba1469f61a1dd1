"""Checkpoint / resume of out-of-core runs.

A run interrupted at a checkpoint and finished by lt_resume -- on another
engine with another cache size, walker pool, scheduler and engine seed --
gives the oracle's counts, endpoints and paths bit for bit: every draw is
keyed by walker and step, so the schedule never shows in the results.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g16():
    return oracle.rmat(16, 1 << 20, seed=21)


def _engine(lt, rp, col, **kw):
    g = lt.Graph.from_csr(rp, col, 256 << 10)
    return g, lt.Engine(g, **kw)


@pytest.mark.parametrize("sched", [0, 2, 4])
def test_ppr_interrupt_and_resume(lt, require_gpu, g16, sched, tmp_path):
    rp, col = g16
    W = 300000
    want, _, _ = oracle.ppr(rp, col, 0, W, prob=0.15, seed=9)
    g, e = _engine(lt, rp, col, partitions=4, batch=20000, sched=sched, seed=9)   # tiny pool: host spills
    path = tmp_path / "run.ckpt"
    e.checkpoint(path, every=3, stop=True)
    with pytest.raises(lt.LTError) as ei:
        e.ppr(0, W, 0.15)
    assert ei.value.status == lt.INTERRUPTED
    info = lt.checkpoint_info(path)
    assert info["iteration"] == 3 and info["num_walkers"] == W and info["app"] == 0
    _, e2 = _engine(lt, rp, col, partitions=2, batch=0, sched=0, seed=12345)
    assert (e2.resume(path) == want).all()
    # the interrupted engine runs normally again once disarmed
    e.checkpoint(None, 0)
    assert (e.ppr(0, W, 0.15) == want).all()


def test_pagerank_checkpoint_in_second_run(lt, require_gpu, g16, tmp_path):
    """Periodic checkpoints while the call completes; the last one falls in
    the second of two runs and resuming it reproduces the whole call."""
    rp, col = g16
    V = len(rp) - 1
    want, _ = oracle.pagerank(rp, col, 2 * V, length=8, runs=2, seed=4, start_mode=2)
    g, e = _engine(lt, rp, col, partitions=4, sched=2, seed=4)
    path = tmp_path / "pr.ckpt"
    e.checkpoint(path, every=2)
    assert (e.pagerank(2 * V, length=8, runs=2, start=2) == want).all()
    info = lt.checkpoint_info(path)
    assert info["runs"] == 2
    _, e2 = _engine(lt, rp, col, partitions=3, sched=4, seed=1)
    assert (e2.resume(path) == want).all()


@pytest.mark.parametrize("start", [1, 2])
def test_walk_paths_resume(lt, require_gpu, g16, start, tmp_path):
    rp, col = g16
    V = len(rp) - 1
    ep, pa, _ = oracle.generic_walk(rp, col, V + 77, length=6, start_mode=start, run=1, seed=6, paths=True)
    g, e = _engine(lt, rp, col, partitions=4, sched=0, seed=6)
    path = tmp_path / "walk.ckpt"
    e.checkpoint(path, every=2, stop=True)
    with pytest.raises(lt.LTError):
        e.walk(V + 77, length=6, run=1, start=start, paths=True)
    _, e2 = _engine(lt, rp, col, partitions=5, sched=2, seed=0)
    gep, gpa = e2.resume(path)
    assert (gep == ep).all() and (gpa == pa).all()


def test_resume_rejects_other_graph(lt, require_gpu, g16, tmp_path):
    rp, col = g16
    g, e = _engine(lt, rp, col, partitions=4, seed=9)
    path = tmp_path / "x.ckpt"
    e.checkpoint(path, every=2, stop=True)
    with pytest.raises(lt.LTError):
        e.ppr(0, 100000, 0.15)
    rp2, col2 = oracle.rmat(15, 1 << 19, seed=3)
    _, e2 = _engine(lt, rp2, col2, partitions=2, seed=9)
    with pytest.raises(lt.LTError) as ei:
        e2.resume(path)
    assert ei.value.status == 1


def _first_queue(raw, V, P):
    """Offset of the first non-empty queue record block of a PPR checkpoint
    (header 96 B, device statistics 64 B, counts u64[V], then per partition
    u64 lazy_total, lazy_next, n and u32 cur[n], step[n], idx[n], query[n])."""
    off = 96 + 64 + 8 * V
    for _ in range(P):
        n = int(np.frombuffer(raw, np.uint64, 3, off)[2])
        if n:
            return off + 24, n
        off += 24
    raise AssertionError("no queued walkers in the checkpoint")


@pytest.mark.parametrize("field,value,status", [
    (0, "V", 3),       # vertex outside the graph
    (2, "W", 3),       # walker index beyond the run
    (1, 1, 3),         # a PPR walker in a queue has at least 2 steps left
    (3, 7, 3),         # query slot of a run that serves no queries
    (None, None, 1),   # partition table of another partition size
])
def test_resume_rejects_corrupt_checkpoint(lt, require_gpu, g16, tmp_path, field, value, status):
    """A corrupt checkpoint is refused before any walker reaches the device."""
    rp, col = g16
    V, W = len(rp) - 1, 300000
    g, e = _engine(lt, rp, col, partitions=4, sched=0, seed=9)
    path = tmp_path / "c.ckpt"
    e.checkpoint(path, every=3, stop=True)
    with pytest.raises(lt.LTError):
        e.ppr(0, W, 0.15)
    raw = bytearray(path.read_bytes())
    if field is None:
        raw[80:88] = bytes(a ^ 0xFF for a in raw[80:88])   # the partition-table hash
    else:
        off, n = _first_queue(bytes(raw), V, g.num_partitions)
        v = {"V": V + 5, "W": W + 1}.get(value, value)
        np.frombuffer(raw, np.uint32, 1, off + 4 * n * field)[:] = v
    path.write_bytes(bytes(raw))
    _, e2 = _engine(lt, rp, col, partitions=2, sched=0, seed=1)
    with pytest.raises(lt.LTError) as ei:
        e2.resume(path)
    assert ei.value.status == status
    # the engine stays usable
    want, _, _ = oracle.ppr(rp, col, 0, 5000, prob=0.15, seed=1)
    assert (e2.ppr(0, 5000, 0.15) == want).all()
