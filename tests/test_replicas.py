"""Replica timing aggregation of bench.py on CPU: two gloo ranks join the
process group, take the barrier and agree on the maximum of their times --
the same calls the benchmark makes around its timed region at N > 1."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update(WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    ws, r, local, dist = bench.init_dist()
    assert (ws, r) == (2, rank) and dist is not None and dist.get_backend() == "gloo"
    dist.barrier()
    out[rank] = bench.max_over_ranks(dist, local, 10.0 + 5.0 * rank)
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_max_time():
    if torch.cuda.is_available():
        pytest.skip("the GPU path uses NCCL; this test covers the CPU (gloo) path")
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    mp.start_processes(_rank, args=(port, out), nprocs=2, join=True, start_method="spawn")
    assert dict(out) == {0: 15.0, 1: 15.0}
