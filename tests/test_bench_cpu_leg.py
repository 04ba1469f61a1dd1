"""bench.py's cpu_baseline leg runs the oracle in a child process without a
CUDA context, the graph passed through an in-memory file: its rate and its
outputs must be those of the same sample run in this process."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402
import oracle  # noqa: E402


def _graph():
    return oracle.rmat(14, 1 << 18, seed=3)


def test_child_leg_counts_equal_in_process_counts():
    rp, col = _graph()
    cpu, got = bench.cpu_baseline_leg("c2s", bench.CONFIGS["c2s"], rp, col, 0.2)
    _, want = bench._cpu_baseline_here("c2s", bench.CONFIGS["c2s"], rp, col, 0.2)
    assert cpu["kind"] == "port" and cpu["value"] > 0 and cpu["cores"] >= 1
    assert got.dtype == want.dtype and np.array_equal(got, want)
    assert int(got.sum()) == 2 * (len(rp) - 1)   # one endpoint per PPR walk


def test_child_leg_per_query_outputs():
    rp, col = _graph()
    _, got = bench.cpu_baseline_leg("c3s", bench.CONFIGS["c3s"], rp, col, 0.1)
    _, want = bench._cpu_baseline_here("c3s", bench.CONFIGS["c3s"], rp, col, 0.1)
    assert len(got) == len(want) > 0
    for (v1, c1), (v2, c2) in zip(got, want):
        assert np.array_equal(v1, v2) and np.array_equal(c1, c2)
