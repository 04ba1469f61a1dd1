"""lt_walk_device_noalloc -- the allocation-free step-kernel entry point.

Callers that cannot allocate device memory (a plugin whose host framework
owns every device allocation and hands over only inputs and outputs, or a
process whose device memory another allocator has reserved) use this entry
point instead of lt_walk_device, which needs a caller-provided scratch
buffer.  Its scratch is a static device array shared by all calls, so this
test checks, through the C ABI, that back-to-back calls give exactly the
outputs of lt_walk_device and of the CPU oracle (integer counts: the
tolerance is zero) -- the shared array must be cleared by each call.

The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _bind(lt):
    f = lt.lib.lt_walk_device_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                  ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_float, ctypes.c_uint32,
                  ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def test_noalloc_matches_walk_device(lt, require_gpu):
    import torch
    noalloc = _bind(lt)
    g = lt.Graph.rmat(15, 1 << 18, seed=5, part_bytes=1 << 30)
    rp, col = g.csr()
    V = g.num_nodes
    dev = torch.device("cuda:0")
    d_rp = torch.from_numpy(rp.view(np.int64)).to(dev)
    d_col = torch.from_numpy(col.view(np.int32)).to(dev)
    d_scr = torch.zeros(lt.lib.lt_walk_scratch_bytes() // 8, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream

    # (app, start, source, walkers, length, prob): PPR, PageRank, PPR again
    calls = [(0, 0, 3, 60000, 0, 0.15), (1, 2, 0, 2 * V, 10, 0.85), (0, 0, 3, 60000, 0, 0.15)]
    for app, start, src, W, length, prob in calls:
        want = torch.zeros(V, dtype=torch.int64, device=dev)
        want_st = torch.zeros(3, dtype=torch.int64, device=dev)
        lt.check(lt.lib.lt_walk_device(app, start, d_rp.data_ptr(), d_col.data_ptr(), V, src, W, length,
                                       ctypes.c_float(prob), 0, 77, want.data_ptr(), None, None,
                                       d_scr.data_ptr(), want_st.data_ptr(), stream))
        got = torch.zeros(V, dtype=torch.int64, device=dev)
        got_st = torch.zeros(3, dtype=torch.int64, device=dev)
        lt.check(noalloc(app, start, d_rp.data_ptr(), d_col.data_ptr(), V, src, W, length,
                         ctypes.c_float(prob), 0, 77, got.data_ptr(), None, None, got_st.data_ptr(), stream))
        torch.cuda.synchronize()
        assert torch.equal(got, want), (app, start)
        assert torch.equal(got_st, want_st)
        expect_sum = W if app == 0 else W * length
        assert int(got.sum().item()) == expect_sum
        if app == 0:
            ref, _, _ = oracle.ppr(rp, col, src, W, prob=prob, seed=77)
        else:
            ref, _ = oracle.pagerank(rp, col, W, length=length, alpha=prob, seed=77, start_mode=start)
        assert (got.cpu().numpy().view(np.uint64) == ref).all(), (app, start)
