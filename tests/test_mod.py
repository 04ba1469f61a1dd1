"""The walk kernels' integer remainder (no 64-bit division) against native %."""
import numpy as np


def test_mod_matches_native(lt):
    rng = np.random.default_rng(0)
    n = 2_000_000
    x = rng.integers(0, np.iinfo(np.uint64).max, n, dtype=np.uint64, endpoint=True)
    d = np.concatenate([
        rng.integers(1, 1 << 16, n // 4, dtype=np.uint64),
        rng.integers(1 << 16, 1 << 32, n // 4, dtype=np.uint64),
        rng.integers(1, 64, n // 4, dtype=np.uint64),
        (np.uint64(1) << rng.integers(0, 32, n // 4, dtype=np.uint64)) + rng.integers(0, 3, n // 4, dtype=np.uint64)])
    d = np.minimum(d, np.uint64(0xFFFFFFFF))
    edge_x = np.array([0, 1, 2**32 - 1, 2**32, 2**63, 2**64 - 1, 2**64 - 2] * 8, dtype=np.uint64)
    edge_d = np.array([1, 2, 3, 65535, 65536, 65537, 2**31, 2**32 - 1] * 7, dtype=np.uint64)
    x = np.concatenate([x, edge_x])
    d = np.concatenate([d, edge_d])
    out = np.zeros_like(x)
    P = lambda a: a.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_uint64))
    lt.check(lt.lib.lt_mod_check(len(x), P(x), P(d), P(out)))
    assert (out == x % d).all()
