"""CPU oracle for the LightTraffic random-walk path.

TEST INFRASTRUCTURE ONLY.  This package is the checker the CUDA product is
compared against; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.

* walks, partitioner and RMAT generator: ``oracle.c`` (C + OpenMP), loaded
  here through ctypes;
* file formats (numpy restatements):
    - ``.bcsr``: ``u32 V | u64 E | u64 rowptr[V+1] | u32 col[E]``, packed
      12-byte header (src/GraphLoader.h:30-48, readme.md "Datasets");
    - ``.part``: ``u16 P | u64 partitionSizeBytes | u32 nodeOffset[P+1] |
      u64 edgeOffset[P+1]``, no padding (src/partition/PartitionStrategy.h:
      76-97 reads it, :325-337 writes it).

Pinning: the partitioner and ``.part`` bytes are pinned to the reference's
own ``EqualSizeStrategy`` (compiled from its sources into ``_ref/``); Philox
to the Random123 known-answer vectors.  Walk outputs: parity unpinned against
reference outputs (the reference's cuRAND seed is uninitialised,
src/Rand.h:29-30); pinned to its sum invariants and hand-checked graphs.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PARTITION = os.path.join(HERE, "_ref", "ref_partition")

APP_PPR, APP_PAGERANK, APP_WALK = 0, 1, 2
START_SOURCE, START_UNIFORM, START_PER_VERTEX = 0, 1, 2
INVALID_NODE = 0xFFFFFFFF

_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or (
        os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "oracle.c"))
    ):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        u32p, u64p = C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)
        L.orc_philox.argtypes = [u32p, u32p, u32p]
        L.orc_threshold53.argtypes = [C.c_float]
        L.orc_threshold53.restype = C.c_uint64
        L.orc_ppr_length.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint64]
        L.orc_ppr_length.restype = C.c_uint32
        L.orc_walk_batch.argtypes = [
            C.c_int, C.c_uint32, u64p, u32p, C.c_int, C.c_uint32, C.c_uint64, C.c_uint32,
            C.c_float, C.c_uint32, C.c_uint64, u64p, u32p, u32p, u64p, C.c_int]
        L.orc_partition.argtypes = [u64p, C.c_uint32, C.c_uint64, u32p, u64p, C.c_uint32, u32p]
        L.orc_rmat_degrees.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.c_uint32, u64p, C.c_int]
        L.orc_rmat_fill.argtypes = [C.c_int, C.c_uint64, C.c_uint32, C.c_uint32, u64p, u32p, C.c_int]
        L.orc_rmat_compact.argtypes = [C.c_uint64, C.c_uint64, u64p, u32p, u32p, C.POINTER(C.c_uint8), u64p,
                                       C.POINTER(C.c_uint64), C.c_int]
        _lib = L
    return _lib


def _p(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


# ------------------------------------------------------------------ RNG

def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox(_p(c, C.c_uint32), _p(k, C.c_uint32), _p(out, C.c_uint32))
    return out


def threshold53(p: float) -> int:
    return int(lib().orc_threshold53(C.c_float(p)))


def ppr_length(seed: int, run: int, idx: int, prob: float) -> int:
    return int(lib().orc_ppr_length(seed, run, idx, threshold53(prob)))


# ---------------------------------------------------------------- walks

def walk_batch(app, rowptr, col, *, start_mode, source=0, walkers, length=0, prob=0.15,
               run=0, seed=1, counts=None, endpoints=False, paths=False, threads=0):
    rowptr = np.ascontiguousarray(rowptr, dtype=np.uint64)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    V = len(rowptr) - 1
    if counts is None:
        counts = np.zeros(V, dtype=np.uint64)
    ep = np.zeros(walkers, dtype=np.uint32) if endpoints else None
    pa = np.zeros(walkers * (length + 1), dtype=np.uint32) if paths else None
    stats = np.zeros(3, dtype=np.uint64)
    rc = lib().orc_walk_batch(app, V, _p(rowptr, C.c_uint64), _p(col, C.c_uint32), start_mode,
                              source, walkers, length, C.c_float(prob), run, seed,
                              _p(counts, C.c_uint64), _p(ep, C.c_uint32), _p(pa, C.c_uint32),
                              _p(stats, C.c_uint64), threads)
    if rc != 0:
        raise ValueError(f"oracle walk rejected its arguments (rc={rc})")
    return counts, ep, pa, stats


def ppr(rowptr, col, source, walkers, prob=0.15, seed=1, threads=0, endpoints=False):
    """Per-vertex endpoint counts of `walkers` PPR walks from `source`."""
    c, ep, _, st = walk_batch(APP_PPR, rowptr, col, start_mode=START_SOURCE, source=source,
                              walkers=walkers, prob=prob, seed=seed, threads=threads,
                              endpoints=endpoints)
    return c, ep, st


def pagerank(rowptr, col, walkers, length=10, runs=1, alpha=0.85, start_mode=START_UNIFORM,
             seed=1, threads=0):
    """Visit counts of `runs` epochs of `walkers` fixed-length PageRank walks."""
    V = len(rowptr) - 1
    counts = np.zeros(V, dtype=np.uint64)
    stats = np.zeros(3, dtype=np.uint64)
    for r in range(runs):
        _, _, _, st = walk_batch(APP_PAGERANK, rowptr, col, start_mode=start_mode,
                                 walkers=walkers, length=length, prob=alpha, run=r,
                                 seed=seed, counts=counts, threads=threads)
        stats += st
    return counts, stats


def generic_walk(rowptr, col, walkers, length=10, start_mode=START_UNIFORM, run=0, seed=1,
                 paths=False, threads=0):
    _, ep, pa, st = walk_batch(APP_WALK, rowptr, col, start_mode=start_mode, walkers=walkers,
                               length=length, run=run, seed=seed, endpoints=True, paths=paths,
                               threads=threads)
    return ep, pa, st


# ----------------------------------------------------------- partitioner

def partition(rowptr, max_bytes: int, cap: int = 1 << 20):
    """EqualSizeStrategy::init restated (src/partition/PartitionStrategy.h:189-218)."""
    rowptr = np.ascontiguousarray(rowptr, dtype=np.uint64)
    V = len(rowptr) - 1
    node_off = np.zeros(cap + 1, dtype=np.uint32)
    edge_off = np.zeros(cap + 1, dtype=np.uint64)
    P = C.c_uint32(0)
    rc = lib().orc_partition(_p(rowptr, C.c_uint64), V, max_bytes, _p(node_off, C.c_uint32),
                             _p(edge_off, C.c_uint64), cap + 1, C.byref(P))
    if rc == -2:
        raise ValueError("a vertex does not fit into the partition size")
    if rc != 0:
        raise ValueError(f"partitioner failed (rc={rc})")
    n = P.value
    return node_off[: n + 1].copy(), edge_off[: n + 1].copy()


# --------------------------------------------------------------- formats

def write_bcsr(path, rowptr, col):
    rowptr = np.ascontiguousarray(rowptr, dtype="<u8")
    col = np.ascontiguousarray(col, dtype="<u4")
    with open(path, "wb") as f:
        f.write(struct.pack("<IQ", len(rowptr) - 1, len(col)))
        f.write(rowptr.tobytes())
        f.write(col.tobytes())


def read_bcsr(path):
    with open(path, "rb") as f:
        V, E = struct.unpack("<IQ", f.read(12))
        rowptr = np.frombuffer(f.read(8 * (V + 1)), dtype="<u8").astype(np.uint64)
        col = np.frombuffer(f.read(4 * E), dtype="<u4").astype(np.uint32)
    if len(rowptr) != V + 1 or len(col) != E:
        raise ValueError("truncated bcsr file")
    return rowptr, col


def write_part(path, part_bytes, node_off, edge_off):
    P = len(node_off) - 1
    with open(path, "wb") as f:
        f.write(struct.pack("<HQ", P, part_bytes))
        f.write(np.ascontiguousarray(node_off, dtype="<u4").tobytes())
        f.write(np.ascontiguousarray(edge_off, dtype="<u8").tobytes())


def read_part(path):
    with open(path, "rb") as f:
        P, size = struct.unpack("<HQ", f.read(10))
        node_off = np.frombuffer(f.read(4 * (P + 1)), dtype="<u4").astype(np.uint32)
        edge_off = np.frombuffer(f.read(8 * (P + 1)), dtype="<u8").astype(np.uint64)
    return P, size, node_off, edge_off


# ------------------------------------------------------------------ RMAT

def rmat_thresholds(a=0.57, b=0.19, c=0.19, d=0.05):
    """16-bit thresholds: source bit is 1 iff lane >= t_src; destination bit is
    1 iff lane >= t_d0 (source bit 0) or t_d1 (source bit 1)."""
    def q(p):
        return int(p * 65536.0 + 0.5)
    return q(a + b), q(a / (a + b)), q(c / (c + d))


def rmat(scale, edges, seed=1, a=0.57, b=0.19, c=0.19, d=0.05, remove_isolated=True, threads=0):
    t_src, t_d0, t_d1 = rmat_thresholds(a, b, c, d)
    V0 = 1 << scale
    deg = np.zeros(V0, dtype=np.uint64)
    L = lib()
    L.orc_rmat_degrees(scale, edges, seed, t_src, _p(deg, C.c_uint64), threads)
    rowptr = np.zeros(V0 + 1, dtype=np.uint64)
    np.cumsum(deg, out=rowptr[1:])
    col = np.zeros(edges, dtype=np.uint32)
    L.orc_rmat_fill(scale, seed, t_d0, t_d1, _p(rowptr, C.c_uint64), _p(col, C.c_uint32), threads)
    if not remove_isolated:
        return rowptr, col
    # tools/rm_isolated_vertices.cc:70-87: keep vertices that appear in any
    # edge, in order (orc_rmat_compact, OpenMP; col is rewritten in place)
    del deg
    newid = np.empty(V0, dtype=np.uint32)
    present = np.empty(V0, dtype=np.uint8)
    out = np.empty(V0 + 1, dtype=np.uint64)
    V = C.c_uint64(0)
    L.orc_rmat_compact(V0, edges, _p(rowptr, C.c_uint64), _p(col, C.c_uint32), _p(newid, C.c_uint32),
                       _p(present, C.c_uint8), _p(out, C.c_uint64), C.byref(V), threads)
    del newid, present, rowptr
    return out[: V.value + 1].copy(), col


# ------------------------------------------------- reference partitioner

def ref_partition(bcsr_path: str, max_bytes: int):
    """Run the reference's own EqualSizeStrategy (built from its sources by
    ``make -C oracle ref``).  Writes ``<bcsr_path>.part`` and returns the
    offsets it printed; raises ValueError on the reference's oversize error."""
    out = subprocess.run([REF_PARTITION, bcsr_path, str(max_bytes)], capture_output=True,
                         text=True)
    lines = [l for l in out.stdout.splitlines() if l and not l.startswith("node with max")]
    if out.returncode == 3:
        raise ValueError(lines[-1] if lines else "reference partitioner error")
    out.check_returncode()
    pairs = [tuple(int(x) for x in l.split()) for l in lines]
    return (np.array([p[0] for p in pairs], dtype=np.uint32),
            np.array([p[1] for p in pairs], dtype=np.uint64))


# ------------------------------------------------- learned prefetcher MLP

MLP_IN, MLP_HIDDEN = 16, 64
MLP_PARAMS = MLP_IN * MLP_HIDDEN + 2 * MLP_HIDDEN + 1


def mlp_forward_backward(x, y, params):
    """Float64 restatement of the prefetcher network: 2 layers, ReLU, mean
    squared error.  Parameter layout W1[i*H+j] | b1 | W2 | b2.  Returns
    (pred, grad, loss)."""
    F, H = MLP_IN, MLP_HIDDEN
    x = np.asarray(x, np.float64).reshape(-1, F)
    y = np.asarray(y, np.float64).reshape(-1)
    p = np.asarray(params, np.float64)
    W1 = p[: F * H].reshape(F, H)
    b1 = p[F * H: F * H + H]
    W2 = p[F * H + H: F * H + 2 * H]
    b2 = p[-1]
    a = x @ W1 + b1
    h = np.maximum(a, 0.0)
    pred = h @ W2 + b2
    n = len(x)
    diff = pred - y
    loss = float(np.mean(diff * diff))
    dy = 2.0 * diff / n
    gW2 = h.T @ dy
    gb2 = dy.sum()
    da = dy[:, None] * W2[None, :] * (a > 0)
    gW1 = x.T @ da
    gb1 = da.sum(axis=0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2, [gb2]])
    return pred, grad, loss


# ------------------------------------------------------ edge-list converter

EDGES_DIRECTED, EDGES_KEEP_DUPLICATES, EDGES_KEEP_SELF_LOOPS, EDGES_KEEP_ISOLATED = 1, 2, 4, 8


def convert_edge_list(path, flags=0):
    """Text edge list -> (rowptr u64[V+1], col u32[E]), restating the
    reference's converter_txt (tools/convert_from_txt.cc:66-218) in numpy:
    a line is used only if its first character is a digit and it holds two
    unsigned ids (read_txt, :66-103); self loops are dropped (:88-91); ids
    that appear in no edge are removed, the rest renumbered in order
    (remove_isolated_vertices, :105-140); every edge is added in both
    directions, the list sorted by (source, destination) and deduplicated
    (to_undirected, :142-166).  `flags` (EDGES_*) switch steps off."""
    src, dst = [], []
    with open(path, "rb") as f:
        for line in f:
            if not line[:1].isdigit():
                continue
            parts = line.split()
            if len(parts) < 2 or not parts[0].isdigit() or not parts[1].isdigit():
                continue
            a, b = int(parts[0]), int(parts[1])
            if a == b and not flags & EDGES_KEEP_SELF_LOOPS:
                continue
            src.append(a)
            dst.append(b)
    if not src:
        raise ValueError("no edges")
    s = np.array(src, dtype=np.uint64)
    d = np.array(dst, dtype=np.uint64)
    if flags & EDGES_KEEP_ISOLATED:
        V = int(max(s.max(), d.max())) + 1
    else:
        ids = np.unique(np.concatenate([s, d]))
        V = len(ids)
        s = np.searchsorted(ids, s).astype(np.uint64)
        d = np.searchsorted(ids, d).astype(np.uint64)
    if not flags & EDGES_DIRECTED:
        s, d = np.concatenate([s, d]), np.concatenate([d, s])
    key = (s << np.uint64(32)) | d
    key = np.sort(key) if flags & EDGES_KEEP_DUPLICATES else np.unique(key)
    rows = (key >> np.uint64(32)).astype(np.int64)
    rowptr = np.zeros(V + 1, dtype=np.uint64)
    np.add.at(rowptr, rows + 1, 1)
    return np.cumsum(rowptr).astype(np.uint64), (key & np.uint64(0xFFFFFFFF)).astype(np.uint32)
