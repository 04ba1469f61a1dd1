"""lighttraffic_gb300 -- Python view of the GB300 random-walk engine.

Every call goes through the C ABI of ``include/lighttraffic.h`` in the in-tree
``liblighttraffic.so`` (built by ``lighttraffic_gb300.build``).  There is no
Python or CPU implementation of the walks here: if the library is missing,
importing the package raises.

The names mirror the reference's app surface (app/ppr.cu, app/pagerank.cu,
app/genericwalk.cu and src/Config.h):

    g = Graph.open("G.bcsr", materialize=True, part_mb=32)      # -f G.bcsr -m -s 32
    eng = Engine(g, partitions=0, batch=0, seed=1)              # -p / -b
    counts = eng.ppr(source=0, walkers=2 * g.num_nodes, prob=0.15)
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "liblighttraffic.so")
BIN_DIR = os.path.join(PKG, "bin")

APP_PPR, APP_PAGERANK, APP_WALK = 0, 1, 2
INTERRUPTED = 10  # lt_status: the run stopped at a checkpoint
START_SOURCE, START_UNIFORM, START_PER_VERTEX = 0, 1, 2
SCHED_PLAIN, SCHED_FIFO, SCHED_LEARNED, SCHED_FREQUENCY, SCHED_BATCHED = 0, 1, 2, 3, 4
INVALID_NODE = 0xFFFFFFFF

STATUS = {0: "LT_OK", 1: "LT_ERR_INVALID", 2: "LT_ERR_IO", 3: "LT_ERR_FORMAT", 4: "LT_ERR_NOMEM",
          5: "LT_ERR_CUDA", 6: "LT_ERR_PARTITION", 7: "LT_ERR_TIMEOUT", 8: "LT_ERR_CAPACITY",
          9: "LT_ERR_UNSUPPORTED"}


class LTError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class GraphInfo(C.Structure):
    _fields_ = [("num_nodes", C.c_uint32), ("num_edges", C.c_uint64), ("num_partitions", C.c_uint32),
                ("partition_bytes", C.c_uint64), ("max_nodes_in_partition", C.c_uint32),
                ("max_edges_in_partition", C.c_uint64)]


class EngineCfg(C.Structure):
    _fields_ = [("device", C.c_int), ("num_device_partitions", C.c_uint32),
                ("num_device_walkers", C.c_uint64), ("sched", C.c_int), ("pipeline", C.c_int),
                ("zerocopy_threshold", C.c_uint64), ("seed", C.c_uint64), ("block_size", C.c_int),
                ("ctas_per_sm", C.c_int), ("resident_index", C.c_int), ("zc_group_bytes", C.c_uint64),
                ("sweep_walkers", C.c_uint64), ("load_factor", C.c_uint32), ("bucket_items", C.c_int),
                ("no_prefill", C.c_int), ("hot_tier", C.c_int), ("no_split", C.c_int),
                ("host_plan", C.c_int)]


class BatchTune(C.Structure):
    _fields_ = [("block", C.c_int), ("ctas_per_sm", C.c_int), ("load_shift", C.c_int), ("tuned", C.c_int)]


class OocTune(C.Structure):
    _fields_ = [("tuned", C.c_int), ("trial_walkers", C.c_uint64), ("zc_group_bytes", C.c_uint64),
                ("load_factor", C.c_uint32), ("ctas_per_sm", C.c_int), ("bucket_items", C.c_int),
                ("default_ms", C.c_double), ("tuned_ms", C.c_double)]


class PolicyStats(C.Structure):
    _fields_ = [("name", C.c_char * 16), ("train_steps", C.c_uint64), ("net_loss", C.c_double),
                ("baseline_loss", C.c_double), ("predictions", C.c_uint64), ("net_used", C.c_uint64)]


class CheckpointInfo(C.Structure):
    _fields_ = [("app", C.c_int), ("start_mode", C.c_int), ("source", C.c_uint32), ("length", C.c_uint32),
                ("runs", C.c_uint32), ("run_index", C.c_uint32), ("num_walkers", C.c_uint64),
                ("num_nodes", C.c_uint32), ("has_endpoints", C.c_int), ("has_paths", C.c_int),
                ("iteration", C.c_uint64)]


class Stats(C.Structure):
    _fields_ = [("updates", C.c_uint64), ("moves", C.c_uint64), ("teleports", C.c_uint64),
                ("iterations", C.c_uint64), ("explicit_iterations", C.c_uint64),
                ("h2d_graph_bytes", C.c_uint64), ("h2d_walker_bytes", C.c_uint64),
                ("d2h_walker_bytes", C.c_uint64), ("zerocopy_bytes", C.c_uint64),
                ("partition_loads", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("running_ms", C.c_double), ("graph_loading_ms", C.c_double),
                ("computing_ms", C.c_double), ("zerocopy_ms", C.c_double),
                ("walker_loading_ms", C.c_double), ("walker_evicting_ms", C.c_double),
                ("graph_loading_calls", C.c_uint64), ("computing_calls", C.c_uint64),
                ("zerocopy_calls", C.c_uint64), ("walker_loading_calls", C.c_uint64),
                ("walker_evicting_calls", C.c_uint64), ("step_kernel_ms", C.c_double),
                ("handoffs", C.c_uint64), ("overlap_computes", C.c_uint64),
                ("zerocopy_groups", C.c_uint64), ("zerocopy_sweeps", C.c_uint64),
                ("cache_slots", C.c_uint64), ("index_on_device", C.c_uint64), ("refill_loads", C.c_uint64),
                ("prefill_loads", C.c_uint64),
                ("bucket_ms", C.c_double), ("host_wait_ms", C.c_double), ("device_plans", C.c_uint64),
                ("host_sched_ms", C.c_double), ("host_submit_ms", C.c_double), ("host_replay_ms", C.c_double),
                ("host_observe_ms", C.c_double), ("split_launches", C.c_uint64), ("hot_vertices", C.c_uint64),
                ("tier_build_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run `python lighttraffic_gb300/build.py` "
                          "(the engine has no fallback implementation)")
    L = C.CDLL(LIB_PATH)
    vp, u64p, u32p = C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)
    sig = {
        "lt_strerror": ([C.c_int], C.c_char_p),
        "lt_last_error": ([], C.c_char_p),
        "lt_version": ([], C.c_char_p),
        "lt_graph_open": ([C.c_char_p, C.c_int, C.c_uint64, C.POINTER(vp)], C.c_int),
        "lt_graph_from_csr": ([C.c_uint32, C.c_uint64, u64p, u32p, C.c_uint64, C.POINTER(vp)], C.c_int),
        "lt_graph_from_edge_list": ([C.c_char_p, C.c_int, C.c_uint64, C.POINTER(vp)], C.c_int),
        "lt_graph_generate_rmat": ([C.c_int, C.c_uint32, C.c_uint64, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_uint64, C.c_uint64, C.POINTER(vp)], C.c_int),
        "lt_graph_info_get": ([vp, C.POINTER(GraphInfo)], C.c_int),
        "lt_graph_partitions": ([vp, u32p, u64p], C.c_int),
        "lt_graph_csr": ([vp, C.POINTER(u64p), C.POINTER(u32p)], C.c_int),
        "lt_graph_write_bcsr": ([vp, C.c_char_p], C.c_int),
        "lt_graph_write_part": ([vp, C.c_char_p], C.c_int),
        "lt_graph_close": ([vp], None),
        "lt_partition_equal_size": ([u64p, C.c_uint32, C.c_uint64, u32p, u64p, C.c_uint32, u32p], C.c_int),
        "lt_engine_cfg_default": ([C.POINTER(EngineCfg)], None),
        "lt_engine_create": ([vp, C.POINTER(EngineCfg), C.POINTER(vp)], C.c_int),
        "lt_engine_destroy": ([vp], None),
        "lt_engine_drop_cache": ([vp], C.c_int),
        "lt_run_ppr": ([vp, C.c_uint32, C.c_uint64, C.c_float, u64p], C.c_int),
        "lt_run_pagerank": ([vp, C.c_uint64, C.c_uint32, C.c_uint32, C.c_float, C.c_int, u64p], C.c_int),
        "lt_run_walk": ([vp, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int, u32p, u32p], C.c_int),
        "lt_engine_stats": ([vp, C.POINTER(Stats)], C.c_int),
        "lt_walk_scratch_bytes": ([], C.c_size_t),
        "lt_engine_policy_stats": ([vp, C.POINTER(PolicyStats)], C.c_int),
        "lt_engine_partition_stats": ([vp, u64p, u64p, u64p], C.c_int),
        "lt_mod_check": ([C.c_uint64, u64p, u64p, u64p], C.c_int),
        "lt_mod_check_device": ([C.c_uint64, vp, vp, vp, vp], C.c_int),
        "lt_host_link_gbs": ([C.c_int, C.POINTER(C.c_double)], C.c_int),
        "lt_host_gather_gbs": ([C.c_int, C.c_uint64, C.POINTER(C.c_double)], C.c_int),
        "lt_ppr_batch": ([vp, C.c_uint32, u32p, u64p, u64p, C.c_float, u64p, u32p, u32p, C.c_uint64], C.c_int),
        "lt_ppr_batch_device": ([vp, C.c_uint32, vp, vp, vp, C.c_float, vp, vp, vp, C.c_uint64, vp], C.c_int),
        "lt_engine_autotune": ([vp], C.c_int),
        "lt_engine_ooc_tune": ([vp, C.POINTER(OocTune)], C.c_int),
        "lt_serve_open": ([vp, C.c_uint32, C.c_uint64, C.c_float, C.POINTER(vp)], C.c_int),
        "lt_serve_submit": ([vp, C.c_uint32, C.c_uint64, C.c_uint64, C.c_double, C.POINTER(C.c_uint64)], C.c_int),
        "lt_serve_step": ([vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)], C.c_int),
        "lt_serve_result": ([vp, C.c_uint64, C.POINTER(C.c_int), C.POINTER(C.c_uint64), u32p, u32p, C.c_uint64,
                             C.POINTER(C.c_double)], C.c_int),
        "lt_serve_close": ([vp], None),
        "lt_serve_finished": ([vp, u64p, C.c_uint64], C.c_uint64),
        "lt_serve_now_ms": ([], C.c_double),
        "lt_engine_batch_tune": ([vp, C.POINTER(BatchTune)], C.c_int),
        "lt_mlp_check": ([C.c_int, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float),
                          C.POINTER(C.c_float), C.c_float, C.c_float, C.POINTER(C.c_float),
                          C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
        "lt_walk_device": ([C.c_int, C.c_int, vp, vp, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                            C.c_float, C.c_uint32, C.c_uint64, vp, vp, vp, vp, vp, vp], C.c_int),
        "lt_walk_device_compact": ([C.c_int, C.c_int, vp, vp, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                                    C.c_float, C.c_uint32, C.c_uint64, vp, vp, vp, vp, vp, vp], C.c_int),
        "lt_rowptr_narrow": ([vp, vp, C.c_uint32, vp], C.c_int),
        "lt_walk_device_packed": ([C.c_int, C.c_int, vp, vp, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                                   C.c_float, C.c_uint32, C.c_uint64, vp, vp, vp, vp, vp], C.c_int),
        "lt_rows_pack": ([vp, vp, C.c_uint32, vp], C.c_int),
        "lt_rows_counts": ([vp, vp, C.c_uint32, vp], C.c_int),
        "lt_host_alloc": ([C.c_uint64, C.POINTER(vp)], C.c_int),
        "lt_engine_checkpoint": ([vp, C.c_char_p, C.c_uint64, C.c_int], C.c_int),
        "lt_checkpoint_read_info": ([C.c_char_p, C.POINTER(CheckpointInfo)], C.c_int),
        "lt_resume": ([vp, C.c_char_p, u64p, u32p, u32p], C.c_int),
        "lt_host_free": ([vp], None),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    return L


lib = _load()


def check(status: int):
    if status != 0:
        raise LTError(status, lib.lt_last_error().decode(errors="replace"))


def _ptr(a, ctype):
    return None if a is None else a.ctypes.data_as(C.POINTER(ctype))


def host_link_gbs(device: int = 0) -> float:
    """Pinned host -> device copy bandwidth (GB/s), best of five 1 GiB copies."""
    v = C.c_double(0)
    check(lib.lt_host_link_gbs(device, C.byref(v)))
    return v.value


def host_gather_gbs(device: int = 0, nbytes: int = 0) -> float:
    """Random 32-byte-sector reads from a mapped pinned host buffer of nbytes
    (0 = 2 GiB), GB/s of sectors: the ceiling of zero-copy hops."""
    v = C.c_double(0)
    check(lib.lt_host_gather_gbs(device, nbytes, C.byref(v)))
    return v.value


def partition_equal_size(rowptr, max_bytes: int):
    """EqualSizeStrategy::init (src/partition/PartitionStrategy.h:193-218) on caller arrays."""
    rowptr = np.ascontiguousarray(rowptr, dtype=np.uint64)
    V = len(rowptr) - 1
    cap = V + 2
    no = np.zeros(cap, dtype=np.uint32)
    eo = np.zeros(cap, dtype=np.uint64)
    P = C.c_uint32(0)
    check(lib.lt_partition_equal_size(_ptr(rowptr, C.c_uint64), V, max_bytes, _ptr(no, C.c_uint32),
                                      _ptr(eo, C.c_uint64), cap, C.byref(P)))
    return no[: P.value + 1].copy(), eo[: P.value + 1].copy()


MLP_PARAMS = 16 * 64 + 2 * 64 + 1


def mlp_check(x, y, params, lr=0.0, momentum=0.0, device=0):
    """Forward + backward (+ one SGD step when lr > 0) of the prefetcher
    network on the GPU.  Returns (pred, grad, loss, new_params)."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    params = np.ascontiguousarray(params, np.float32)
    n = len(y)
    pred = np.zeros(n, np.float32)
    grad = np.zeros(MLP_PARAMS, np.float32)
    newp = np.zeros(MLP_PARAMS, np.float32)
    loss = C.c_float(0)
    f = C.POINTER(C.c_float)
    check(lib.lt_mlp_check(device, n, x.ctypes.data_as(f), y.ctypes.data_as(f), params.ctypes.data_as(f),
                           lr, momentum, pred.ctypes.data_as(f), grad.ctypes.data_as(f), C.byref(loss),
                           newp.ctypes.data_as(f)))
    return pred, grad, loss.value, newp


class Graph:
    """A bcsr graph in pinned host memory with its partition table."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle
        info = GraphInfo()
        check(lib.lt_graph_info_get(self._h, C.byref(info)))
        self.info = info

    @classmethod
    def open(cls, path: str, materialize: bool = False, part_mb: int = 32) -> "Graph":
        h = C.c_void_p()
        check(lib.lt_graph_open(path.encode(), int(materialize), part_mb, C.byref(h)))
        return cls(h)

    @classmethod
    def from_csr(cls, rowptr, col, part_bytes: int) -> "Graph":
        rowptr = np.ascontiguousarray(rowptr, dtype=np.uint64)
        col = np.ascontiguousarray(col, dtype=np.uint32)
        h = C.c_void_p()
        check(lib.lt_graph_from_csr(len(rowptr) - 1, len(col), _ptr(rowptr, C.c_uint64),
                                    _ptr(col, C.c_uint32), part_bytes, C.byref(h)))
        return cls(h)

    @classmethod
    def from_edge_list(cls, path, part_bytes: int = 1 << 62, directed: bool = False,
                       keep_duplicates: bool = False, keep_self_loops: bool = False,
                       keep_isolated: bool = False) -> "Graph":
        """Text edge list -> graph, as the reference's converter_txt
        (symmetrised, deduplicated, self loops and isolated ids removed,
        unless the flags say otherwise)."""
        flags = (1 if directed else 0) | (2 if keep_duplicates else 0) | (4 if keep_self_loops else 0) | \
            (8 if keep_isolated else 0)
        h = C.c_void_p()
        check(lib.lt_graph_from_edge_list(os.fsencode(path), flags, part_bytes, C.byref(h)))
        return cls(h)

    @classmethod
    def rmat(cls, scale: int, edges: int, seed: int = 1, part_bytes: int = 32 << 20,
             a=0.57, b=0.19, c=0.19, d=0.05, device: int = 0) -> "Graph":
        h = C.c_void_p()
        check(lib.lt_graph_generate_rmat(device, scale, edges, a, b, c, d, seed, part_bytes,
                                         C.byref(h)))
        return cls(h)

    @property
    def num_nodes(self) -> int:
        return self.info.num_nodes

    @property
    def num_edges(self) -> int:
        return self.info.num_edges

    @property
    def num_partitions(self) -> int:
        return self.info.num_partitions

    def partitions(self):
        P = self.info.num_partitions
        no = np.zeros(P + 1, dtype=np.uint32)
        eo = np.zeros(P + 1, dtype=np.uint64)
        check(lib.lt_graph_partitions(self._h, _ptr(no, C.c_uint32), _ptr(eo, C.c_uint64)))
        return no, eo

    def csr_views(self):
        """(rowptr, col) as numpy views of the graph's host memory (no copy;
        valid while the graph is open)."""
        rp, cl = C.POINTER(C.c_uint64)(), C.POINTER(C.c_uint32)()
        check(lib.lt_graph_csr(self._h, C.byref(rp), C.byref(cl)))
        V, E = self.num_nodes, self.num_edges
        return (np.ctypeslib.as_array(rp, shape=(V + 1,)), np.ctypeslib.as_array(cl, shape=(E,)))

    def csr(self):
        """Copies of (rowptr, col)."""
        rp, cl = C.POINTER(C.c_uint64)(), C.POINTER(C.c_uint32)()
        check(lib.lt_graph_csr(self._h, C.byref(rp), C.byref(cl)))
        V, E = self.num_nodes, self.num_edges
        rowptr = np.ctypeslib.as_array(rp, shape=(V + 1,)).copy()
        col = np.ctypeslib.as_array(cl, shape=(E,)).copy() if E else np.zeros(0, np.uint32)
        return rowptr, col

    def write_bcsr(self, path: str):
        check(lib.lt_graph_write_bcsr(self._h, path.encode()))

    def write_part(self, bcsr_path: str):
        check(lib.lt_graph_write_part(self._h, bcsr_path.encode()))

    def close(self):
        if self._h:
            lib.lt_graph_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Pinned:
    def __init__(self, nbytes):
        self.ptr = C.c_void_p()
        check(lib.lt_host_alloc(nbytes, C.byref(self.ptr)))
        self.nbytes = nbytes

    def __del__(self):
        if self.ptr:
            lib.lt_host_free(self.ptr)
            self.ptr = C.c_void_p()


def checkpoint_info(path) -> dict:
    """Header of a checkpoint file written by Engine.checkpoint."""
    i = CheckpointInfo()
    check(lib.lt_checkpoint_read_info(os.fsencode(path), C.byref(i)))
    return {k: getattr(i, k) for k, _ in CheckpointInfo._fields_}


def pinned_empty(n: int, dtype=np.uint64) -> np.ndarray:
    """Uninitialised numpy array in page-locked host memory (lt_host_alloc),
    freed with the array: host buffers for results that come back from the
    device at the link's speed."""
    dt = np.dtype(dtype)
    owner = _Pinned(max(1, n * dt.itemsize))
    raw = (C.c_uint8 * owner.nbytes).from_address(owner.ptr.value)
    raw._lt_owner = owner
    return np.frombuffer(raw, dtype=dt, count=n)


class Server:
    """Continuous-batching PPR server on an out-of-core engine."""

    def __init__(self, engine: "Engine", max_active: int = 1024, table_slots: int = 1 << 26, prob: float = 0.15):
        self.engine = engine
        self._h = C.c_void_p()
        check(lib.lt_serve_open(engine._h, max_active, table_slots, prob, C.byref(self._h)))

    @staticmethod
    def now_ms() -> float:
        return lib.lt_serve_now_ms()

    def submit(self, source: int, walkers: int, seed: int, arrival_ms: float = 0.0) -> int:
        t = C.c_uint64()
        check(lib.lt_serve_submit(self._h, source, walkers, seed, arrival_ms, C.byref(t)))
        return t.value

    def step(self):
        c, a, p = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(lib.lt_serve_step(self._h, C.byref(c), C.byref(a), C.byref(p)))
        return c.value, a.value, p.value

    def finished(self, cap: int = 1 << 16):
        """Tickets finished since the last call."""
        buf = np.zeros(cap, np.uint64)
        n = lib.lt_serve_finished(self._h, _ptr(buf, C.c_uint64), cap)
        return buf[:n].tolist()

    def latency_ms(self, ticket: int):
        done, n, lat = C.c_int(), C.c_uint64(), C.c_double()
        check(lib.lt_serve_result(self._h, ticket, C.byref(done), C.byref(n), None, None, 0, C.byref(lat)))
        return lat.value if done.value else None

    def result(self, ticket: int):
        """None while running; else (dict vertex -> count, latency ms)."""
        done, n, lat = C.c_int(), C.c_uint64(), C.c_double()
        check(lib.lt_serve_result(self._h, ticket, C.byref(done), C.byref(n), None, None, 0, C.byref(lat)))
        if not done.value:
            return None
        v = np.zeros(max(1, n.value), np.uint32)
        c = np.zeros(max(1, n.value), np.uint32)
        check(lib.lt_serve_result(self._h, ticket, C.byref(done), C.byref(n), _ptr(v, C.c_uint32),
                                  _ptr(c, C.c_uint32), len(v), C.byref(lat)))
        k = n.value
        return dict(zip(v[:k].tolist(), c[:k].tolist())), lat.value

    def close(self):
        if self._h:
            lib.lt_serve_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    """One engine = the reference's LightTraffic<AppManager,App,Walker> object.

    partitions / batch are the reference's -p / -b.  resident_index=True
    (default) keeps the vertex index on the device when the graph is out of
    core, so loads and zero-copy reads move only edges; False uses the
    reference's slot layout.  Results are identical either way."""

    def __init__(self, graph: Graph, partitions: int = 0, batch: int = 0, seed: int = 0x5EED5EED,
                 sched: int = SCHED_PLAIN, pipeline: bool = True, zerocopy_threshold=None,
                 device: int = 0, ctas_per_sm: int = 0, resident_index: bool = True, zc_group_bytes: int = 0,
                 sweep_walkers: int = 0, load_factor: int = 0, bucket_items: int = 0, prefill: bool = True,
                 host_plan: bool = False, hot_tier: int = 0, split: bool = True):
        cfg = EngineCfg()
        lib.lt_engine_cfg_default(C.byref(cfg))
        cfg.device = device
        cfg.num_device_partitions = partitions
        cfg.num_device_walkers = batch
        cfg.seed = seed
        cfg.sched = sched
        cfg.pipeline = int(pipeline)
        if zerocopy_threshold is not None:
            cfg.zerocopy_threshold = zerocopy_threshold
        cfg.ctas_per_sm = ctas_per_sm
        cfg.resident_index = int(resident_index)
        cfg.zc_group_bytes = zc_group_bytes
        cfg.sweep_walkers = sweep_walkers
        cfg.load_factor = load_factor
        cfg.bucket_items = bucket_items
        cfg.no_prefill = 0 if prefill else 1
        cfg.host_plan = int(host_plan)
        cfg.hot_tier = hot_tier
        cfg.no_split = 0 if split else 1
        self.graph = graph
        self._h = C.c_void_p()
        check(lib.lt_engine_create(graph._h, C.byref(cfg), C.byref(self._h)))

    def ppr(self, source: int, walkers: int, prob: float = 0.15, out=None):
        V = self.graph.num_nodes
        counts = out if out is not None else np.zeros(V, dtype=np.uint64)
        check(lib.lt_run_ppr(self._h, source, walkers, prob, _ptr(counts, C.c_uint64)))
        return counts

    def pagerank(self, walkers: int, length: int = 10, runs: int = 1, alpha: float = 0.85,
                 start: int = START_UNIFORM, out=None):
        V = self.graph.num_nodes
        counts = out if out is not None else np.zeros(V, dtype=np.uint64)
        check(lib.lt_run_pagerank(self._h, walkers, length, runs, alpha, start,
                                  _ptr(counts, C.c_uint64)))
        return counts

    def walk(self, walkers: int, length: int = 10, run: int = 0, start: int = START_UNIFORM,
             paths: bool = False):
        ep = np.zeros(walkers, dtype=np.uint32)
        pa = np.zeros(walkers * (length + 1), dtype=np.uint32) if paths else None
        check(lib.lt_run_walk(self._h, walkers, length, run, start, _ptr(ep, C.c_uint32),
                              _ptr(pa, C.c_uint32)))
        return ep, pa

    def ppr_batch(self, sources, walkers, seeds=None, prob: float = 0.15, out=None):
        """Batched multi-source PPR: returns (offsets[n+1], vertices, counts);
        query q's pairs are [offsets[q], offsets[q+1]).  `out` = (offsets,
        vertices, counts) arrays to fill (u64[n+1], u32[>= sum(walkers)] x 2),
        e.g. from pinned_empty, instead of fresh ones."""
        src = np.ascontiguousarray(sources, dtype=np.uint32)
        w = np.ascontiguousarray(walkers, dtype=np.uint64)
        sd = None if seeds is None else np.ascontiguousarray(seeds, dtype=np.uint64)
        n = len(src)
        cap = int(w.sum())
        if out is None:
            off = np.zeros(n + 1, np.uint64)
            v = np.zeros(max(1, cap), np.uint32)
            c = np.zeros(max(1, cap), np.uint32)
        else:
            off, v, c = out
            if len(off) < n + 1 or len(v) < cap or len(c) < cap:
                raise ValueError("output arrays too small for the batch")
            cap = min(len(v), len(c))
        check(lib.lt_ppr_batch(self._h, n, _ptr(src, C.c_uint32), _ptr(w, C.c_uint64), _ptr(sd, C.c_uint64),
                               prob, _ptr(off, C.c_uint64), _ptr(v, C.c_uint32), _ptr(c, C.c_uint32), cap))
        tot = int(off[-1])
        return off, v[:tot], c[:tot]

    def autotune(self) -> dict:
        """Resident engine: tune the batch pipeline (block size, table load
        factor).  Out-of-core engine: tune the zero-copy group footprint,
        load threshold factor, step-kernel CTAs per SM and bucketing tile on
        cold-cache PPR trial runs.  Returns the chosen values."""
        check(lib.lt_engine_autotune(self._h))
        if self.graph.num_partitions > 0 and self._ooc():
            return self.ooc_tune()
        return self.batch_tune()

    def _ooc(self) -> bool:
        return bool(self.ooc_tune_raw().tuned)

    def ooc_tune_raw(self):
        t = OocTune()
        check(lib.lt_engine_ooc_tune(self._h, C.byref(t)))
        return t

    def ooc_tune(self) -> dict:
        t = self.ooc_tune_raw()
        return {k: getattr(t, k) for k, _ in t._fields_}

    def batch_tune(self) -> dict:
        t = BatchTune()
        check(lib.lt_engine_batch_tune(self._h, C.byref(t)))
        return {"block": t.block, "ctas_per_sm": t.ctas_per_sm, "load_shift": t.load_shift, "tuned": bool(t.tuned)}

    def checkpoint(self, path, every: int, stop: bool = False):
        """Write the state of every following run to `path` every `every`
        scheduler iterations; stop=True ends the run after the first one
        (LTError with status INTERRUPTED).  path=None disarms."""
        check(lib.lt_engine_checkpoint(self._h, None if path is None else os.fsencode(path), every, int(stop)))

    def resume(self, path):
        """Finish the run saved in `path`: counts (PPR / PageRank) or
        (endpoints, paths or None) (generic walk)."""
        info = checkpoint_info(path)
        V, W = info["num_nodes"], info["num_walkers"]
        counts = ep = pa = None
        if info["app"] != APP_WALK:
            counts = np.zeros(V, dtype=np.uint64)
        if info["has_endpoints"]:
            ep = np.zeros(W, dtype=np.uint32)
        if info["has_paths"]:
            pa = np.zeros(W * (info["length"] + 1), dtype=np.uint32)
        check(lib.lt_resume(self._h, os.fsencode(path), _ptr(counts, C.c_uint64), _ptr(ep, C.c_uint32),
                            _ptr(pa, C.c_uint32)))
        if info["app"] != APP_WALK:
            return counts
        return ep, pa

    def policy_stats(self) -> dict:
        s = PolicyStats()
        check(lib.lt_engine_policy_stats(self._h, C.byref(s)))
        return {"name": s.name.decode(), "train_steps": s.train_steps, "net_loss": s.net_loss,
                "baseline_loss": s.baseline_loss, "predictions": s.predictions, "net_used": s.net_used}

    def partition_stats(self) -> dict:
        """Per partition over the last out-of-core run: walkers entering it,
        those entering while it was cached, launches it was cached for."""
        P = self.graph.num_partitions
        v, cv, cl = (np.zeros(P, np.uint64) for _ in range(3))
        check(lib.lt_engine_partition_stats(self._h, _ptr(v, C.c_uint64), _ptr(cv, C.c_uint64),
                                            _ptr(cl, C.c_uint64)))
        return {"visits": v, "cached_visits": cv, "cached_launches": cl}

    def drop_cache(self):
        check(lib.lt_engine_drop_cache(self._h))

    def stats(self) -> dict:
        s = Stats()
        check(lib.lt_engine_stats(self._h, C.byref(s)))
        return s.as_dict()

    def close(self):
        if self._h:
            lib.lt_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
