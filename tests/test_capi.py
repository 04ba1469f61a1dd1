"""The C-ABI library loads and exports every function include/*.h declares;
host-side error paths work without a GPU."""
import ctypes
import glob
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, gpu_available


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(lt_\w+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = _declared()
    assert "lt_run_ppr" in names and "lt_walk_device" in names and len(names) >= 20


@pytest.mark.parametrize("name", _declared())
def test_symbol_exported(lt, name):
    lib = ctypes.CDLL(lt.LIB_PATH)
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_strerror_and_version(lt):
    assert lt.lib.lt_strerror(0) == b"ok"
    assert b"sm_103a" in lt.lib.lt_version()


def test_engine_without_gpu_fails_loudly(lt):
    if gpu_available():
        pytest.skip("a GPU is visible")
    rp = np.array([0, 1, 2], np.uint64)
    col = np.array([1, 0], np.uint32)
    g = lt.Graph.from_csr(rp, col, 1 << 20)
    with pytest.raises(lt.LTError) as ei:
        lt.Engine(g)
    assert ei.value.status == 5                      # LT_ERR_CUDA, no silent fallback


def test_cli_requires_file(lt):
    exe = os.path.join(lt.BIN_DIR, "ppr")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "-f option must be given" in r.stderr
    r = subprocess.run([exe, "-f", "/nonexistent.bcsr", "-m"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr


def test_compact_rejects_counter_overflow(lt):
    """u32 counters: a call whose updates reach 2^32 is refused before any
    device work (W * length for PageRank, W for PPR)."""
    fake = ctypes.c_void_p(0x1000)
    rc = lt.lib.lt_walk_device_compact(1, 1, fake, fake, 10, 0, 1 << 29, 8, ctypes.c_float(0.85), 0, 1, fake,
                                       None, None, fake, None, None)
    assert rc == 1 and b"overflow u32" in lt.lib.lt_last_error()
    rc = lt.lib.lt_walk_device_compact(0, 0, fake, fake, 10, 0, 1 << 32, 0, ctypes.c_float(0.15), 0, 1, fake,
                                       None, None, fake, None, None)
    assert rc == 1 and b"overflow u32" in lt.lib.lt_last_error()


def test_checkpoint_info_rejects_bad_files(lt, tmp_path):
    info = lt.CheckpointInfo()
    assert lt.lib.lt_checkpoint_read_info(str(tmp_path / "missing").encode(), ctypes.byref(info)) == 2   # LT_ERR_IO
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(b"not a checkpoint at all")
    assert lt.lib.lt_checkpoint_read_info(str(bad).encode(), ctypes.byref(info)) == 3     # LT_ERR_FORMAT


def _ckpt_header(app=0, start=0, source=0, length=0, runs=1, run_base=0, run_index=0, flags=1, W=64,
                 prob=0.15, seed=1, V=100, E=400, P=2, part_hash=0, iteration=3):
    import struct
    return (b"LTCKPT01" + struct.pack("<I", 2)
            + struct.pack("<8I", app, start, source, length, runs, run_base, run_index, flags)
            + struct.pack("<Qf", W, prob) + struct.pack("<QIQI", seed, V, E, P)
            + struct.pack("<QQ", part_hash, iteration))


@pytest.mark.parametrize("bad", [
    dict(source=100),                      # source outside the graph
    dict(prob=0.0),                        # PPR stop probability outside (0, 1]
    dict(prob=float("nan")),
    dict(app=1, prob=1.5, length=10),      # PageRank probability outside [0, 1]
    dict(app=1, length=0, prob=0.85),      # no steps
    dict(app=2, length=0, flags=2),
    dict(app=2, length=5, flags=1),        # generic walks write no counts
    dict(flags=3),                         # PPR writes counts only
    dict(W=0), dict(V=0), dict(P=0), dict(P=101),
    dict(run_index=1, runs=1), dict(app=3), dict(start=3),
])
def test_checkpoint_header_rejects_corrupt_fields(lt, tmp_path, bad):
    """A checkpoint whose header describes a run the engine could not have
    started is refused with LT_ERR_FORMAT before anything reaches the device."""
    info = lt.CheckpointInfo()
    good = tmp_path / "good.ckpt"
    good.write_bytes(_ckpt_header())
    assert lt.lib.lt_checkpoint_read_info(str(good).encode(), ctypes.byref(info)) == 0
    assert info.num_walkers == 64 and info.num_nodes == 100 and info.iteration == 3
    path = tmp_path / "bad.ckpt"
    path.write_bytes(_ckpt_header(**bad))
    assert lt.lib.lt_checkpoint_read_info(str(path).encode(), ctypes.byref(info)) == 3   # LT_ERR_FORMAT


def test_checkpoint_header_rejects_old_version(lt, tmp_path):
    import struct
    path = tmp_path / "v1.ckpt"
    hdr = bytearray(_ckpt_header())
    hdr[8:12] = struct.pack("<I", 1)
    path.write_bytes(bytes(hdr))
    info = lt.CheckpointInfo()
    assert lt.lib.lt_checkpoint_read_info(str(path).encode(), ctypes.byref(info)) == 3


def test_engine_cfg_defaults(lt):
    """lt_engine_cfg_default: reference threshold, pipelining on, the vertex
    index resident on the device."""
    cfg = lt.EngineCfg()
    lt.lib.lt_engine_cfg_default(ctypes.byref(cfg))
    assert cfg.pipeline == 1 and cfg.resident_index == 1
    assert cfg.zerocopy_threshold == 2**64 - 1 and cfg.sched == 0


def test_cli_accepts_host_index(lt):
    exe = os.path.join(lt.BIN_DIR, "ppr")
    r = subprocess.run([exe, "-f", "/nonexistent.bcsr", "--host-index"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr


_MIRRORS = {"lt_graph_info": "GraphInfo", "lt_engine_cfg": "EngineCfg", "lt_stats": "Stats",
            "lt_checkpoint_info": "CheckpointInfo", "lt_batch_tune": "BatchTune", "lt_ooc_tune": "OocTune",
            "lt_policy_stats": "PolicyStats"}


@pytest.mark.parametrize("ctype", sorted(_MIRRORS))
def test_ctypes_mirror_matches_abi_layout(lt, ctype):
    """Every field of the package's ctypes mirror sits at the offset, with the
    size, the library reports for its C struct, and the structs are the same
    size: a field added to the header in one place but not the other, or in
    another order, fails here (no GPU needed)."""
    lib = ctypes.CDLL(lt.LIB_PATH)
    lib.lt_abi_field.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t),
                                 ctypes.POINTER(ctypes.c_size_t)]
    lib.lt_abi_field.restype = ctypes.c_int
    lib.lt_abi_sizeof.argtypes = [ctypes.c_char_p]
    lib.lt_abi_sizeof.restype = ctypes.c_size_t
    mirror = getattr(lt, _MIRRORS[ctype])
    assert lib.lt_abi_sizeof(ctype.encode()) == ctypes.sizeof(mirror)
    for name, _ in mirror._fields_:
        off, size = ctypes.c_size_t(), ctypes.c_size_t()
        assert lib.lt_abi_field(ctype.encode(), name.encode(), ctypes.byref(off), ctypes.byref(size)) == 0, name
        f = getattr(mirror, name)
        assert (f.offset, f.size) == (off.value, size.value), f"{ctype}.{name}"


def test_abi_layout_rejects_unknown_names(lt):
    lib = ctypes.CDLL(lt.LIB_PATH)
    lib.lt_abi_sizeof.restype = ctypes.c_size_t
    off, size = ctypes.c_size_t(), ctypes.c_size_t()
    assert lib.lt_abi_field(b"lt_engine_cfg", b"no_such_field", ctypes.byref(off), ctypes.byref(size)) == 1
    assert lib.lt_abi_sizeof(b"lt_no_such_struct") == 0
