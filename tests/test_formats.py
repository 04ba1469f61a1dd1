"""bcsr / .part formats and the partitioner: the product and the oracle are
both checked against the reference's own EqualSizeStrategy outputs
(tests/golden/graphs/*.part, made by tests/golden/make_golden.py)."""
import hashlib
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

with open(os.path.join(GOLDEN, "partitions.json")) as _f:
    PARTS = json.load(_f)


def _graph(name):
    return oracle.read_bcsr(os.path.join(GOLDEN, "graphs", f"{name}.bcsr"))


@pytest.mark.parametrize("key", sorted(PARTS))
def test_oracle_partitioner_matches_reference(key):
    name, size = key.split(":")
    rp, _ = _graph(name)
    want = PARTS[key]
    if "error" in want:
        with pytest.raises(ValueError):
            oracle.partition(rp, int(size))
        return
    no, eo = oracle.partition(rp, int(size))
    assert no.tolist() == want["node_off"] and eo.tolist() == want["edge_off"]


@pytest.mark.parametrize("key", sorted(PARTS))
def test_product_partitioner_matches_reference(lt, key):
    name, size = key.split(":")
    rp, _ = _graph(name)
    want = PARTS[key]
    if "error" in want:
        with pytest.raises(lt.LTError) as ei:
            lt.partition_equal_size(rp, int(size))
        assert ei.value.status == 6          # LT_ERR_PARTITION
        return
    no, eo = lt.partition_equal_size(rp, int(size))
    assert no.tolist() == want["node_off"] and eo.tolist() == want["edge_off"]


@pytest.mark.parametrize("key", [k for k in sorted(PARTS) if "error" not in PARTS[k]])
def test_materialize_writes_reference_bytes(lt, tmp_path, key):
    """Graph.open(materialize=True) == Config -m: the .part bytes equal the
    reference's materialize() output byte for byte."""
    name, size = key.split(":")
    size = int(size)
    src = os.path.join(GOLDEN, "graphs", f"{name}.bcsr")
    dst = str(tmp_path / f"{name}.bcsr")
    shutil.copy(src, dst)
    rp, col = _graph(name)
    g = lt.Graph.from_csr(rp, col, size)
    g.write_part(dst)
    with open(dst + ".part", "rb") as a, open(os.path.join(GOLDEN, "graphs", f"{name}.{size}.part"), "rb") as b:
        assert a.read() == b.read()
    # and the oracle's reader agrees with the header
    P, psize, no, eo = oracle.read_part(dst + ".part")
    assert psize == size and P == len(PARTS[key]["node_off"]) - 1


def test_open_materialize_mb(lt, tmp_path):
    rp, col = _graph("rmat12")
    path = str(tmp_path / "g.bcsr")
    oracle.write_bcsr(path, rp, col)
    g = lt.Graph.open(path, materialize=True, part_mb=1)
    no, eo = g.partitions()
    wno, weo = oracle.partition(rp, 1 << 20)
    assert no.tolist() == wno.tolist() and eo.tolist() == weo.tolist()
    P, size, pno, peo = oracle.read_part(path + ".part")
    assert size == 1 << 20 and pno.tolist() == wno.tolist()
    # reopening without -m reads the .part back (MaterializedStrategy)
    g2 = lt.Graph.open(path, materialize=False)
    assert g2.partitions()[0].tolist() == wno.tolist()
    r2, c2 = g2.csr()
    assert (r2 == rp).all() and (c2 == col).all()


def test_bcsr_round_trip(lt, tmp_path):
    rp, col = oracle.rmat(11, 1 << 14, seed=9)
    g = lt.Graph.from_csr(rp, col, 1 << 20)
    path = str(tmp_path / "rt.bcsr")
    g.write_bcsr(path)
    r2, c2 = oracle.read_bcsr(path)
    assert (r2 == rp).all() and (c2 == col).all()
    with open(path, "rb") as f:
        head = f.read(12)
    assert int.from_bytes(head[:4], "little") == len(rp) - 1
    assert int.from_bytes(head[4:12], "little") == len(col)


def test_bad_files(lt, tmp_path):
    with pytest.raises(lt.LTError) as ei:
        lt.Graph.open(str(tmp_path / "missing.bcsr"), materialize=True)
    assert ei.value.status == 2              # LT_ERR_IO
    rp, col = _graph("gaps8")
    path = str(tmp_path / "t.bcsr")
    oracle.write_bcsr(path, rp, col)
    with open(path, "r+b") as f:             # truncate the col array
        f.truncate(os.path.getsize(path) - 4)
    with pytest.raises(lt.LTError) as ei:
        lt.Graph.open(path, materialize=True)
    assert ei.value.status == 3              # LT_ERR_FORMAT
    oracle.write_bcsr(path, rp, col)
    with pytest.raises(lt.LTError) as ei:    # no .part and no -m
        lt.Graph.open(path, materialize=False)
    assert ei.value.status == 2
    with open(path + ".part", "wb") as f:    # truncated .part
        f.write(b"\x02\x00")
    with pytest.raises(lt.LTError) as ei:
        lt.Graph.open(path, materialize=False)
    assert ei.value.status == 3
    bad = col.copy()
    bad[0] = len(rp) + 5                     # out-of-range vertex id
    oracle.write_bcsr(path, rp, bad)
    with pytest.raises(lt.LTError) as ei:
        lt.Graph.open(path, materialize=True)
    assert ei.value.status == 3


def test_oversize_vertex_is_an_error(lt, tmp_path):
    rp, col = _graph("hub10")
    path = str(tmp_path / "h.bcsr")
    oracle.write_bcsr(path, rp, col)
    with pytest.raises(lt.LTError) as ei:
        lt.Graph.open(path, materialize=True, part_mb=0)
    assert ei.value.status == 6
    assert "cannot fit" in str(ei.value)


# ------------------------------------------------------ edge-list converter

with open(os.path.join(GOLDEN, "edgelists.json")) as _f:
    EDGELISTS = json.load(_f)["bcsr"]


def _bcsr_bytes(rp, col):
    rp = np.ascontiguousarray(rp, np.uint64)
    col = np.ascontiguousarray(col, np.uint32)
    return (np.array([len(rp) - 1], np.uint32).tobytes() + np.array([len(col)], np.uint64).tobytes()
            + rp.tobytes() + col.tobytes())


@pytest.mark.parametrize("name", sorted(EDGELISTS))
def test_oracle_converter_matches_reference(name):
    """The oracle's restatement of converter_txt writes the bytes the
    reference's own tools/convert_from_txt.cc wrote."""
    rp, col = oracle.convert_edge_list(os.path.join(GOLDEN, "edgelists", name + ".el"))
    assert hashlib.sha256(_bcsr_bytes(rp, col)).hexdigest() == EDGELISTS[name]["sha256"]


@pytest.mark.parametrize("name", sorted(EDGELISTS))
def test_product_converter_matches_reference(lt, name, tmp_path):
    """lt_graph_from_edge_list + lt_graph_write_bcsr, and the converter_txt
    binary, write the reference converter's bytes."""
    src = os.path.join(GOLDEN, "edgelists", name + ".el")
    g = lt.Graph.from_edge_list(src)
    out = tmp_path / "g.bcsr"
    g.write_bcsr(str(out))
    assert hashlib.sha256(out.read_bytes()).hexdigest() == EDGELISTS[name]["sha256"]
    el = tmp_path / (name + ".el")
    el.write_bytes(open(src, "rb").read())
    r = subprocess.run([os.path.join(lt.BIN_DIR, "converter_txt"), str(el)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert f"nodes: {EDGELISTS[name]['V']} edges: {EDGELISTS[name]['E']}" in r.stdout
    assert hashlib.sha256((tmp_path / (name + ".bcsr")).read_bytes()).hexdigest() == EDGELISTS[name]["sha256"]


@pytest.mark.parametrize("flags", [1, 2, 4, 8, 3, 15])
@pytest.mark.parametrize("name", ["tiny", "sparse3000"])
def test_converter_options_match_oracle(lt, name, flags):
    """Each step the reference always takes (symmetrise, dedup, drop self
    loops, drop isolated ids) can be switched off; product and oracle agree."""
    src = os.path.join(GOLDEN, "edgelists", name + ".el")
    if flags & 8 and name == "sparse3000":
        flags &= ~8          # ids up to 10^6: keeping them all is fine but slow in the oracle's add.at
    g = lt.Graph.from_edge_list(src, directed=bool(flags & 1), keep_duplicates=bool(flags & 2),
                                keep_self_loops=bool(flags & 4), keep_isolated=bool(flags & 8))
    rp, col = g.csr()
    wrp, wcol = oracle.convert_edge_list(src, flags)
    assert (rp == wrp).all() and (col == wcol).all()


def test_converter_rejects_bad_input(lt, tmp_path):
    empty = tmp_path / "empty.el"
    empty.write_text("# nothing but comments\n\n")
    with pytest.raises(lt.LTError) as ei:
        lt.Graph.from_edge_list(str(empty))
    assert ei.value.status == 3
    with pytest.raises(lt.LTError) as ei:
        lt.Graph.from_edge_list(str(tmp_path / "missing.el"))
    assert ei.value.status == 2
    r = subprocess.run([os.path.join(lt.BIN_DIR, "converter_txt"), str(tmp_path / "x.txt")],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "not supported" in r.stderr
