"""bcsr / .part formats and the partitioner: the product and the oracle are
both checked against the reference's own EqualSizeStrategy outputs
(tests/golden/graphs/*.part, made by tests/golden/make_golden.py)."""
import json
import os
import shutil

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
