"""The drop-in binaries: reference flags, stdout lines, counts dump."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bcsr(tmp_path_factory):
    rp, col = oracle.rmat(16, 1 << 20, seed=21)
    d = tmp_path_factory.mktemp("g")
    path = str(d / "g.bcsr")
    oracle.write_bcsr(path, rp, col)
    return path, rp, col


def _run(lt, name, *args):
    r = subprocess.run([os.path.join(lt.BIN_DIR, name), *args], capture_output=True, text=True, timeout=300)
    return r


def test_ppr_binary(lt, require_gpu, bcsr, tmp_path):
    path, rp, col = bcsr
    V = len(rp) - 1
    out = str(tmp_path / "counts.u64")
    r = _run(lt, "ppr", "-f", path, "-m", "-s", "1", "--seed", "9", "--counts-out", out)
    assert r.returncode == 0, r.stderr
    assert f"num nodes: {V}, num edges: {len(col)}, num walkers: {2 * V}" in r.stdout
    assert "number of partitons:" in r.stdout               # the reference's spelling
    assert "result correct" in r.stdout
    # benchmark/figure9/run.sh greps six "<number with a dot> ms" values
    assert len(re.findall(r"[0-9]+\.[0-9]+ ms", r.stdout)) == 6
    got = np.fromfile(out, dtype=np.uint64)
    want, _, _ = oracle.ppr(rp, col, 0, 2 * V, prob=0.15, seed=9)
    assert (got == want).all()
    # second run reads the materialised .part, out of core with 2 cached partitions
    r = _run(lt, "ppr", "-f", path, "-p", "2", "-w", "50000", "--source", "5", "--prob", "0.2", "--seed", "9",
             "--counts-out", out)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, dtype=np.uint64)
    want, _, _ = oracle.ppr(rp, col, 5, 50000, prob=0.2, seed=9)
    assert (got == want).all()


def test_pagerank_and_walk_binaries(lt, require_gpu, bcsr, tmp_path):
    path, rp, col = bcsr
    V = len(rp) - 1
    r = _run(lt, "pagerank", "-f", path, "-m", "-s", "1", "-l", "8", "--runs", "2", "--seed", "3",
             "--counts-out", str(tmp_path / "c"))
    assert r.returncode == 0, r.stderr
    assert "result correct" in r.stdout and "node 0, degree" in r.stdout
    got = np.fromfile(str(tmp_path / "c"), dtype=np.uint64)
    want, _ = oracle.pagerank(rp, col, 2 * V, length=8, runs=2, seed=3, start_mode=oracle.START_UNIFORM)
    assert (got == want).all()
    r = _run(lt, "genericwalk", "-f", path, "-p", "3", "-l", "5", "-w", "1000", "--seed", "4", "--start", "pervertex",
             "--paths-out", str(tmp_path / "p"))
    assert r.returncode == 0, r.stderr
    paths = np.fromfile(str(tmp_path / "p"), dtype=np.uint32)
    _, want, _ = oracle.generic_walk(rp, col, 1000, length=5, start_mode=oracle.START_PER_VERTEX, seed=4, paths=True)
    assert (paths == want).all()


def test_ppr_binary_checkpoint_and_resume(lt, require_gpu, bcsr, tmp_path):
    """--checkpoint ... --stop-at-checkpoint ends the run (exit 4); --resume on
    another cache size finishes it with the counts of an uninterrupted run."""
    path, rp, col = bcsr
    ck = str(tmp_path / "run.ckpt")
    out = str(tmp_path / "counts.u64")
    r = _run(lt, "ppr", "-f", path, "-m", "-s", "1", "-p", "3", "-w", "200000", "--seed", "9",
             "--checkpoint", ck, "--checkpoint-every", "4", "--stop-at-checkpoint")
    assert r.returncode == 4, r.stdout + r.stderr
    assert "interrupted at checkpoint" in r.stdout and os.path.exists(ck)
    r = _run(lt, "ppr", "-f", path, "-p", "2", "--resume", ck, "--counts-out", out)
    assert r.returncode == 0, r.stderr
    assert "result correct" in r.stdout
    want, _, _ = oracle.ppr(rp, col, 0, 200000, prob=0.15, seed=9)
    assert (np.fromfile(out, dtype=np.uint64) == want).all()
