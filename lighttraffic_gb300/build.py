"""In-tree build of the native library and the CLI binaries.

    python lighttraffic_gb300/build.py

Produces
  lighttraffic_gb300/liblighttraffic.so   (C ABI of include/lighttraffic.h)
  lighttraffic_gb300/bin/{ppr,pagerank,genericwalk,converter_txt}

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a); translation units are compiled in
parallel and relinked only when a source or header is newer than the output.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
APPS = os.path.join(PKG, "apps")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblighttraffic.so")
BIN = os.path.join(PKG, "bin")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-fopenmp,-Wall",
              "-Xptxas", "-O3", f"-I{INCLUDE}"]
APP_NAMES = {"ppr": 0, "pagerank": 1, "genericwalk": 2}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build lighttraffic_gb300")
    return p


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    nv = nvcc()
    headers = _headers()
    srcs = _sources()
    objs, todo = [], []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s) + ".o")
        objs.append(o)
        if _newer(o, [s, *headers, __file__]):
            todo.append([nv, *NVCC_FLAGS, "-c", s, "-o", o])
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for r in ex.map(_run, todo):
            if verbose and r.stderr:
                sys.stderr.write(r.stderr)
    if todo or _newer(LIB, objs):
        _run([nv, "-shared", *ARCH, "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"])
    cli = os.path.join(APPS, "lt_cli.cpp")
    cmds = []
    for name, app in APP_NAMES.items():
        out = os.path.join(BIN, name)
        if _newer(out, [cli, LIB, *headers]):
            cmds.append(["g++", "-std=c++17", "-O2", f"-DLT_CLI_APP={app}", f"-I{INCLUDE}", cli, "-o", out,
                         f"-L{PKG}", "-llighttraffic", "-Wl,-rpath,$ORIGIN/.."])
    conv = os.path.join(APPS, "lt_convert.cpp")
    out = os.path.join(BIN, "converter_txt")
    if _newer(out, [conv, LIB, *headers]):
        cmds.append(["g++", "-std=c++17", "-O2", f"-I{INCLUDE}", conv, "-o", out, f"-L{PKG}", "-llighttraffic",
                     "-Wl,-rpath,$ORIGIN/.."])
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(_run, cmds))
    return LIB


def ptxas_report() -> str:
    """Register / spill / shared-memory usage of every kernel (-Xptxas -v)."""
    nv = nvcc()
    out = []
    for s in _sources():
        if s.endswith(".cu"):
            r = subprocess.run([nv, *NVCC_FLAGS, "-Xptxas", "-v", "-c", s, "-o", os.devnull],
                               capture_output=True, text=True)
            out.append(r.stderr)
    return "\n".join(out)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--ptxas":
        print(ptxas_report())
    else:
        print(build(verbose=True))
