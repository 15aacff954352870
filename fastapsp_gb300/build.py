"""In-tree build of the engine's shared library ``libfastapsp.so``.

Compiles every CUDA translation unit for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) and the host C++ units with the
system compiler, in parallel, then links one shared library next to this file.
Objects go to ``fastapsp_gb300/_build/``.  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libfastapsp.so"
EXAMPLE = PKG / "fap_single_node"
INCLUDE = PKG.parent / "include"

CUDA_SOURCES = ["minplus.cu", "sssp.cu", "bgraph.cu", "transform.cu", "query.cu", "adjoint.cu",
                "probe.cu", "engine.cu", "noalloc.cu"]
CXX_SOURCES = ["host_prep.cpp", "fap_graph.cpp", "fap_more_task.cpp"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.rglob("*.h"))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *_headers()])


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for name in CUDA_SOURCES:
        src = CSRC / name
        obj = BUILD / (name + ".o")
        objs.append(obj)
        if _stale(obj, src) or ptxas_info:
            cmd = [nvcc, *GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    cxx = os.environ.get("CXX", "g++")
    for name in CXX_SOURCES:
        src = CSRC / name
        obj = BUILD / (name + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append([cxx, "-O2", "-std=c++17", "-fPIC", "-I", str(INCLUDE), "-c", str(src),
                         "-o", str(obj)])
    outputs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outputs = list(ex.map(_run, jobs))
    if jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *GENCODE, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs),
              "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
    ex_src = CSRC / "single_node_example.cpp"
    if not EXAMPLE.exists() or EXAMPLE.stat().st_mtime < max(LIB.stat().st_mtime, ex_src.stat().st_mtime):
        _run([cxx, "-O2", "-std=c++17", "-I", str(INCLUDE), str(ex_src), "-o", str(EXAMPLE),
              "-L", str(PKG), "-lfastapsp", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        for o in outputs:
            if o.strip():
                print(o)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
