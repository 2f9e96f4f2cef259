"""In-tree build of the native libraries (no cmake, no pip install).

* ``zeno_gb300/libzsmpm.so``: the CUDA substep behind the C ABI of
  ``include/zsmpm.h``, compiled for sm_103a only, one object per .cu file,
  compiled in parallel.
* ``zeno_gb300/libzsmpm_nodes.so``: the C++ MPM node wrappers (zeno node
  API mirror in ``nodes/zeno_api.hpp``) over that ABI.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libzsmpm.so")
NODES_LIB = os.path.join(PKG, "libzsmpm_nodes.so")
NODES = os.path.join(PKG, "nodes")
NODE_SOURCES = ["MPMNodes.cpp", "nodes_capi.cpp"]

SOURCES = ["partition.cu", "transfer.cu", "flip.cu", "cloth.cu", "adjoint.cu", "io.cu", "output.cu", "api.cu", "noalloc.cu", "persistent.cu", "boundary_grid.cu"]
HEADERS = ["zsmpm_internal.cuh", "mpm_math.cuh", "binning.cuh", "tile_scatter.cuh", "cp_async.cuh",
           "adj_moments.cuh", "partition_stages.cuh", "transfer_stages.cuh",
           "colliders.cuh", "blocks.cuh", "cloth_grid.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "zsmpm.h")]
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _newer(o, [s] + hdrs) or ptxas_info:
            cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    if jobs or _newer(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        run(cmd)
    node_srcs = [os.path.join(NODES, f) for f in NODE_SOURCES]
    node_deps = node_srcs + [os.path.join(NODES, "zeno_api.hpp"),
                             os.path.join(ROOT, "include", "zsmpm.h"), LIB]
    if _newer(NODES_LIB, node_deps):
        cxx = os.environ.get("CXX", "g++")
        run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-Wno-unused-variable",
             "-I", os.path.join(ROOT, "include"), "-o", NODES_LIB] + node_srcs +
            ["-L", PKG, "-lzsmpm", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
