"""Builds the MPM node layer into a real zeno core, for the host test.

The zeno core (the node-graph runtime that hosts the CuLagrange nodes) is
compiled straight from the sources of a zenustech/zeno checkout (given by
the ZENO_REFERENCE environment variable) with g++, no cmake: every
zeno/src/**/*.cpp into libzeno.so with the flags that checkout needs on
gcc 13 (-fpermissive for zeno/src/extra/GlobalComm.cpp, -mavx2 for
zeno/tpls/include/uuid_v4.h, an x86-64 host).  Then the node file
zeno_gb300/nodes/MPMNodes.cpp is compiled against zeno's own headers
(ZSMPM_WITH_ZENO) into a plugin library linked to libzeno.so and
libzsmpm.so, and tests/zeno_host/host.cpp into a host program that loads
both.  Outputs go to zeno_gb300/_build/zeno_host/ (not committed); the
library is rebuilt only when a source is newer than it."""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(ROOT, "zeno_gb300", "_build", "zeno_host")
CXX = os.environ.get("CXX", "g++")
FLAGS = ["-std=c++17", "-O1", "-fPIC", "-fpermissive", "-w", "-mavx2", "-fopenmp",
         "-DZENO_BENCHMARKING"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def zeno_includes(ref):
    z = os.path.join(ref, "zeno")
    return ["-I", os.path.join(z, "include"), "-I", os.path.join(z, "tpls", "include"),
            "-I", os.path.join(z, "tpls", "deprecated")]


def build(ref: str | None = None) -> dict:
    ref = ref or os.environ.get("ZENO_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "zeno", "src")):
        raise FileNotFoundError("a zeno checkout is needed (ZENO_REFERENCE)")
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(ref, "zeno", "src", "**", "*.cpp"), recursive=True))
    inc = zeno_includes(ref)
    objs, jobs = [], []
    for s in srcs:
        o = os.path.join(OUT, "obj", os.path.relpath(s, ref).replace(os.sep, "_") + ".o")
        objs.append(o)
        if _newer(o, [s]):
            jobs.append([CXX] + FLAGS + ["-DZENO_DLLEXPORT"] + inc + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(" ".join(cmd[-3:]) + "\n" + r.stderr[-3000:])

    with cf.ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        list(ex.map(run, jobs))
    libzeno = os.path.join(OUT, "libzeno.so")
    if jobs or _newer(libzeno, objs):
        run([CXX, "-shared", "-fopenmp", "-o", libzeno] + objs + ["-ldl", "-lpthread"])
    pkg = os.path.join(ROOT, "zeno_gb300")
    nodes_src = os.path.join(pkg, "nodes", "MPMNodes.cpp")
    plugin = os.path.join(OUT, "libzsmpm_zeno_nodes.so")
    if _newer(plugin, [nodes_src, libzeno, os.path.join(ROOT, "include", "zsmpm.h"),
                       os.path.join(pkg, "libzsmpm.so")]):
        run([CXX] + FLAGS + ["-DZSMPM_WITH_ZENO", "-shared"] + inc +
            ["-I", os.path.join(ROOT, "include"), "-o", plugin, nodes_src,
             "-L", OUT, "-lzeno", "-L", pkg, "-lzsmpm",
             "-Wl,-rpath," + OUT + ":" + pkg])
    host_src = os.path.join(HERE, "host.cpp")
    host = os.path.join(OUT, "zeno_host")
    if _newer(host, [host_src, plugin, libzeno]):
        run([CXX] + FLAGS + inc + ["-I", os.path.join(ROOT, "include"), "-o", host, host_src,
                                   "-L", OUT, "-lzeno", "-lzsmpm_zeno_nodes",
                                   "-Wl,--no-as-needed,-rpath," + OUT + ":" + pkg])
    return {"libzeno": libzeno, "plugin": plugin, "host": host}


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
