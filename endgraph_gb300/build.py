"""Builds libendgraph_gb300.so in-tree: one nvcc compile per translation unit (in parallel), sm_103a
only, then a shared-library link.  No cmake, no torch extension machinery."""
from __future__ import annotations

import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libendgraph_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills", f"-I{INCLUDE}"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return (_sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
            + glob.glob(os.path.join(INCLUDE, "*.cuh")))


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps() + [__file__])


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    srcs = _sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


TOOLKIT_SRC = os.path.join(HERE, "toolkits", "toolkits.cpp")
TOOLKIT_DIR = os.path.join(HERE, "toolkits", "bin")
TOOLKITS = ("pagerank", "bfs", "cc", "sssp")


def build_toolkits() -> str:
    """The C++ toolkit programs (host side over the C ABI via include/core/graph.hpp)."""
    lib = build()
    os.makedirs(TOOLKIT_DIR, exist_ok=True)
    exe = os.path.join(TOOLKIT_DIR, "eg_toolkit")
    deps = [TOOLKIT_SRC, lib] + glob.glob(os.path.join(INCLUDE, "core", "*.hpp"))
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(p) for p in deps):
        cmd = ["g++", "-std=c++14", "-O2", "-Wall", f"-I{INCLUDE}", TOOLKIT_SRC, "-o", exe + ".tmp", f"-L{HERE}",
               "-lendgraph_gb300", f"-Wl,-rpath,{HERE}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"toolkit build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(exe + ".tmp", exe)
    for t in TOOLKITS:
        link = os.path.join(TOOLKIT_DIR, t)
        if not os.path.lexists(link):
            os.symlink("eg_toolkit", link)
    # betweenness centrality: device operators on the engine API, compiled with nvcc
    bc_src = os.path.join(os.path.dirname(TOOLKIT_SRC), "bc.cu")
    bc_exe = os.path.join(TOOLKIT_DIR, "bc")
    bc_deps = [bc_src, lib] + glob.glob(os.path.join(INCLUDE, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "core", "*.hpp"))
    if not os.path.exists(bc_exe) or os.path.getmtime(bc_exe) < max(os.path.getmtime(p) for p in bc_deps):
        cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "--expt-relaxed-constexpr", f"-I{INCLUDE}", bc_src, "-o",
               bc_exe + ".tmp", f"-L{HERE}", "-lendgraph_gb300", "-Xlinker", f"-rpath={HERE}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"bc toolkit build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(bc_exe + ".tmp", bc_exe)
    return TOOLKIT_DIR


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    print(build_toolkits())
