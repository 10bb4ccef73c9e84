"""Builds liblsb.so (CUDA, sm_103a) and the C++ driver ``lsb_sort`` in-tree.

One ``nvcc -c`` per translation unit, run in parallel, then one link. Outputs
go to ``distributed-lsb_gb300/_build/`` (objects) and
``distributed-lsb_gb300/lib/`` (liblsb.so, lsb_sort); both are git-ignored.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # distributed-lsb_gb300/
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
HOST = os.path.join(PKG_ROOT, "host")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
LIB_PATH = os.path.join(LIB_DIR, "liblsb.so")
DRIVER_PATH = os.path.join(LIB_DIR, "lsb_sort")
SHARD_SIM_PATH = os.path.join(LIB_DIR, "lsb_shard_sim")
INCLUDE = os.path.join(REPO_ROOT, "include")

CUDA_SOURCES = ["lsb_onesweep.cu", "lsb_wide.cu", "lsb_task.cu", "lsb_segmented.cu", "lsb_server.cu", "lsb_capi.cu", "lsb_noalloc.cu", "lsb_host.cu", "lsb_sharded.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-I" + INCLUDE]


def lib_path() -> str:
    return os.environ.get("LSB_LIB", LIB_PATH)


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise FileNotFoundError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(_nvcc()))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA translation unit for sm_103a and link liblsb.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "lsb.h"))
    objs, jobs = [], []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if force or _stale(LIB_PATH, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB_PATH, *objs, "-lcudart"])
    drv_src = os.path.join(HOST, "lsb_main.cpp")
    drv_deps = [drv_src, os.path.join(HOST, "lsb_gb300.hpp"), os.path.join(INCLUDE, "lsb.h"), LIB_PATH]
    if os.path.exists(drv_src) and (force or _stale(DRIVER_PATH, drv_deps)):
        cuda = _cuda_home()
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, "-I" + HOST, "-I" + os.path.join(cuda, "include"),
              drv_src, "-o", DRIVER_PATH, "-L" + LIB_DIR, "-llsb", "-L" + os.path.join(cuda, "lib64"),
              "-lcudart", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(cuda, "lib64")])
    sim_src = os.path.join(HOST, "lsb_shard_sim.cpp")
    sim_deps = [sim_src, os.path.join(HOST, "lsb_gb300.hpp"), os.path.join(INCLUDE, "lsb.h"), LIB_PATH]
    if os.path.exists(sim_src) and (force or _stale(SHARD_SIM_PATH, sim_deps)):
        cuda = _cuda_home()
        _run(["g++", "-O2", "-std=c++17", "-pthread", "-I" + INCLUDE, "-I" + HOST,
              "-I" + os.path.join(cuda, "include"), sim_src, "-o", SHARD_SIM_PATH, "-L" + LIB_DIR, "-llsb",
              "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN",
              "-Wl,-rpath," + os.path.join(cuda, "lib64")])
    if verbose:
        print("built", LIB_PATH)
    return LIB_PATH
