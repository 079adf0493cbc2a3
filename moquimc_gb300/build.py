"""Build recipe for libmqigpu.so (the C ABI + sm_103a kernels) and the C++ host tools.

Everything is compiled in-tree with nvcc/g++ directly (no CMake): two CUDA translation units
compiled in parallel for ``sm_103a`` and linked into ``moquimc_gb300/_lib/libmqigpu.so``, plus the
``phantom_env`` host executable that mirrors moqui's example driver on top of the C ABI.
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
HOST = os.path.join(PKG, "host")
LIB_DIR = os.path.join(PKG, "_lib")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(LIB_DIR, "libmqigpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CUDA_SOURCES = ["mqi_kernels.cu", "mqi_capi.cu", "mqi_capi_dij.cu", "mqi_dij.cu", "mqi_noalloc.cu", "mqi_stat.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compile the CUDA sources for sm_103a and link libmqigpu.so; returns its path."""
    os.makedirs(LIB_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "mqi_gpu.h"))
    objs = []
    jobs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(LIB_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), *NVCC_FLAGS, *ARCH, f"-I{INCLUDE}", f"-I{CSRC}", "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(CUDA_SOURCES)) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc(), "-shared", *ARCH, *objs, "-o", LIB])
    if verbose:
        print(LIB)
    return LIB


def build_host_tools(force: bool = False) -> str:
    """Build the phantom_env and tps_env executables (C++ hosts over the C ABI)."""
    hdrs = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith((".hpp", ".h"))]
    jobs = []
    for name in ("phantom_env", "tps_env"):
        src = os.path.join(HOST, f"{name}_main.cpp")
        out = os.path.join(LIB_DIR, name)
        if os.path.exists(src) and (force or _stale(out, [src, LIB] + hdrs)):
            jobs.append(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{HOST}", src, "-o", out,
                         f"-L{LIB_DIR}", "-lmqigpu", f"-Wl,-rpath,{LIB_DIR}"])
    with cf.ThreadPoolExecutor(max_workers=max(len(jobs), 1)) as ex:
        list(ex.map(_run, jobs))
    return os.path.join(LIB_DIR, "phantom_env")


def build_all(force: bool = False) -> None:
    build_library(force=force)
    if os.path.exists(os.path.join(HOST, "phantom_env_main.cpp")):
        build_host_tools(force=force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
