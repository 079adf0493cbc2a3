"""Build recipe for the CPU oracles (test infrastructure, never part of the product path).

* ``oracle/_ref/bin/ref_oracle_{dbg,rel}``: the reference's own CPU code path, compiled with g++ from
  the staged, patched copy of its headers (``oracle/stage_ref.py``) and ``oracle/ref_driver.cpp``.
  ``dbg`` is built with ``-D__PHYSICS_DEBUG__`` (moqui's phantom example build), ``rel`` without.
  When the reference checkout is present the copy is re-staged first; elsewhere the copy that
  travelled with the repository is compiled as is.
* ``oracle/_ref/bin/ref_parser``: moqui's input-file reader (``mqi::file_parser``) from the staged
  copy of its header without the DICOM includes, driven by ``oracle/ref_parser.cpp``.
* ``oracle/_ref/bin/ref_gpu_{dbg,rel}``: the reference's own CUDA kernel for sm_103a, compiled with
  nvcc from the same staged copy and ``oracle/ref_gpu_driver.cu`` with the phantom example's flags
  (``--use_fast_math``, and ``-D__PHYSICS_DEBUG__`` for ``dbg``) plus ``-maxrregcount=128``: uncapped, ptxas gives the
  kernel 170 registers, and 170 x 512 threads exceeds the 65,536 registers of an SM, so the stock
  512-thread launch would be refused.  Built on demand (``build_reference_gpu``), not by
  ``build_all``: it takes about 20 s and only the reference-GPU timing and parity runs use it.
* ``oracle/_build/libmqi_oracle.so``: the C restatement ``oracle/mqi_oracle.c`` (FP32 stepping), and
  ``oracle/_build/libmqi_oracle64.so``: the same source with ``-DMQO_FP64``, the all-FP64 oracle.

All builds use ``-ffp-contract=off`` so the x86 and Arm builds round identically.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = os.path.join(HERE, "_ref", "src")
REF_BIN = os.path.join(HERE, "_ref", "bin")
BUILD = os.path.join(HERE, "_build")
# The reference checkout to stage from: MOQUI_REFERENCE_ROOT (the directory holding moqui/), set
# by the build entry point of the machine that has the checkout.  Without it the staged copy that
# travelled with the repository is compiled as is.
def reference_root() -> str:
    return os.environ.get("MOQUI_REFERENCE_ROOT", "")


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{res.stdout[-4000:]}\n{res.stderr[-4000:]}")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def ref_binary(debug: bool) -> str:
    return os.path.join(REF_BIN, "ref_oracle_dbg" if debug else "ref_oracle_rel")


def ref_parser_binary() -> str:
    return os.path.join(REF_BIN, "ref_parser")


def build_reference(force: bool = False) -> bool:
    """Stage (when possible) and compile the reference CPU oracle.  Returns False when no staged
    copy exists (the reference was never available to this checkout)."""
    root = reference_root()
    if root and os.path.isdir(os.path.join(root, "moqui")):
        sys.path.insert(0, HERE)
        import stage_ref  # noqa: E402

        if force or not os.path.isdir(os.path.join(REF_SRC, "moqui")):
            stage_ref.stage(root)
        elif not os.path.exists(os.path.join(REF_SRC, "moqui", "base", "mqi_file_handler_parser.hpp")):
            stage_ref.stage_parser(root)
    if not os.path.isdir(os.path.join(REF_SRC, "moqui")):
        return False
    os.makedirs(REF_BIN, exist_ok=True)
    drv = os.path.join(HERE, "ref_driver.cpp")
    jobs = []
    for debug in (True, False):
        out = ref_binary(debug)
        if force or _stale(out, [drv, os.path.join(HERE, "ref_beams.hpp"),
                                 os.path.join(REF_SRC, "moqui", "base", "mqi_p_ionization.hpp")]):
            cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w", f"-I{REF_SRC}", drv, "-o", out, "-lz"]
            if debug:
                cmd.insert(4, "-D__PHYSICS_DEBUG__")
            jobs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    parser_hdr = os.path.join(REF_SRC, "moqui", "base", "mqi_file_handler_parser.hpp")
    parser_src = os.path.join(HERE, "ref_parser.cpp")
    if os.path.exists(parser_hdr) and (force or _stale(ref_parser_binary(), [parser_src, parser_hdr])):
        jobs.append(subprocess.Popen(["g++", "-std=c++17", "-O1", "-w", f"-I{REF_SRC}", parser_src, "-o",
                                      ref_parser_binary()], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    for j in jobs:
        out, err = j.communicate()
        if j.returncode != 0:
            raise RuntimeError(f"reference oracle build failed:\n{err[-4000:]}")
    return True


def ref_gpu_binary(debug: bool = True) -> str:
    return os.path.join(REF_BIN, "ref_gpu_dbg" if debug else "ref_gpu_rel")


def build_reference_gpu(debug: bool = True, force: bool = False) -> str:
    """Compile the reference GPU driver; returns its path, or "" without a staged copy or nvcc."""
    root = reference_root()
    if root and os.path.isdir(os.path.join(root, "moqui")) and not os.path.isdir(os.path.join(REF_SRC, "moqui")):
        sys.path.insert(0, HERE)
        import stage_ref  # noqa: E402

        stage_ref.stage(root)
    if not os.path.isdir(os.path.join(REF_SRC, "moqui")):
        return ""
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if not os.path.exists(nvcc):
        return ""
    drv = os.path.join(HERE, "ref_gpu_driver.cu")
    out = ref_gpu_binary(debug)
    os.makedirs(REF_BIN, exist_ok=True)
    if force or _stale(out, [drv, os.path.join(HERE, "ref_beams.hpp"),
                             os.path.join(REF_SRC, "moqui", "base", "mqi_p_ionization.hpp")]):
        _run([nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "--use_fast_math"]
             + (["-D__PHYSICS_DEBUG__"] if debug else [])
             + ["-maxrregcount=128", "-w", f"-I{REF_SRC}", "-x", "cu", drv, "-o", out, "-lz"])
    return out


def oracle_lib(fp64: bool = False) -> str:
    return os.path.join(BUILD, "libmqi_oracle64.so" if fp64 else "libmqi_oracle.so")


def build_restatement(force: bool = False, fp64: bool = False) -> str:
    """The C restatement: FP32 stepping (moqui's float instantiation) or, with fp64, the all-FP64
    oracle (-DMQO_FP64)."""
    src = os.path.join(HERE, "mqi_oracle.c")
    hdr = os.path.join(HERE, "mqi_oracle.h")
    out = oracle_lib(fp64)
    if not os.path.exists(src):
        return ""
    os.makedirs(BUILD, exist_ok=True)
    if force or _stale(out, [src, hdr]):
        _run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-shared"] + (["-DMQO_FP64"] if fp64 else [])
             + [src, "-o", out, "-lm"])
    return out


def build_all(force: bool = False) -> None:
    build_restatement(force)
    build_restatement(force, fp64=True)
    build_reference(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
