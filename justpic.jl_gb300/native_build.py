"""Build libjustpic_gb300.so (the C-ABI library) with nvcc for sm_103a.

Each translation unit compiles in its own nvcc process (in parallel), then one
link step produces the shared library next to this file, in ``_build/``.
``-fmad=false`` keeps every product and sum separately rounded; the kernels
spell out each fused multiply-add with fma() where the reference uses muladd.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libjustpic_gb300.so")

SOURCES = ["jp_capi.cu", "jp_particles.cu", "jp_move.cu", "jp_f32.cu", "jp_adjoint.cu", "jp_transfer.cu",
           "jp_layout.cu"]
HEADERS = ["jp_internal.cuh", "jp_move_core.cuh", "jp_f32_core.cuh", "jp_weight.cuh"]
PUBLIC_HEADERS = ["justpic_gb300.h", "justpic_gb300_rng.h"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libjustpic_gb300")
    return path


def _deps_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    files += [os.path.join(REPO, "include", f) for f in PUBLIC_HEADERS]
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def is_stale() -> bool:
    return not os.path.exists(LIB) or os.path.getmtime(LIB) < _deps_mtime()


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    if not force and not is_stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
