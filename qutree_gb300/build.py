"""Compile libqtgpu.so (sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel to an object file under
qutree_gb300/_build/, then linked into qutree_gb300/_build/libqtgpu.so
(git-ignored).  Nothing is installed into site-packages.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libqtgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["qt_api.cu", "qt_kernels.cu", "qt_plan.cpp", "qt_cdvr_plan.cpp",
           "qt_wsd.cu", "qt_umma.cu"]  # qt_plan_export.cpp: host-only lib
# per-file flags: the simultaneous diagonalisation follows a fixed operation
# order without fused multiply-adds (its CPU restatement does the same)
EXTRA = {"qt_wsd.cu": ["-fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "qtgpu.h"))
    return files


def _stale(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(f) > t for f in _deps())


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [NVCC, *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
           *EXTRA.get(src, []), "-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd[cmd.index("-c"):cmd.index("-c")] = ["-x", "cu"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not force and not _stale(LIB):
        return LIB
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


PLAN_LIB = os.path.join(BUILD, "libqtplan.so")


def build_plan_lib(force: bool = False) -> str:
    """Host-only planner library (g++, no CUDA calls) used by the CPU tests to
    inspect the sweep schedule without a GPU."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and not _stale(PLAN_LIB):
        return PLAN_LIB
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    tmp = PLAN_LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", cuda_inc, "-I", INCLUDE,
           os.path.join(CSRC, "qt_plan.cpp"), os.path.join(CSRC, "qt_cdvr_plan.cpp"),
           os.path.join(CSRC, "qt_plan_export.cpp"), "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for the planner library:\n{r.stderr}")
    os.replace(tmp, PLAN_LIB)
    return PLAN_LIB


if __name__ == "__main__":
    print(build_plan_lib(force="--force" in sys.argv))
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
