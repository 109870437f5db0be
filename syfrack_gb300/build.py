"""In-tree build of libsyfrack_gpu.so for sm_103a (nvcc; no cmake).

Each translation unit compiles in parallel, then one link step. Rebuilds only
when a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsyfrack_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = ["sf_kernels.cu", "sf_escape.cu", "sf_trace_box.cu", "sf_trace_bulb.cu", "sf_trace_menger.cu", "sf_trace_any.cu",
         "sf_batch.cu", "sf_noalloc.cu", "sf_preview.cu", "sf_host.cpp",
         "sf_batch_host.cpp", "sf_serve.cpp", "sf_export.cpp", "sf_preview.cpp", "sf_environment.cpp"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsyfrack_gpu.so")


def _inputs():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "syfrack_gpu.h"))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _inputs())


def _compile(unit: str) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit + ".o")
    # host code rounds every operation (no contraction): the host-derived constants
    # and instance hierarchies are then the same on x86-64 and aarch64 hosts
    flags = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-lineinfo"]
    if unit.endswith(".cu"):
        flags += ARCH
    cmd = [nvcc(), *flags, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(_compile, UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
