"""Build recipe of the CUDA library (libeprem_gpu.so) for sm_103a.

Each translation unit is compiled by its own nvcc process (in parallel) and
the objects are linked into one shared library beside this file.  No cmake,
no torch extension machinery: the library has a plain C ABI
(include/eprem_gpu.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libeprem_gpu.so")
SOURCES = ["eprem_gpu.cu", "geometry.cu", "stream.cu", "node.cu", "mhd.cu", "peak.cu", "node32.cu", "mas.cu", "stream2.cu", "mlp.cu", "surrogate.cu", "ensemble.cu", "surrogate_host.cu", "shell.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]
# The background and node-motion kernels evaluate the reference's geometry
# (acos(z / |r|), sqrt(|r|^2 - z^2)) without fused multiply-adds, as the
# reference does: a contracted |r| can fall below |z| at the poles and turn
# those into NaN.  They are a negligible share of a step.
PER_FILE_FLAGS = {"mas.cu": ["-fmad=false"], "mhd.cu": ["-fmad=false"], "shell.cu": ["-fmad=false"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "eprem_gpu.h"))
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if ptxas_info or _stale(o, [s] + headers):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *PER_FILE_FLAGS.get(src, []), "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, res in zip(jobs, results):
        if verbose or ptxas_info or res.returncode:
            sys.stdout.write(res.stdout + res.stderr)
        if res.returncode:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}")
    if jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode:
            raise RuntimeError(res.stdout + res.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
