"""Builds the engine's native libraries in-tree.

  sop_gb300/libsopgpu.so   CUDA kernels + C ABI (include/sop_gpu.h), sm_103a
  sop_gb300/libsopgen.so   synthetic structure generator (host C++)

Translation units compile in parallel; one -gencode (compute_103a / sm_103a).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["engine.cu", "kernels_lists.cu", "kernels_step.cu", "energy_noalloc.cu"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_gpu(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    out = os.path.join(HERE, "libsopgpu.so")
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "sop_gpu.h"))
    flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
             "--expt-relaxed-constexpr", *ARCH, "-I", os.path.join(ROOT, "include")]
    if verbose:
        flags += ["-Xptxas", "-v"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _newer(o, [s, *headers]):
            jobs.append([nvcc(), *flags, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if force or jobs or not _newer(out, objs):
        _run([nvcc(), "-shared", *ARCH, "-o", out, *objs, "-lcudart"])
    return out


def build_gen(force: bool = False) -> str:
    out = os.path.join(HERE, "libsopgen.so")
    src = os.path.join(CSRC, "generator.cpp")
    if force or not _newer(out, [src]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", out, src])
    return out


def build_all(force: bool = False) -> None:
    build_gen(force)
    build_gpu(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built")
