"""Build the GB300 solver library ``_build/liblesgpu.so`` (sm_103a) in-tree.

Each translation unit compiles in parallel; the library links the CUDA runtime
statically, so it loads without torch.  Flags that matter for parity:
``--fmad=false`` (no multiply-add contraction, like gfortran -O on the reference),
IEEE division and square root (nvcc's defaults without --use_fast_math), and
``-ffp-contract=off`` for the host set-up code.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblesgpu.so")
MAIN = os.path.join(OUT, "les_main")  # the main.f95 time loop on the library (host/les_main.cpp)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
    "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-warn-spills",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall"]

CU_SOURCES = ["les_kernels.cu", "les_fused.cu", "les_sor.cu", "les_sor16.cu", "les_sor2.cu", "les_sor_batch.cu", "les_step.cu", "les_api.cu", "les_noalloc.cu", "les_batch.cu", "les_tune.cu", "les_aveflow.cu"]
CXX_SOURCES = ["setup.cpp", "les_io.cpp"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the solver library needs the CUDA toolkit")
    return cand


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_nvcc: list[str] | None = None) -> str:
    """Compile every source for sm_103a and link liblesgpu.so; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "les_gpu.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers + [__file__]):
            jobs.append([nvcc] + NVCC_FLAGS + (extra_nvcc or []) + ["-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers + [__file__]):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        logs.append(_run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]))
        os.replace(tmp, LIB)
    src_main = os.path.join(HERE, "host", "les_main.cpp")
    if force or _stale(MAIN, [src_main, LIB, os.path.join(HERE, "..", "include", "les_gpu.h")]):
        tmp = MAIN + ".tmp"
        logs.append(_run(["g++"] + CXX_FLAGS + ["-I", os.path.join(HERE, "..", "include"), src_main, "-o", tmp,
                          "-L", OUT, "-llesgpu", "-Wl,-rpath,$ORIGIN"]))
        os.replace(tmp, MAIN)
    if verbose:
        for lg in logs:
            if lg.strip():
                print(lg)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
