"""Build the CUDA shared library libfftperm.so (the C ABI of include/fftperm.h).

Every .cu file under csrc/ is compiled for sm_103a with nvcc, in parallel,
and linked into fft_method_test_gb300/_build/libfftperm.so.  The library is
built in the source tree so that the process that loads it is visibly using
this build.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libfftperm.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]
# Files whose arithmetic must round exactly like the reference's (no FMA
# contraction): the Brinkman stencils reproduce the reference field values.
NO_FMA = {"kernels_brinkman.cu"}


# rough relative compile cost per source, to order the parallel jobs
_COST = {"fft_ztma32.cu": 10, "fft_z32.cu": 9, "fft_y32.cu": 5, "fft_ztma64.cu": 4,
         "fft_x32.cu": 3, "fft_z64.cu": 3}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfftperm.so")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (when sources changed) and return the path of libfftperm.so."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "fftperm.h"))
    srcs = sources()
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            extra = ["-fmad=false"] if os.path.basename(s) in NO_FMA else []
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stderr)
        if verbose and r.stderr:
            print(r.stderr)
        return cmd

    if jobs:
        # the FP32 z passes take minutes (fully unrolled radix-16 code): start
        # them first so that they overlap everything else
        jobs.sort(key=lambda c: -_COST.get(os.path.basename(c[-3]), 1))
        workers = min(len(jobs), max(2, os.cpu_count() or 2), 16)
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
