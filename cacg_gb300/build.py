"""In-tree build of libcacg.so for GB300 (sm_103a).

Every CUDA translation unit is compiled by nvcc with exactly one
``-gencode arch=compute_103a,code=sm_103a`` (no PTX for other targets, no
multi-arch fatbin), in parallel; the generator C file is compiled with
``-ffp-contract=off`` so the synthetic inputs are bit-identical across hosts.
The CUDA runtime is linked statically, so the library has no dependency on
a libcudart on the library path.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcacg.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
if not os.path.exists(NVCC):
    NVCC = "nvcc"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "--expt-relaxed-constexpr",
                   "-I", os.path.join(REPO, "include"), "-I", CSRC]
C_FLAGS = ["-O2", "-fPIC", "-std=gnu99", "-ffp-contract=off",
           "-I", os.path.join(REPO, "include")]

CU_SOURCES = ["k_spmm.cu", "k_gram.cu", "k_gram_tc.cu", "k_gram_tc5.cu", "k_tsm_tc5.cu", "k_dia.cu", "k_dia_ring.cu", "k_dia_wide.cu", "k_update.cu", "k_xr16.cu", "k_lu.cu", "solver.cu", "bcg.cu", "server.cu", "k_batch.cu", "k_tsqr.cu"]
C_SOURCES = ["cacg_gen.c", "cacg_io.c"]
HEADERS = ["cacg_internal.cuh", "cacg_solver.h", "tc5_util.cuh", "ff_util.cuh", "tma_util.cuh",
           "batch.h"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    common_deps = [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(REPO, "include", "cacg.h"), os.path.join(REPO, "include", "cacg_ref_types.h"),
        os.path.abspath(__file__)]
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + common_deps):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([NVCC, *CU_FLAGS, *extra, "-c", s, "-o", o])
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".c", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + common_deps):
            jobs.append(["gcc", *C_FLAGS, "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            for r in ex.map(_run, jobs):
                if verbose or ptxas_info:
                    sys.stderr.write(r.stderr)
    if jobs or not os.path.exists(LIB) or _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
