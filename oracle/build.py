"""Build recipe for the two CPU oracles (test infrastructure, never the product).

1. ``oracle/_ref/libcacgref.so`` -- the reference sclc/cacg solver sources
   (src/bcbcgKernel.c, src/cbcgKernel.c, src/bcgKernel.c, src/common.c,
   src/BLAS3.c, src/DLSsolvers.c, src/MatrixOperations.c, src/matrixType.c,
   src/readMTX.c and the Matrix Market library it vendors, src/mmio.c) compiled with
   gcc against the project-written MPI shim (oracle/mpi_shim) and the harness
   (oracle/ref_harness.c).  The sources are staged into ``oracle/_ref/src``
   (git-ignored) because three constants must become variables:
   ``#define MAXITER 100`` (src/bcbcgKernel.c:3),
   ``#define CBCG_MAXITER 1000`` (src/cbcgKernel.c:2) and
   ``#define BCG_MAXITER 1000`` (src/bcgKernel.c:2) are rewritten to read
   ``cacg_ref_maxiter``.  No other line changes.  Missing prototypes in the
   reference (e.g. get_same_shape_denseType used by src/bcbcgKernel.c:57
   without matrixType.h) are supplied with ``-include``.  Staging happens
   only where the reference tree exists; elsewhere the staged copy that
   travelled with the repository is compiled.
2. ``oracle/_build/liboracle.so`` -- the project's own C restatement
   (oracle/cacg_oracle.c) plus the shared generators.

Both are compiled with ``-ffp-contract=off`` so that x86-64 and aarch64 produce
bit-identical results (no fused multiply-add contraction).
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REF_SRC_DEFAULT = "/root/reference/src"
REF_OUT = os.path.join(HERE, "_ref")
REF_STAGE = os.path.join(REF_OUT, "src")
PORT_OUT = os.path.join(HERE, "_build")

REF_C_FILES = [
    "bcbcgKernel.c",
    "cbcgKernel.c",
    "common.c",
    "BLAS3.c",
    "DLSsolvers.c",
    "MatrixOperations.c",
    "matrixType.c",
    "readMTX.c",
    "mmio.c",
    "bcgKernel.c",
]
CFLAGS = ["-O2", "-fPIC", "-std=gnu99", "-ffp-contract=off", "-w"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def stage_reference(ref_src: str = REF_SRC_DEFAULT) -> bool:
    """Copy the reference sources into oracle/_ref/src (MAXITER -> variable)."""
    if not os.path.isdir(ref_src):
        return False
    os.makedirs(REF_STAGE, exist_ok=True)
    for name in sorted(os.listdir(ref_src)):
        if not (name.endswith(".h") or name in REF_C_FILES):
            continue
        with open(os.path.join(ref_src, name), "r", errors="replace") as f:
            text = f.read()
        if name == "bcbcgKernel.c":
            text, k = re.subn(r"^#define MAXITER 100\b", "#define MAXITER cacg_ref_maxiter",
                              text, flags=re.M)
            assert k == 1, "MAXITER line not found"
        if name == "cbcgKernel.c":
            text, k = re.subn(r"^#define CBCG_MAXITER 1000\b",
                              "#define CBCG_MAXITER cacg_ref_maxiter", text, flags=re.M)
            assert k == 1, "CBCG_MAXITER line not found"
        if name == "bcgKernel.c":
            text, k = re.subn(r"^#define BCG_MAXITER 1000\b",
                              "#define BCG_MAXITER cacg_ref_maxiter", text, flags=re.M)
            assert k == 1, "BCG_MAXITER line not found"
        dst = os.path.join(REF_STAGE, name)
        if os.path.exists(dst):
            with open(dst) as f:
                if f.read() == text:
                    continue
        with open(dst, "w") as f:
            f.write(text)
    with open(os.path.join(REF_STAGE, "cacg_ref_hooks.h"), "w") as f:
        f.write("/* generated by oracle/build.py */\nextern long cacg_ref_maxiter;\n")
    return True


def build_reference(ref_src: str = REF_SRC_DEFAULT, force: bool = False) -> str | None:
    """Build oracle/_ref/libcacgref.so; returns its path or None if unavailable."""
    stage_reference(ref_src)
    if not os.path.isfile(os.path.join(REF_STAGE, "bcbcgKernel.c")):
        return None
    lib = os.path.join(REF_OUT, "libcacgref.so")
    objdir = os.path.join(REF_OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "mpi_shim"), "-I", REF_STAGE]
    forced = ["-include", "cacg_ref_hooks.h", "-include", "matrixType.h",
              "-include", "MatrixOperations.h", "-include", "BLAS3.h",
              "-include", "common.h", "-include", "DLSsolvers.h"]
    jobs = []
    for name in REF_C_FILES:
        extra = []
        if name == "common.c":
            extra = ["-Dgerschgorin_v1=gerschgorin_v1_ref"]
        if name in ("bcbcgKernel.c", "cbcgKernel.c", "bcgKernel.c"):
            extra = ["-Dnorm2square_dist_denseMat_col_n=cacg_ref_norm_hook"]
        src = os.path.join(REF_STAGE, name)
        obj = os.path.join(objdir, name[:-2] + ".o")
        jobs.append(["gcc", *CFLAGS, *inc, *forced, *extra, "-c", src, "-o", obj])
    for src in (os.path.join(HERE, "ref_harness.c"),
                os.path.join(HERE, "mpi_shim", "mpi_threads.c")):
        obj = os.path.join(objdir, os.path.basename(src)[:-2] + ".o")
        jobs.append(["gcc", *CFLAGS, *inc, "-c", src, "-o", obj])
    objs = [j[-1] for j in jobs]
    if not force and os.path.exists(lib):
        newest = max(os.path.getmtime(j[-3]) for j in jobs)
        newest = max(newest, os.path.getmtime(__file__))
        if os.path.getmtime(lib) > newest:
            return lib
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    _run(["gcc", "-shared", "-o", lib, *objs, "-lm", "-lpthread"])
    return lib


def build_port(force: bool = False) -> str:
    """Build oracle/_build/liboracle.so (restatement + shared generators)."""
    os.makedirs(PORT_OUT, exist_ok=True)
    lib = os.path.join(PORT_OUT, "liboracle.so")
    srcs = [os.path.join(HERE, "cacg_oracle.c"),
            os.path.join(REPO, "cacg_gb300", "csrc", "cacg_gen.c")]
    if not force and os.path.exists(lib):
        if os.path.getmtime(lib) > max(os.path.getmtime(s) for s in srcs + [__file__]):
            return lib
    _run(["gcc", *CFLAGS, "-I", os.path.join(REPO, "include"), "-shared", "-o", lib,
          *srcs, "-lm"])
    return lib


def build_all(force: bool = False) -> dict:
    return {"reference": build_reference(force=force), "port": build_port(force=force)}


if __name__ == "__main__":
    print(build_all(force=True))
