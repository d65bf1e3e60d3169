"""Build libpike.so in-tree with nvcc for sm_103a (GB300).

All translation units compile in parallel.  Arithmetic flags are part of the
library's contract: IEEE division and square root, no FMA contraction on the
device (-fmad=false) or the host (-ffp-contract=off), denormals preserved.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libpike.so")
BUILD_DIR = os.path.join(HERE, "_build")

SOURCES = ["pk_api.cu", "pk_render.cu", "pk_scene.cu", "pk_util.cu", "pk_bvh.cu", "pk_cast.cu", "pk_env.cu", "pk_diff.cu", "pk_batch.cu", "pk_probe.cu", "pk_wide.cu", "pk_host_tables.cpp"]
HEADERS = ["pk_internal.cuh", "pk_math.cuh", "pk_render.h", "pk_util.h", "pk_bvh.h", "pk_host_tables.h", "pk_ctx.h",
           "pk_traverse.cuh", "pk_traverse_wide.cuh", "pk_wide.h", "pk_shade.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
           "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpike.so")


def _stale() -> bool:
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(HERE, "..", "include", "pike.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    if not force and not _stale():
        return OUT
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD_DIR, src.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        cmd = [cc, *ARCH, *NVFLAGS, *(extra or []), "-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [cc, "-x", "c++", *NVFLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(f"--- {src}\n{out}")
        if p.returncode:
            failed.append(src)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    tmp = OUT + ".tmp"
    link = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode:
        raise RuntimeError("link failed:\n" + r.stdout)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
