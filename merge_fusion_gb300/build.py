"""Builds libkifi_gpu.so, the sm_103a depth-fusion library, in-tree.

    python -m merge_fusion_gb300.build [-v]

Each translation unit of csrc/ is compiled by nvcc in parallel for
``-gencode arch=compute_103a,code=sm_103a`` and linked into
merge_fusion_gb300/lib/libkifi_gpu.so (CUDA runtime linked statically).
Host code is built with -ffp-contract=off: the few float expressions that
run on the host (derived camera matrices) must round exactly like the
device code and the reference.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libkifi_gpu.so")

SOURCES = ["kifi_api.cu", "kifi_api_icp.cu", "kifi_api_pipeline.cu", "kifi_integrate.cu",
           "kifi_sort.cu", "kifi_sort_static.cu", "kifi_api_batch.cu", "kifi_api_io.cu", "kifi_api_learn.cu", "kifi_tc_gemm.cu", "kifi_proposer.cu", "kifi_autotune.cu", "kifi_mesh.cu", "kifi_icp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-prec-div=true",
    "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
    "-I", os.path.join(HERE, "..", "include"),
]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "kifi_gpu.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, extra_flags=()):
    os.makedirs(OBJDIR, exist_ok=True)
    nv = nvcc()
    procs, objs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        objs.append(o)
        if not force and not _stale(o, s):
            continue
        cmd = [nv] + NVCC_FLAGS + list(extra_flags) + ["-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((subprocess.Popen(cmd), src))
    failed = [src for p, src in procs if p.wait() != 0]
    if failed:
        raise RuntimeError("nvcc failed on " + ", ".join(failed))
    if procs or not os.path.exists(LIB):
        cmd = [nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fPIC"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
