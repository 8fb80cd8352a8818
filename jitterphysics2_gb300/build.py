"""Builds the CUDA library (libjitter_gpu.so, sm_103a) in-tree.

Each translation unit is compiled in parallel with nvcc, then linked with the CUDA
runtime statically so the library loads without a driver (the C-ABI symbol check runs
on machines with no GPU).  FP32 arithmetic is compiled unfused (-fmad=false) with IEEE
division and square root, the way .NET evaluates the reference's float code.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libjitter_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["jg_api.cu", "jg_broadphase.cu", "jg_narrowphase.cu", "jg_contacts.cu", "jg_sched.cu", "jg_solver.cu",
              "jg_mlp.cu", "jg_islands.cu"]
CPP_SOURCES = ["jg_host.cpp"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-Xcompiler", "-fPIC", "-Xptxas", "-v"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(HERE, "..", "include", "jitter_gpu.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if not _stale(obj, [path] + _headers()):
        return obj, ""
    if src.endswith(".cu"):
        cmd = [_nvcc()] + ARCH + NVCC_FLAGS + ["-c", path, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = CU_SOURCES + CPP_SOURCES
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(_compile, srcs))
    objs = [o for o, _ in results]
    log = "".join(e for _, e in results)
    if log:
        with open(os.path.join(BUILD, "ptxas.log"), "a") as f:
            f.write(log)
    if verbose and log:
        sys.stderr.write(log)
    if _stale(LIB, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "--cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
