"""Build recipe of the engine: every translation unit compiled in parallel for
sm_103a, linked into openbcsim_gb300/libbcsim_gb300.so (in-tree, git-ignored).

    python -m openbcsim_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbcsim_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"

CU_SOURCES = ["project.cu", "conv.cu", "fftconv.cu", "noalloc.cu", "ingest.cu", "imaging.cu"]
CPP_SOURCES = ["engine.cpp", "host_dsp.cpp", "capi.cpp", "batch.cpp", "server.cpp", "imaging_host.cpp"]
HEADERS = ["kernels.hpp", "dfloat.cuh", "fixedpoint.cuh", "async_copy.cuh", "noise.cuh", "engine.hpp", "host_dsp.hpp", "imaging.hpp", "imaging_host.hpp"]

HOST_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-std=c++17", "-Wall", "-Wno-unused-function", "-pthread"]


def _newer(src_list, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_list)


def _compile(src: str, extra_dep):
    name = os.path.basename(src)
    obj = os.path.join(BUILD, name + ".o")
    if not _newer([src] + extra_dep, obj):
        return obj, None
    if src.endswith(".cu"):
        cmd = [NVCC, "-c", src, "-o", obj, "-O3", "-std=c++17", "-lineinfo", *ARCH,
               "-Xcompiler", ",".join(["-fPIC", "-ffp-contract=off"]), "-Xptxas", "-warn-spills",
               "-I" + CSRC]
    else:
        cmd = ["g++", "-c", src, "-o", obj, *HOST_FLAGS, "-I" + CSRC, "-I" + os.path.join(CUDA_HOME, "include")]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        return obj, "FAILED: " + " ".join(cmd) + "\n" + out.stdout + out.stderr
    return obj, (out.stdout + out.stderr).strip() or None


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "bcsim_gb300.h")]
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES]
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, deps), srcs))
    errors = [m for _, m in results if m and m.startswith("FAILED")]
    if errors:
        raise RuntimeError("\n".join(errors))
    if verbose:
        for _, m in results:
            if m:
                print(m)
    objs = [o for o, _ in results]
    if force or _newer(objs, LIB):
        cmd = [NVCC, "-shared", "-o", LIB, *objs, *ARCH, "-Xcompiler", "-fPIC", "-lpthread"]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("link failed: " + " ".join(cmd) + "\n" + out.stdout + out.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
