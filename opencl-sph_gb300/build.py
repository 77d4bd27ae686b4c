"""Builds libsph_gb300.so in-tree (opencl-sph_gb300/lib/) for sm_103a.

    python opencl-sph_gb300/build.py [--verbose-ptxas]

CUDA sources are compiled by nvcc with -gencode arch=compute_103a,code=sm_103a
and no fast-math (the cell hash and neighbour tests depend on IEEE
rounding); host sources by g++.  Translation units compile in parallel and
the library links the CUDA runtime statically.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIB_DIR, "libsph_gb300.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCLUDES = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

CU_SOURCES = ["kernels.cu", "driver.cu", "batch.cu", "noalloc.cu"]
CPP_SOURCES = ["psdata.cpp", "store.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _compile(src, ptxas_verbose):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-DNDEBUG",
                               "--expt-relaxed-constexpr"] + INCLUDES + ["-c", path, "-o", obj]
        if ptxas_verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-DNDEBUG", "-I" + os.path.join(CUDA_HOME, "include")] \
            + INCLUDES + ["-c", path, "-o", obj]
    return obj, _run(cmd)


def sources():
    return [s for s in CU_SOURCES + CPP_SOURCES if os.path.exists(os.path.join(CSRC, s))]


def build(ptxas_verbose=False, quiet=True):
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_verbose), srcs))
    objs = [o for o, _ in results]
    log = "".join(out for _, out in results)
    tmp = LIB + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    if not quiet or ptxas_verbose:
        sys.stdout.write(log)
    return LIB


if __name__ == "__main__":
    print(build(ptxas_verbose="--verbose-ptxas" in sys.argv, quiet=False))
