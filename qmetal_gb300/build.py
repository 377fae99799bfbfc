"""Build the native library in-tree.

Compiles the CUDA kernels for sm_103a and the C++ host, and links
``qmetal_gb300/libqmetal.so`` (the C ABI of include/qmetal/qmetal.h plus the
thin kernel layer of include/qmetal/qmetal_kernels.h). Translation units are
compiled in parallel and skipped when their object is newer than every input.

    python qmetal_gb300/build.py
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
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libqmetal.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
             "-I" + os.path.join(CUDA_HOME, "include")]

CU_SOURCES = ["k_gates.cu", "k_diag.cu", "k_reduce.cu", "k_sample.cu", "k_adjoint.cu",
              "k_noalloc.cu", "k_perm.cu", "k_adjoint_tiles.cu", "k_adjoint_uniform.cu",
              "k_xfield.cu"]
CXX_SOURCES = ["circuit.cpp", "plan.cpp", "schedule.cpp", "simulator.cpp", "batch.cpp", "capi.cpp"]
HEADERS = ["kcommon.cuh", "kquad.cuh", "kreduce.cuh", "kadjoint.cuh", "kadjoint_ops.cuh",
           "circuit.hpp", "schedule.hpp",
           "simulator.hpp", "batch.hpp"]
PUBLIC = [os.path.join(ROOT, "include", "qmetal", "qmetal.h"),
          os.path.join(ROOT, "include", "qmetal", "qmetal_kernels.h")]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _compile(src: str) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    deps = [path] + [os.path.join(CSRC, h) for h in HEADERS] + PUBLIC
    if _newer(obj, deps):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC] + NVCC_FLAGS + ["-c", path, "-o", obj]
    else:
        cmd = [CXX] + CXX_FLAGS + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    """Compile and link; returns the library path. Raises on any failure."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(OBJ, exist_ok=True)
    sources = CU_SOURCES + CXX_SOURCES
    with cf.ThreadPoolExecutor(max_workers=min(len(sources), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, sources))
    if not _newer(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static",
                                                                "-Xcompiler", "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def clean() -> None:
    shutil.rmtree(OBJ, ignore_errors=True)
    if os.path.exists(LIB):
        os.remove(LIB)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    build(verbose=True)
