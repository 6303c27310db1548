"""In-tree build of the sm_103a library and the ``busseq`` executable.

Outputs (git-ignored): ``busseq_gpu_gb300/lib/libbusseq_gb300.so`` and
``busseq_gpu_gb300/bin/busseq``.  Translation units are compiled in parallel;
nvcc cross-compiles sm_103a device code on machines without a GPU.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "lib", "obj")
LIB = os.path.join(PKG, "lib", "libbusseq_gb300.so")
CLI = os.path.join(PKG, "bin", "busseq")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["gene_kernels.cu", "cell_kernels.cu", "init_kernels.cu", "hmc_kernels.cu", "correct_kernels.cu", "capi.cu", "checkpoint.cu", "batch.cu",
              "format_kernels.cu", "noalloc.cu", "sampler_draws.cu"]
CPP_SOURCES = ["host_io.cpp", "simulate.cpp"]
HEADERS = ["busseq_dev.h", "rng.h", "kernels.h", "kernels_common.cuh", "correct_math.h", "capi_internal.h",
           "bic_series.h"]


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _newer(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps(src):
    hdr = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "busseq_gb300.h")]
    return [os.path.join(CSRC, src)] + hdr


def _compile(src, force):
    obj = os.path.join(OBJ, src + ".o")
    if not force and not _newer(obj, _deps(src)):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
               "-c", os.path.join(CSRC, src), "-o", obj]
    else:
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-pthread", "-I", INCLUDE, "-I", CSRC,
               "-I", os.path.join(CUDA_HOME, "include"), "-c", os.path.join(CSRC, src), "-o", obj]
    _run(cmd)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    srcs = CU_SOURCES + CPP_SOURCES
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), srcs))
    if force or _newer(LIB, objs):
        _run([NVCC, "-shared", *ARCH, "-o", LIB, *objs, "-lpthread"])  # dlopen: in libc (glibc >= 2.34)
    cli_src = os.path.join(CSRC, "cli_main.cpp")
    if force or _newer(CLI, [cli_src, LIB, os.path.join(INCLUDE, "busseq_gb300.h")]):
        _run(["g++", "-std=c++17", "-O2", "-I", INCLUDE, "-o", CLI, cli_src, "-L", os.path.dirname(LIB),
              "-lbusseq_gb300", "-Wl,-rpath,$ORIGIN/../lib"])
    if verbose:
        print("built", LIB, CLI)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
