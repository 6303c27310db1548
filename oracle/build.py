"""Build recipe for the checker side (test infrastructure only).

* ``liborc.so``    -- the FP64 OpenMP oracle (oracle/oracle.cpp), built with g++.
* ``busseq_ref.cubin`` -- the reference's device code, compiled with nvcc from
  BUSseq_gpu.cu WHERE IT LIES (the reference checkout); only done when that
  checkout exists.  Output goes to ``oracle/_ref/`` (git-ignored).
* ``ref_harness``  -- oracle/ref_harness.cpp, a CUDA-driver-API loader that runs
  the reference's deterministic kernels from that cubin (needs libcuda, so it
  is built where a driver is installed, i.e. on the GPU machine).
* ``ref_sweep_timer`` -- oracle/ref_sweep_timer.cpp, which replays the
  reference's per-sweep launch sequence from that cubin to time it.
* ``ref_chain``    -- oracle/ref_chain.cpp, which runs a whole chain (init,
  burn-in, kept sweeps) with the reference's kernels from that cubin, for the
  chain-level comparison of oracle/ref_chain.py.
* ``libsim.so``    -- the synthetic-data generator alone (oracle/sim_standalone.cpp),
  so that bench.py's CPU arms never map the product library.

Nothing in the product package imports this module.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
REF_DIR = os.path.join(HERE, "_ref")
# The reference checkout's single source file; BUSSEQ_REFERENCE_SRC points
# elsewhere when the checkout lives somewhere else.
REFERENCE_SRC = os.environ.get("BUSSEQ_REFERENCE_SRC", "/root/reference/BUSseq_gpu.cu")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")

ORACLE_SO = os.path.join(LIB_DIR, "liborc.so")
REF_CUBIN = os.path.join(REF_DIR, "busseq_ref.cubin")
HARNESS_BIN = os.path.join(LIB_DIR, "ref_harness")
SIM_SO = os.path.join(LIB_DIR, "libsim.so")
ROOT = os.path.dirname(HERE)
TIMER_BIN = os.path.join(LIB_DIR, "ref_sweep_timer")
CHAIN_BIN = os.path.join(LIB_DIR, "ref_chain")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), proc.stdout))


def _stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs if os.path.exists(s))


def oracle_cmd() -> list[str]:
    src = os.path.join(HERE, "oracle.cpp")
    return ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", ORACLE_SO, src]


def build_oracle(force: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    src = os.path.join(HERE, "oracle.cpp")
    if force or _stale(ORACLE_SO, [src]):
        _run(oracle_cmd())
    return ORACLE_SO


def build_sim(force: bool = False) -> str:
    """The generator of busseq_gpu_gb300/csrc/simulate.cpp as its own library."""
    os.makedirs(LIB_DIR, exist_ok=True)
    src = os.path.join(HERE, "sim_standalone.cpp")
    csrc = os.path.join(ROOT, "busseq_gpu_gb300", "csrc")
    inc = os.path.join(ROOT, "include")
    deps = [src, os.path.join(csrc, "simulate.cpp"), os.path.join(csrc, "rng.h"), os.path.join(inc, "busseq_gb300.h")]
    if force or _stale(SIM_SO, deps):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-pthread", "-shared", "-I", inc, "-I", csrc, "-o", SIM_SO, src])
    return SIM_SO


def build_ref_cubin(force: bool = False) -> str | None:
    """Compile the reference's kernels to a cubin (only where the reference exists)."""
    if not os.path.exists(REFERENCE_SRC):
        return REF_CUBIN if os.path.exists(REF_CUBIN) else None
    os.makedirs(REF_DIR, exist_ok=True)
    if force or _stale(REF_CUBIN, [REFERENCE_SRC]):
        nvcc = os.path.join(CUDA_HOME, "bin", "nvcc")
        _run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-o", REF_CUBIN, REFERENCE_SRC])
    return REF_CUBIN


def build_harness(force: bool = False) -> str | None:
    """Build the driver-API harness; needs libcuda (skipped where no driver is installed)."""
    src = os.path.join(HERE, "ref_harness.cpp")
    os.makedirs(LIB_DIR, exist_ok=True)
    if not force and not _stale(HARNESS_BIN, [src]):
        return HARNESS_BIN
    libdirs = [os.path.join(CUDA_HOME, "lib64"), os.path.join(CUDA_HOME, "lib64", "stubs")]
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(CUDA_HOME, "include"), "-o", HARNESS_BIN, src]
    for d in libdirs:
        cmd += ["-L", d]
    cmd += ["-lcuda"]
    try:
        _run(cmd)
    except RuntimeError:
        return None
    return HARNESS_BIN


def _driver_api_tool(src_name: str, out: str, force: bool) -> str | None:
    """A driver-API program (needs libcuda; None where it cannot be linked)."""
    src = os.path.join(HERE, src_name)
    os.makedirs(LIB_DIR, exist_ok=True)
    if not force and not _stale(out, [src]):
        return out
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(CUDA_HOME, "include"), "-o", out, src]
    for d in (os.path.join(CUDA_HOME, "lib64"), os.path.join(CUDA_HOME, "lib64", "stubs")):
        cmd += ["-L", d]
    cmd += ["-lcuda"]
    try:
        _run(cmd)
    except RuntimeError:
        return None
    return out


def build_ref_timer(force: bool = False) -> str | None:
    """Build the reference sweep timer (driver API; needs libcuda, like the harness)."""
    return _driver_api_tool("ref_sweep_timer.cpp", TIMER_BIN, force)


def build_ref_chain(force: bool = False) -> str | None:
    """Build the reference chain runner (driver API; needs libcuda)."""
    return _driver_api_tool("ref_chain.cpp", CHAIN_BIN, force)


def build_all(force: bool = False) -> dict:
    out = {"oracle": build_oracle(force), "sim": build_sim(force), "ref_cubin": build_ref_cubin(force)}
    if shutil.which("g++"):
        out["harness"] = build_harness(force)
        out["ref_timer"] = build_ref_timer(force)
        out["ref_chain"] = build_ref_chain(force)
    return out


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
