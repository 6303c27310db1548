"""The single-precision logarithm helpers of rng.h against double precision,
on the CPU (the header is compiled for the host with g++; the host build uses
an exact division where the device uses the 1-ulp reciprocal, whose extra
error is one more float rounding of the quotient).

log1p_shift(c mu, 2 phi + (2 + c) mu) must equal log(1 + c mu / (phi + mu))
to 4e-7 relative over |c| <= 1/2, means 1e-4 to 1e5 and dispersions 0.05 to
1e4; log_fast, log1p_fast and log_ratio to 4e-7 relative (1e-7 absolute near
log 1 = 0) over their ranges.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("logs")
    src = d / "l.cpp"
    src.write_text('#include "rng.h"\n'
                   'extern "C" float shift(float cmu, float den) { return bq::log1p_shift(cmu, den); }\n'
                   'extern "C" float lf(float x) { return bq::log_fast(x); }\n'
                   'extern "C" float l1p(float y) { return bq::log1p_fast(y); }\n'
                   'extern "C" float lr(float a, float b, float d) { return bq::log_ratio(a, b, d); }\n')
    so = str(d / "l.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I",
                    os.path.join(ROOT, "busseq_gpu_gb300", "csrc"), str(src), "-o", so], check=True)
    L = C.CDLL(so)
    for f, n in (("shift", 2), ("lf", 1), ("l1p", 1), ("lr", 3)):
        getattr(L, f).restype = C.c_float
        getattr(L, f).argtypes = [C.c_float] * n
    return L


def test_log1p_shift(lib):
    rng = np.random.default_rng(3)
    c = rng.uniform(-0.5, 0.5, 20000).astype(np.float32)
    mu = np.exp(rng.uniform(np.log(1e-4), np.log(1e5), c.size)).astype(np.float32)
    phi = np.exp(rng.uniform(np.log(0.05), np.log(1e4), c.size)).astype(np.float32)
    worst = 0.0
    for ci, mi, pi in zip(c, mu, phi):
        cmu = np.float32(ci * mi)
        den = np.float32(np.fma(np.float32(2.0) + ci, mi, np.float32(2.0) * pi)) if hasattr(np, "fma") else \
            np.float32((np.float32(2.0) + ci) * mi + np.float32(2.0) * pi)
        got = lib.shift(cmu, den)
        want = np.log1p(float(ci) * float(mi) / (float(pi) + float(mi)))
        if want != 0.0:
            worst = max(worst, abs(got - want) / abs(want))
    assert worst <= 4e-7, worst


def test_log_fast_family(lib):
    rng = np.random.default_rng(4)
    x = np.exp(rng.uniform(-80, 80, 20000)).astype(np.float32)
    for v in x:
        want = np.log(float(v))
        assert abs(lib.lf(v) - want) <= 4e-7 * abs(want) + 1e-7, v
    y = rng.uniform(-0.9, 20.0, 20000).astype(np.float32)
    for v in y:
        want = np.log1p(float(v))
        assert abs(lib.l1p(v) - want) <= 4e-7 * abs(want) + 1e-12, v
    a = np.exp(rng.uniform(-10, 10, 20000)).astype(np.float32)
    b = (a * np.exp(rng.uniform(-3, 3, a.size))).astype(np.float32)
    for ai, bi in zip(a, b):
        want = np.log(float(ai) / float(bi))
        assert abs(lib.lr(ai, bi, np.float32(ai - bi)) - want) <= 4e-7 * abs(want) + 1e-7, (ai, bi)
