"""The series of the BIC's zero counts (bic_series.h), in double precision and
in the float-float arithmetic the device runs, against the reference's own
formula (BUSseq_gpu.cu:967-1003), on the CPU.

The header is compiled for the host with g++ and called through ctypes.  The
reference sums, for Y = 0, log[ NB(0) + sum_{x=1}^{floor(3 mu)-1} NB(x)
sigmoid(g0 + g1 x) ] term by term in log space with lgamma; it is restated
here in Python double precision.  The recurrence must agree to 1e-12
relative (both sides round differently; the truncated tail is below 2^-60 of
the sum) over means 0.1 to 1100, dispersions 0.4 to 400, and dropout slopes
down to -2.7 and up to 0 (the log-space fallback); the float-float version to
2e-12.
"""
import ctypes as C
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# C entry points over the header: zs (double series), zf (float-float
# series), zt (the device BIC's zero-count term, per-cell constants hoisted),
# lg / l1p (the table logarithm and log1p)
_WRAP = r"""
#include "bic_series.h"
static double tab[2 * bq::BIC_LOG_TAB];
static int init() { for (int j = 0; j < bq::BIC_LOG_TAB; ++j) bq::bic_log_entry(tab, j); return 0; }
static int done = init();
extern "C" double zs(double mu, double lp, double l1, double phi, double g0, double g1) {
  return bq::bic_zero_series(mu, lp, l1, phi, g0, g1); }
extern "C" double zf(double mu, double lp, double l1, double phi, double g0, double g1) {
  return bq::bic_zero_series_ff(mu, lp, l1, phi, g0, g1); }
extern "C" double zt(double mu, double lp, double l1, double phi, double g0, double g1) {
  const bq::BicCell c = bq::bic_cell(g0, g1);
  return bq::bic_zero_term(c, tab, mu, lp, l1, phi); }
extern "C" double lg(double x) { return bq::bic_log(tab, x); }
extern "C" double l1p(double x) { return bq::bic_log1p(tab, x); }
"""


@pytest.fixture(scope="module")
def series(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("bic")
    src = d / "s.cpp"
    src.write_text(_WRAP)
    so = str(d / "s.so")
    # no contraction of a * b + c into fma beyond the explicit fmaf calls: the
    # float-float steps rely on IEEE rounding of each operation
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I",
                    os.path.join(ROOT, "busseq_gpu_gb300", "csrc"), str(src), "-o", so], check=True)
    lib = C.CDLL(so)
    for f in (lib.zs, lib.zf, lib.zt):
        f.restype = C.c_double
        f.argtypes = [C.c_double] * 6
    for f in (lib.lg, lib.l1p):
        f.restype = C.c_double
        f.argtypes = [C.c_double]
    return lib


def _clamped_logs(mu, phi):
    # BUSseq_gpu.cu:977-986
    pb = mu / (mu + phi)
    if pb < math.exp(-250.0):
        return -250.0, math.log(1 - pb)
    if 1 - pb < math.exp(-250.0):
        return math.log(pb), -250.0
    return math.log(pb), math.log(1 - pb)


def _reference(mu, phi, g0, g1):
    logp, l1 = _clamped_logs(mu, phi)
    s = phi * l1
    for x in range(1, int(3 * mu)):
        t = g0 + g1 * x
        ls = -math.log1p(math.exp(-t)) if t > 0 else t - math.log1p(math.exp(t))
        term = ls + math.lgamma(phi + x) - math.lgamma(1 + x) - math.lgamma(phi) + x * logp + phi * l1
        s = term + math.log1p(math.exp(s - term)) if term > s else s + math.log1p(math.exp(term - s))
    return s, logp, l1


def test_zero_count_series_matches_the_reference_formula(series):
    rng = np.random.default_rng(7)
    cases = [(0.3, 5, -0.5, -0.2), (12, 5, -0.5, -0.2), (150, 3, -0.5, -0.2), (1000, 20, 0.5, -0.05),
             (50, 0.5, -1, -0.3), (5, 200, 2, -1), (300, 400, -0.2, -0.01), (0.34, 7, 0, -0.3), (1.0, 5, 0, -0.3),
             (40, 5, -0.5, 0.0), (25, 3, 1.0, 0.02)]  # the last two: the log-space fallback (g1 >= 0)
    for _ in range(150):
        cases.append((float(np.exp(rng.uniform(-2.3, 7))), float(np.exp(rng.uniform(-0.9, 6))),
                      float(rng.normal(0, 2)), -float(np.exp(rng.uniform(-7, 1)))))
    worst, worst_ff, worst_t = 0.0, 0.0, 0.0
    for mu, phi, g0, g1 in cases:
        want, logp, l1 = _reference(mu, phi, g0, g1)
        got = series.zs(mu, logp, l1, phi, g0, g1)
        err = abs(got - want) / max(1.0, abs(want))
        assert err <= 1e-12, (mu, phi, g0, g1, got, want)
        worst = max(worst, err)
        # the float-float version the device runs: the same sum to 48 bits
        got_ff = series.zf(mu, logp, l1, phi, g0, g1)
        err_ff = abs(got_ff - want) / max(1.0, abs(want))
        assert err_ff <= 2e-12, (mu, phi, g0, g1, got_ff, want)
        worst_ff = max(worst_ff, err_ff)
        # the device BIC's form: hoisted constants, one log1p at the close
        got_t = series.zt(mu, logp, l1, phi, g0, g1)
        err_t = abs(got_t - want) / max(1.0, abs(want))
        assert err_t <= 2e-12, (mu, phi, g0, g1, got_t, want)
        worst_t = max(worst_t, err_t)
    print("worst relative difference: double", worst, "float-float", worst_ff, "device form", worst_t)


def test_table_logarithm_and_log1p(series):
    """Tang's table method: within a few units of 2^-53 times max(1, |log x|)
    of the library logarithm over normal doubles (arguments from 1e-300 to
    1e300, near powers of two and near 1), and log1p to the same bound (an
    absolute bound near 0: the BIC adds these values to sums of order one and
    larger, so only absolute errors reach it)."""
    rng = np.random.default_rng(11)
    xs = list(np.exp(rng.uniform(-690, 690, 4000))) + list(1.0 + rng.uniform(-1e-3, 1e-3, 2000))
    xs += [2.0 ** e * f for e in range(-60, 61) for f in (1.0, 1.0 - 2 ** -52, 1.0 + 2 ** -52, 1.5)]
    xs += [1.0, 2.2250738585072014e-308, 1.7976931348623157e308, 0.75, 1.4142135623730951]
    worst = 0.0
    for x in xs:
        want = math.log(x)
        err = abs(series.lg(x) - want) / max(1.0, abs(want))
        worst = max(worst, err)
    assert worst <= 8 * 2.0 ** -53, worst
    ss = list(np.exp(rng.uniform(-700, 80, 4000))) + [0.0, 1e-320, 2.0 ** -53, 0.5, 1.0, 3.0, 1e15, 1e300]
    worst1 = 0.0
    for v in ss:
        want = math.log1p(v)
        err = abs(series.l1p(v) - want) / max(1.0, want)
        worst1 = max(worst1, err)
    assert worst1 <= 8 * 2.0 ** -53, worst1
    print("table log worst", worst / 2.0 ** -53, "ulp-units; log1p", worst1 / 2.0 ** -53)
