"""Helpers shared by the GPU parity tests (kernels vs the FP64 oracle).

Tolerances (single-precision kernels against a double-precision oracle that
consumes the same uniforms):
  * float parameters where both sides took the same decision: rtol 1e-5,
    atol 1e-6 (the kernels store parameters in float);
  * log acceptance ratios: |lr_gpu - lr_orc| <= 5e-3 + 5e-5 |lr_orc|
    + 4e-7 scale.  The kernels evaluate each entry's term in float, in pieces
    that can be far larger than the term (for a highly expressed gene the
    ratio is a difference of two sums of ~1e5); `scale` (from the oracle) is
    the summed size of those pieces, and 4e-7 the relative accuracy of the
    single-precision logarithms (tests/test_log_helpers.py), so the last term
    is the worst case of a correct float evaluation.  A formula error (for
    instance the cancellation of log1p(d/b) when a Gamma proposal lands far
    below phi) shows up as 0.1 to 2 nats and fails this bound.  Where both
    ratios are below -20 the proposal is rejected on both sides whatever their
    difference (every uniform is at least 2^-24, so log u >= -16.7), and the
    ratios are not compared: such a ratio can be far off on the GPU when a
    Gamma proposal underflows single precision (it is then held at 1e-30);
  * a Metropolis decision may differ only where log(u) lies between the two
    log ratios, i.e. the oracle's margin |log u - lr_orc| <= |lr_gpu - lr_orc|;
  * integer draws (X, Z, L, W, ...) must be bit-exact except where the oracle
    certifies a near-tie: its normalised margin at a deciding comparison is
    below TIE_TOL.
"""
from __future__ import annotations

import numpy as np

from oracle import pyoracle as po

RTOL = 1e-5
ATOL = 1e-6
LR_ATOL = 5e-3
LR_RTOL = 5e-5
LR_SCALE = 4e-7
LR_CERTAIN_REJECT = -20.0
TIE_TOL = 3e-5


def lr_ok(lg, lo, scale=None):
    """Mask of the log ratios within tolerance (certain rejections pass)."""
    lg, lo = np.asarray(lg, np.float64), np.asarray(lo, np.float64)
    sc = 0.0 if scale is None else np.asarray(scale, np.float64)
    tol = LR_ATOL + LR_RTOL * np.abs(lo) + LR_SCALE * sc
    return (np.abs(lg - lo) <= tol) | ((lg < LR_CERTAIN_REJECT) & (lo < LR_CERTAIN_REJECT))


def oracle_state(Y, n_b, K, seed, st: dict) -> po.State:
    o = po.State(Y, n_b, K, seed)
    o.X[:] = st["X"]
    o.Z[:] = st["Z"]
    o.W[:] = st["W"]
    o.L[:] = st["L"]
    for f in ("alpha", "mu_alpha", "beta", "nu", "mu_nu", "delta", "mu_delta", "phi", "gamma", "pi", "p_tau0"):
        getattr(o, f)[...] = np.asarray(st[f], dtype=np.float64).reshape(getattr(o, f).shape)
    return o


def check_mh(name, old, new_gpu, new_orc, lr_gpu, lr_orc, mg_orc, mask=None, report=None, scale=None):
    """Compare one family of Metropolis updates.  Returns the number of
    certified near-tie flips."""
    old = np.asarray(old, np.float64).ravel()
    ng = np.asarray(new_gpu, np.float64).ravel()
    no = np.asarray(new_orc, np.float64).ravel()
    lg = np.asarray(lr_gpu, np.float64).ravel()
    lo = np.asarray(lr_orc, np.float64).ravel()
    mg = np.asarray(mg_orc, np.float64).ravel()
    sc = None if scale is None else np.asarray(scale, np.float64).ravel()
    m = np.ones_like(old, bool) if mask is None else np.asarray(mask, bool).ravel()
    dlr = np.abs(lg - lo)
    bad_lr = m & ~lr_ok(lg, lo, sc)
    assert not bad_lr.any(), "%s: log ratio off at %s: gpu %s orc %s" % (
        name, np.flatnonzero(bad_lr)[:5], lg[bad_lr][:5], lo[bad_lr][:5])
    acc_g = ng != old
    acc_o = no != old
    flip = m & (acc_g != acc_o)
    if flip.any():
        ok = mg[flip] <= dlr[flip] + 1e-6
        assert ok.all(), "%s: decision flips that are not near-ties at %s (margin %s, |dlr| %s)" % (
            name, np.flatnonzero(flip)[~ok][:5], mg[flip][~ok][:5], dlr[flip][~ok][:5])
    same = m & ~flip
    np.testing.assert_allclose(ng[same], no[same], rtol=RTOL, atol=ATOL, err_msg=name)
    if report is not None:
        live = m & ~((lg < LR_CERTAIN_REJECT) & (lo < LR_CERTAIN_REJECT))
        report[name] = dict(n=int(m.sum()), accepted=int((acc_g & m).sum()), flips=int(flip.sum()),
                            max_dlr=float(dlr[live].max()) if live.any() else 0.0,
                            max_dlr_over_scale=float((dlr[live] / np.maximum(sc[live], 1e-300)).max())
                            if sc is not None and live.any() else None)
    return int(flip.sum())


def check_discrete(name, got, want, margin, mask=None, tol=TIE_TOL, max_frac=1e-3, report=None):
    got = np.asarray(got).ravel()
    want = np.asarray(want).ravel()
    margin = np.asarray(margin, np.float64).ravel()
    m = np.ones_like(got, bool) if mask is None else np.asarray(mask, bool).ravel()
    diff = m & (got != want)
    if diff.any():
        ok = margin[diff] < tol
        assert ok.all(), "%s: %d mismatches that are not near-ties (margins %s, at %s)" % (
            name, int((~ok).sum()), margin[diff][~ok][:5], np.flatnonzero(diff)[~ok][:5])
    assert diff.sum() <= max(1, max_frac * m.sum()), "%s: too many near-tie mismatches (%d of %d)" % (
        name, int(diff.sum()), int(m.sum()))
    if report is not None:
        report[name] = dict(n=int(m.sum()), mismatches=int(diff.sum()))
    return int(diff.sum())
