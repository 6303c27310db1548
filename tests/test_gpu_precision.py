"""Error of the single-precision kernels against the FP64 oracle, per parameter
and per block log acceptance ratio, at the demo (config 0) and headline
(config 1, on a cell subset) shapes.

From one warm state, every stage of the sweep runs on the GPU and in the
oracle at the same sweep index (the same uniforms).  For each parameter, over
the coordinates whose accept / reject decision agrees, the table gives the
largest and the median relative error |gpu - orc| / |orc| (over all such
coordinates, and over the accepted ones, where a new value was computed).
For each block's log acceptance ratio it gives the largest and the median
absolute error, the largest error relative to max(1, |lr|), and the largest
error relative to the summed size of the ratio's float pieces.

The kernels keep parameters in float and sum every cross-thread reduction as
a float-float pair (about 48 bits); the decision compares log u with that
pair converted to double.  The table shows where the error comes from: the
parameters carry float rounding (relative 1e-7 to 1e-6), and the log ratios
carry the float evaluation of each entry's term, not the summation.

The table is printed, and written as JSON to $BUSSEQ_PRECISION_TABLE when set.
Bounds asserted: parameters 2e-5 relative (values below 1e-3 in size against
1e-3); log ratios within the parity tolerance 5e-3 + 5e-5 |lr| + 4e-7 times
the summed size of their float pieces (ratios below -20 on both sides are
certain rejections and are left out).
"""
import json
import os

import numpy as np
import pytest

import busseq_gpu_gb300 as bq
from oracle import pyoracle as po
from tests.parity_util import LR_CERTAIN_REJECT, lr_ok, oracle_state

pytestmark = pytest.mark.gpu

CASES = {
    "config0 (B=4: 300/300/200/200, G=3000, K=5)": ([300, 300, 200, 200], 3000, 5, 13579, 30),
    "config1 shape (B=4 x 250 cells, G=10^4, K=8)": ([250, 250, 250, 250], 10000, 8, 13580, 20),
}


def _param_stats(old, g, o, mask=None):
    """Relative error over the coordinates whose decision agrees; values below
    1e-3 in size are measured against 1e-3 (the parity tests' atol / rtol)."""
    old, g, o = (np.asarray(a, np.float64).ravel() for a in (old, g, o))
    m = np.ones_like(old, bool) if mask is None else np.asarray(mask, bool).ravel()
    same = m & ((g != old) == (o != old))
    rel = np.abs(g - o) / np.maximum(np.abs(o), 1e-3)
    acc = same & (o != old)
    out = {"coords": int(m.sum()), "decisions_agree": int(same.sum()),
           "max_rel": float(rel[same].max()) if same.any() else 0.0,
           "median_rel": float(np.median(rel[same])) if same.any() else 0.0,
           "accepted": int(acc.sum()),
           "max_rel_accepted": float(rel[acc].max()) if acc.any() else 0.0,
           "median_rel_accepted": float(np.median(rel[acc])) if acc.any() else 0.0}
    return out, float(rel[same].max()) if same.any() else 0.0


def _lr_stats(lg, lo, mask=None, scale=None):
    """Errors of the log ratios that can decide (not both below -20)."""
    lg, lo = np.asarray(lg, np.float64).ravel(), np.asarray(lo, np.float64).ravel()
    sc = np.zeros_like(lo) if scale is None else np.asarray(scale, np.float64).ravel()
    m = np.isfinite(lo) & np.isfinite(lg) & ~((lg < LR_CERTAIN_REJECT) & (lo < LR_CERTAIN_REJECT))
    if mask is not None:
        m &= np.asarray(mask, bool).ravel()
    ok = bool(np.all(lr_ok(lg[m], lo[m], sc[m])))
    if not m.any():
        return {"n": 0}, ok
    d = np.abs(lg - lo)[m]
    return {"n": int(m.sum()), "max_abs": float(d.max()), "median_abs": float(np.median(d)),
            "max_rel_to_max1": float((d / np.maximum(1.0, np.abs(lo[m]))).max()),
            "max_over_piece_size": float((d / np.maximum(sc[m], 1e-300)).max()) if scale is not None else None,
            "median_piece_size": float(np.median(sc[m])) if scale is not None else None,
            "typical_abs_lr": float(np.median(np.abs(lo[m])))}, ok


def _stage(s, st, stage, it, n_unch=1 << 30):
    s.set_state(st)
    s.run_stage(stage, it, n_unch)
    return s.get_state(), s.log_ratios()


def test_precision_table():
    table = {}
    for name, (n_b, G, K, seed, warm) in CASES.items():
        Y, _, _ = bq.simulate(n_b, G, K, seed)
        s = bq.Sampler(Y, n_b, K, seed=seed, p0=0.3)
        try:
            s.begin(warm, warm, 0)
            s.sweeps(warm)
            s.synchronize()
            st = s.get_state()
            nb = np.array(n_b)
            B = len(n_b)
            first = np.zeros(sum(n_b), bool)
            first[np.concatenate([[0], np.cumsum(n_b)[:-1]])] = True
            params, lrs, worst = {}, {}, 0.0
            checks = []

            def orc():
                o = oracle_state(Y, nb, K, seed, st)
                return o, po.Debug(o)

            # stage 0: Z/X, gamma0, gamma1, alpha, L, p / tau0
            g, lr = _stage(s, st, 0, 41, 10)
            o, d = orc()
            o.step("zx", 41, debug=d)
            o.X[:], o.Z[:] = g["X"], g["Z"]
            o.step("gamma", 41, debug=d)
            o.step("alpha", 41, debug=d)
            o.step("L", 41, debug=d)
            o.L[:] = g["L"]
            o.step("ptau", 41, debug=d)
            # gamma1's ratio uses the new gamma0: compared where the gamma0 decisions agree
            same0 = (g["gamma"][0] != st["gamma"][0]) == (o.gamma[0] != st["gamma"][0])
            for k, idx, m in (("gamma0", 0, None), ("gamma1", 1, same0)):
                params[k], w = _param_stats(st["gamma"][idx], g["gamma"][idx], o.gamma[idx], m)
                worst = max(worst, w)
                lrs[k], ok = _lr_stats(lr["gamma"][idx], d.lr_gamma[idx], m, d.sc_gamma[idx])
                checks.append((k, ok))
            params["alpha"], w = _param_stats(st["alpha"], g["alpha"], o.alpha)
            worst = max(worst, w)
            lrs["alpha"], ok = _lr_stats(lr["alpha"], d.lr_alpha, None, d.sc_alpha)
            checks.append(("alpha", ok))
            for k, idx in (("p", 0), ("tau0", 1)):
                if d.mg_ptau[idx] > 1e-5:
                    params[k], w = _param_stats(st["p_tau0"][idx:idx + 1], g["p_tau0"][idx:idx + 1],
                                                o.p_tau0[idx:idx + 1])
                    worst = max(worst, w)
            # stage 1: beta, nu
            g, lr = _stage(s, st, 1, 57)
            o, d = orc()
            o.step("beta", 57, debug=d)
            params["beta"], w = _param_stats(st["beta"][1:], g["beta"][1:], o.beta[1:])
            worst = max(worst, w)
            lrs["beta"], ok = _lr_stats(lr["beta"][1:], d.lr_beta[1:], None, d.sc_beta[1:])
            checks.append(("beta", ok))
            o.beta[:] = g["beta"]
            o.step("nu", 57, debug=d)
            params["nu"], w = _param_stats(st["nu"][1:], g["nu"][1:], o.nu[1:])
            worst = max(worst, w)
            lrs["nu"], ok = _lr_stats(lr["nu"][1:], d.lr_nu[1:], None, d.sc_nu[1:])
            checks.append(("nu", ok))
            # stage 2: delta
            g, lr = _stage(s, st, 2, 63)
            o, d = orc()
            o.step("delta", 63, debug=d)
            params["delta"], w = _param_stats(st["delta"], g["delta"], o.delta, ~first)
            worst = max(worst, w)
            lrs["delta"], ok = _lr_stats(lr["delta"], d.lr_delta, ~first, d.sc_delta)
            checks.append(("delta", ok))
            # stage 3: phi
            g, lr = _stage(s, st, 3, 71)
            o, d = orc()
            o.step("phi", 71, debug=d)
            params["phi"], w = _param_stats(st["phi"], g["phi"], o.phi)
            worst = max(worst, w)
            lrs["phi"], ok = _lr_stats(lr["phi"], d.lr_phi, None, d.sc_phi)
            checks.append(("phi", ok))
            # stage 4: W (the reference's MH move)
            g, lr = _stage(s, st, 4, 83)
            o, d = orc()
            o.step("W", 83, w_update=0, debug=d)
            lrs["W"], ok = _lr_stats(lr["W"], d.lr_W, None, d.sc_W)
            checks.append(("W", ok))
            # stage 5: pi
            g, _ = _stage(s, st, 5, 97)
            o, d = orc()
            o.step("pi", 97, debug=d)
            okpi = d.mg_pi.min(axis=1) > 1e-5
            rel = np.abs(g["pi"][okpi] - o.pi[okpi]) / o.pi[okpi]
            params["pi"] = {"coords": int(okpi.sum() * K), "max_rel": float(rel.max()) if rel.size else 0.0,
                            "median_rel": float(np.median(rel)) if rel.size else 0.0}
            worst = max(worst, params["pi"]["max_rel"])
        finally:
            s.close()
        table[name] = {"parameters": params, "log_ratios": lrs}
        bad = [k for k, ok in checks if not ok]
        assert not bad, (name, bad)
        assert worst <= 2e-5, (name, worst)
    path = os.environ.get("BUSSEQ_PRECISION_TABLE")
    if path:
        with open(path, "w") as f:
            json.dump(table, f, indent=1)
    for name, t in table.items():
        print(name)
        for k, v in t["parameters"].items():
            print("  %-7s max rel %.2e  median rel %.2e" % (k, v["max_rel"], v["median_rel"]))
        for k, v in t["log_ratios"].items():
            print("  lr %-6s max abs %.2e  median abs %.2e  (median |lr| %.1f)" % (k, v["max_abs"], v["median_abs"],
                                                                                v["typical_abs_lr"]))
