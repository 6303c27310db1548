"""Whole-chain parity with the reference's own kernels, replayed on the CPU.

oracle/ref_chain.py ran, on a GB300, a chain of the reference's kernels
(oracle/ref_chain.cpp, compiled from BUSseq_gpu.cu where it lies) and a chain
of this sampler on the same data, both from one state in the posterior's bulk,
and stored every scalar's posterior mean, batch-means and ESS-based Monte Carlo
standard errors and posterior sd, with both chains' posterior-mode cell types
(tests/golden/ref_chain_<name>.npz, the record in .json).  This test recomputes
the comparison from the stored summaries and checks:

* the stored record is what the summaries give;
* ARI of the posterior-mode types against the simulated ones within 0.01 of
  the reference chain's;
* for each block, over the scalars whose effective sample size reaches 100 in
  both chains (a Monte Carlo error from fewer effective draws is itself
  unreliable), at most max(1, 3 %) of the scalars lie beyond 3 combined MCSE
  (about 0.3 % would for independent normal errors; the MCSE themselves are
  estimates from one chain each, and the scalars of a block are correlated),
  and where there are at least 100 such scalars their mean z-score stays
  within 0.25 (a systematic offset between the samplers would move it).

Blocks whose scalars mix too slowly for that floor in 600 kept sweeps (at the
demo size alpha, beta and delta, along the alpha/beta and delta/nu directions
the likelihood leaves nearly flat) are covered by the small-data record, where
5,000 sweeps give them enough effective draws.
"""
import json
import os

import numpy as np
import pytest

from oracle import chain_compare as cc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RECORDS = sorted(f[len("ref_chain_"):-len(".npz")] for f in os.listdir(GOLDEN)
                 if f.startswith("ref_chain_") and f.endswith(".npz"))


def _dims(z):
    G = z["a/alpha/mean"].size
    B = z["a/gamma/mean"].size // 2
    K = z["a/pi/mean"].size // B
    return B, K, G


@pytest.mark.parametrize("name", RECORDS)
def test_reference_chain_record_replays(name):
    z = np.load(os.path.join(GOLDEN, "ref_chain_%s.npz" % name))
    with open(os.path.join(GOLDEN, "ref_chain_%s.json" % name)) as f:
        rec = json.load(f)
    B, K, G = _dims(z)
    a, b = cc.from_npz(z, "a/"), cc.from_npz(z, "b/")
    got = cc.compare(a, b, B, K, G, z["W_true"])
    assert got["perm_b_to_a"] == rec["perm_b_to_a"]
    assert abs(got["ari_a"] - rec["ari_a"]) < 1e-9 and abs(got["ari_b"] - rec["ari_b"]) < 1e-9
    for blk, st in rec["blocks"].items():  # the summaries were stored in float32
        assert abs(got["blocks"][blk]["se_ess"]["frac_abs_z_gt_3"] - st["se_ess"]["frac_abs_z_gt_3"]) <= 0.01, blk
    assert abs(got["ari_diff"]) <= 0.01, got["ari_diff"]
    tested = 0
    for blk, st in got["blocks"].items():
        e = st["ess_ge_100"]
        n = e["coords"]
        if n == 0:
            continue
        tested += n
        assert round(e["frac_abs_z_gt_3"] * n) <= max(1, int(0.03 * n)), (blk, e)
        if n >= 100:
            assert abs(e["mean_z"]) <= 0.25, (blk, e)
    assert tested >= 1000, tested


def test_records_exist():
    assert RECORDS, "no reference-chain record under tests/golden"
