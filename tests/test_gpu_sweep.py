"""Whole-sweep behaviour on the GPU: invariants, reproducibility, posterior
summaries, BIC parity with the oracle, recovery of the simulated cell types,
and the drop-in command line with the reference's output files."""
import os
import subprocess

import numpy as np
import pytest

import busseq_gpu_gb300 as bq
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

DEMO = ([300, 300, 200, 200], 3000, 5, 13579)


def _first_cells(n_b):
    return np.concatenate([[0], np.cumsum(n_b)[:-1]])


def _check_invariants(st, Y, n_b, K):
    y0 = Y == 0
    assert np.array_equal(st["X"][~y0], Y[~y0])
    assert not st["Z"][~y0].any()
    assert np.all(st["Z"][y0 & (st["X"] > 0)] == 1)
    assert np.all(st["X"] >= 0)
    assert np.all(st["beta"][0] == 0) and np.all(st["nu"][0] == 0)
    assert np.all(st["delta"][_first_cells(n_b)] == 0)
    assert np.all((st["W"] >= 0) & (st["W"] < K))
    assert np.all(np.isfinite(st["alpha"])) and np.all(np.isfinite(st["beta"])) and np.all(np.isfinite(st["nu"]))
    assert np.all(st["phi"] > 0) and np.all(np.isfinite(st["phi"]))
    np.testing.assert_allclose(st["pi"].sum(axis=1), 1.0, rtol=1e-5)
    assert 0 < st["p_tau0"][0] < 1 and st["p_tau0"][1] > 0
    assert np.all(st["gamma"][1] < 0)


def _ari(a, b):
    from math import comb
    a = np.asarray(a)
    b = np.asarray(b)
    ua, ia = np.unique(a, return_inverse=True)
    ub, ib = np.unique(b, return_inverse=True)
    M = np.zeros((len(ua), len(ub)), np.int64)
    np.add.at(M, (ia, ib), 1)
    s_ij = sum(comb(int(x), 2) for x in M.ravel())
    s_a = sum(comb(int(x), 2) for x in M.sum(1))
    s_b = sum(comb(int(x), 2) for x in M.sum(0))
    n = comb(len(a), 2)
    exp = s_a * s_b / n
    return (s_ij - exp) / (0.5 * (s_a + s_b) - exp)


def test_init_matches_oracle():
    n_b, G, K, seed = [50, 40, 30], 400, 4, 5
    Y, _, _ = bq.simulate(n_b, G, K, seed)
    s = bq.Sampler(Y, n_b, K, seed=seed, p0=0.2)
    st = s.get_state()
    s.close()
    o = po.State(Y, n_b, K, seed)
    o.init(0.2)
    np.testing.assert_array_equal(st["W"], o.W)
    np.testing.assert_allclose(st["delta"], o.delta, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(st["alpha"], o.alpha, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(st["beta"], o.beta, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(st["nu"], o.nu, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(st["mu_nu"], o.mu_nu, rtol=1e-5, atol=1e-6)
    assert np.mean(st["L"] != o.L) < 1e-3
    np.testing.assert_array_equal(st["X"], Y)
    assert not st["Z"].any()


def test_sweeps_invariants_and_reproducible():
    n_b, G, K, seed = DEMO
    Y, _, _ = bq.simulate(n_b, G, K, seed)
    states = []
    for _ in range(2):
        s = bq.Sampler(Y, n_b, K, seed=seed)
        s.begin(60, 30, 20)
        s.sweeps(60)
        s.finish()
        states.append(s.get_state())
        s.close()
    _check_invariants(states[0], Y, np.array(n_b), K)
    for k in states[0]:
        assert np.array_equal(states[0][k], states[1][k]), k


def test_posterior_summaries_match_draws():
    n_b, G, K, seed = [40, 30, 30], 200, 3, 21
    Y, _, _ = bq.simulate(n_b, G, K, seed)
    s = bq.Sampler(Y, n_b, K, seed=seed, keep_draws=True)
    s.run(40, 20, 10)
    e = s.estimates()
    p = s.preserved()
    s.close()
    np.testing.assert_allclose(e["alpha"], p["alpha"].mean(1), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(e["beta"][1:].ravel(), p["beta"].mean(1), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(e["L"].ravel(), p["L"].mean(1), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(e["nu"][1:].ravel(), p["nu"].mean(1), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(e["delta"], p["delta"].mean(1), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(e["phi"].ravel(), p["phi"].mean(1), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(e["gamma"].ravel(), p["gamma"].mean(1), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(e["pi"].ravel(), p["pi"].mean(1), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(e["p_tau0"], p["p_tau0"].mean(1), rtol=1e-6, atol=1e-9)
    counts = np.stack([(p["W"] == k).sum(1) for k in range(K)])
    np.testing.assert_array_equal(e["W"], counts.argmax(0))


@pytest.mark.parametrize("n_b,G,K,seed", [
    ([60, 50, 40], 300, 3, 8),                   # 256 threads per cell, two gene passes
    ([40, 55, 30, 45, 35, 50], 500, 12, 21),     # 160 threads (12 job slots each), four passes
    ([70, 66, 80], 100, 64, 5),                  # the largest K: 32 threads, 2048 job slots
])
def test_bic_matches_oracle(n_b, G, K, seed):
    """The BIC kernel forms its per-CTA thread count and job queue from K
    (K slots per thread, at most 2048); each shape against the FP64 oracle."""
    Y, _, _ = bq.simulate(n_b, G, K, seed)
    s = bq.Sampler(Y, n_b, K, seed=seed)
    s.run(30, 15, 10)
    e = s.estimates(with_XZ=False)
    bic = s.bic()
    s.close()
    o = po.State(Y, n_b, K, seed)
    o.alpha[:] = e["alpha"]
    o.beta[:] = e["beta"]
    o.nu[:] = e["nu"]
    o.delta[:] = e["delta"]
    o.phi[:] = e["phi"]
    o.gamma[:] = e["gamma"]
    o.pi[:] = e["pi"]
    want, _ = o.bic()
    # every part of the BIC is double precision on both sides (the zero counts'
    # series included), so only the order of the sums differs
    assert abs(bic - want) <= 1e-10 * abs(want), (bic, want)


def test_recovers_cell_types_demo():
    """Demo-size data: single-site Gibbs updates of W can lock two simulated
    types into one cluster (a local mode the reference's sampler shares), so
    the bar is that most of the structure is found."""
    n_b, G, K, seed = DEMO
    Y, W_true, _ = bq.simulate(n_b, G, K, seed)
    s = bq.Sampler(Y, n_b, K, seed=seed)
    s.run(600, 300, 150)
    e = s.estimates(with_XZ=False)
    s.close()
    assert _ari(e["W"], W_true) > 0.7


def test_chain_matches_oracle_chain():
    """Whole chains: the GPU sampler and the FP64 oracle start from the same
    data and seed and consume the same Philox streams, so their cell-type
    assignments and ARI against the simulated truth must agree (this data set
    collapses two simulated types into one cluster in both chains)."""
    n_b, G, K, seed = [200, 200, 200], 2000, 3, 4242
    Y, W_true, _ = bq.simulate(n_b, G, K, seed, de_frac=0.4)
    s = bq.Sampler(Y, n_b, K, seed=seed, p0=0.25)
    s.begin(120, 60, 60)
    s.sweeps(120)
    s.finish()
    g = s.get_state()
    s.close()
    o = po.State(Y, n_b, K, seed)
    o.init(0.25)
    for it in range(120):
        o.sweep(it, 60)
    assert abs(_ari(g["W"], W_true) - _ari(o.W, W_true)) <= 0.01
    assert np.mean(g["W"] == o.W) >= 0.99


def test_cli_drop_in(tmp_path):
    n_b, G, K = [30, 25, 20], 120, 3
    Y, _, _ = bq.simulate(n_b, G, K, 99)
    cnt = tmp_path / "counts.txt"
    dim = tmp_path / "dim.txt"
    np.savetxt(cnt, Y, fmt="%d", delimiter=" ")
    dim.write_text("\n".join(str(x) for x in n_b))
    prefix = str(tmp_path / "out")
    r = subprocess.run([bq.CLI_PATH, "-B", "3", "-N", str(dim), "-G", str(G), "-K", str(K), "-s", "99", "-c",
                        str(cnt), "-i", "40", "-b", "20", "-u", "10", "-p", "-o", prefix],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines() == [
        "Seed is 99", "Start reading file.", "Start initialization.", "Start MCMC.",
        "Burnin completed. Start recording iterations.", "Start posterior inference.",
        "Start writing output files.", "Start writing preserved iterations."]
    N = sum(n_b)
    shapes = {"_post_Z.txt": (N, G), "_post_X.txt": (N, G), "_post_gamma.txt": (2, 3), "_post_alpha.txt": (G, 1),
              "_post_L.txt": (K - 1, G), "_post_beta.txt": (K, G), "_post_nu.txt": (3, G),
              "_post_delta.txt": (N, 1), "_post_phi.txt": (3, G), "_post_W.txt": (N, 1), "_post_pi.txt": (3, K),
              "_BIC.txt": (1, 1), "_preserved_gamma.txt": (6, 20), "_preserved_alpha.txt": (G, 20),
              "_preserved_L.txt": ((K - 1) * G, 20), "_preserved_beta.txt": ((K - 1) * G, 20),
              "_preserved_p.txt": (2, 20), "_preserved_nu.txt": (2 * G, 20), "_preserved_delta.txt": (N, 20),
              "_preserved_phi.txt": (3 * G, 20), "_preserved_W.txt": (N, 20), "_preserved_pi.txt": (3 * K, 20)}
    for suffix, shp in shapes.items():
        text = open(prefix + suffix).read()
        rows = text.rstrip("\n").split("\n")
        assert len(rows) == shp[0], suffix
        assert all(len(r.split("\t")) == shp[1] for r in rows), suffix
        assert text.endswith("\n")
    beta_rows = open(prefix + "_post_beta.txt").read().split("\n")
    assert beta_rows[0] == "\t".join(["0.000000"] * G)
    ptxt = open(prefix + "_post_p.txt").read()
    assert ptxt.count("\t") == 2 and ptxt.endswith("\t") and "\n" not in ptxt
    Z = np.loadtxt(prefix + "_post_Z.txt", dtype=np.int64, ndmin=2)
    X = np.loadtxt(prefix + "_post_X.txt", dtype=np.int64, ndmin=2)
    assert np.array_equal(X[Y > 0], Y[Y > 0]) and not Z[Y > 0].any()
    for line in open(prefix + "_post_alpha.txt"):
        whole, frac = line.strip().split(".")
        assert len(frac) == 6


def test_full_size_config1_properties():
    """Config 1 (B=4 x 2500 cells, G=10^4, K=8): size-independent properties."""
    n_b, G, K, seed = [2500] * 4, 10000, 8, 13580
    Y, W_true, _ = bq.simulate(n_b, G, K, seed)
    s = bq.Sampler(Y, n_b, K, seed=seed)
    s.begin(40, 20, 10)
    s.sweeps(40)
    s.finish()
    st = s.get_state()
    e = s.estimates(with_XZ=False)
    s.close()
    _check_invariants(st, Y, np.array(n_b), K)
    assert np.all(np.isfinite(e["alpha"])) and np.all(np.isfinite(e["phi"]))
