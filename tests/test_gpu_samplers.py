"""The device samplers against closed-form distributions and against the FP64
oracle, and the failure path of a sampler cap.

* Gamma (Marsaglia-Tsang, with the U^(1/a) boost below shape 1): KS test
  against scipy's Gamma distribution function.
* Poisson (inversion below 10, PTRS above), NB (CDF inversion for mean < 32
  and size >= 1, Gamma-Poisson otherwise, and each method forced): chi-square
  goodness of fit against the closed-form pmf, tail bins merged so that every
  expected count is at least 5.
* Dirichlet: the pi draw of the sweep (k_sort_pi) repeated at many sweep
  indices from one state; each pi_bk must follow its Beta(c_k + 2,
  sum_j (c_j + 2) - c_k - 2) marginal (KS).
* The same Philox streams drive the oracle's FP64 samplers, so the GPU's
  draws must equal the oracle's except where a single-precision rejection or
  inversion step decides a near-tie the other way (at most 0.1 % of draws).
* A chain whose NB inversion cap is lowered to one step must stop with
  BUSSEQ_ERR_SAMPLER and say which cap was reached, and the process must stay
  able to run the next chain.

Significance: every distribution test rejects at p < 1e-4 (about one false
failure in 10^4 runs per test; the draws are deterministic, so a pass is
reproducible).
"""
import re

import numpy as np
import pytest

import busseq_gpu_gb300 as bq
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
stats = pytest.importorskip("scipy.stats")

P_MIN = 1e-4
N_DRAWS = 200000


def _chi2_discrete(x, pmf, cdf):
    """Chi-square p-value of integer draws x against a pmf, with the lower and
    upper tails merged into bins of expected count >= 5."""
    n = x.size
    lo, hi = int(x.min()), int(x.max())
    ks = np.arange(0, max(hi, 1) + 1)
    exp_ = n * pmf(ks)
    obs = np.bincount(x, minlength=ks.size)[:ks.size].astype(np.float64)
    # merge from the top into the bin below while its expectation is small; the
    # last bin takes the whole upper tail
    tail_hi = n * (1.0 - cdf(ks[-1]))
    exp_[-1] += tail_hi
    e_bins, o_bins = [], []
    e_acc = o_acc = 0.0
    for e, o in zip(exp_, obs):
        e_acc += e
        o_acc += o
        if e_acc >= 5.0:
            e_bins.append(e_acc)
            o_bins.append(o_acc)
            e_acc = o_acc = 0.0
    if e_acc > 0 and e_bins:
        e_bins[-1] += e_acc
        o_bins[-1] += o_acc
    e_bins, o_bins = np.array(e_bins), np.array(o_bins)
    chi2 = ((o_bins - e_bins) ** 2 / e_bins).sum()
    return float(stats.chi2.sf(chi2, df=len(e_bins) - 1)), lo, hi


@pytest.mark.parametrize("a", [0.4, 2.5, 12.0])
def test_gamma_draws(a):
    x = bq.sample_draws("gamma", a, seed=101, n=N_DRAWS).astype(np.float64)
    p = stats.kstest(x, stats.gamma(a).cdf).pvalue
    assert p > P_MIN, (a, p)
    o = po.sample_gamma(101, a, N_DRAWS)
    off = np.abs(x - o) > 2e-5 * np.maximum(o, 1e-30) + 1e-30
    assert off.mean() <= 1e-3, (a, off.mean())


@pytest.mark.parametrize("lam", [3.3, 250.0])
def test_poisson_draws(lam):
    x = bq.sample_draws("poisson", lam, seed=202, n=N_DRAWS)
    p, _, _ = _chi2_discrete(x, stats.poisson(lam).pmf, stats.poisson(lam).cdf)
    assert p > P_MIN, (lam, p)
    o = po.sample_poisson(202, lam, N_DRAWS)
    assert (x != o).mean() <= 1e-3


@pytest.mark.parametrize("kind,mu,phi", [
    ("negbin", 24.0, 3.0),                 # inversion (mean < 32, size >= 1)
    ("negbin", 40.0, 4.0),                 # Gamma-Poisson
    ("negbin", 0.5, 20.0),                 # mostly zeros
    ("negbin", 31.5, 1.0),                 # inversion with a long tail
    ("negbin_gamma_poisson", 24.0, 3.0),   # the other method at the same point
    ("negbin_inversion", 12.0, 1.5),
])
def test_negbin_draws(kind, mu, phi):
    x = bq.sample_draws(kind, mu, phi, seed=303, n=N_DRAWS)
    d = stats.nbinom(phi, phi / (phi + mu))
    p, _, _ = _chi2_discrete(x, d.pmf, d.cdf)
    assert p > P_MIN, (kind, mu, phi, p)
    if kind == "negbin":  # the oracle draws NB as the Z/X update does
        o = po.sample_negbin(303, mu, phi, N_DRAWS)
        assert (x != o).mean() <= 1e-3


def test_dirichlet_draws_of_the_pi_update():
    n_b, G, K, seed = [30, 20], 8, 3, 404
    Y, _, _ = bq.simulate(n_b, G, K, seed)
    s = bq.Sampler(Y, n_b, K, seed=seed)
    try:
        st = s.get_state()
        st["W"] = np.array([0] * 5 + [1] * 10 + [2] * 15 + [0] * 12 + [1] * 2 + [2] * 6, np.int32)
        s.set_state(st)
        draws = []
        for it in range(3000):
            s.run_stage("pi", it)
            draws.append(s.get_state()["pi"].copy())
            s.set_state({"W": st["W"]})
    finally:
        s.close()
    pi = np.array(draws, np.float64)  # [draw][b][k]
    counts = [[5, 10, 15], [12, 2, 6]]
    for b in range(2):
        a = np.array(counts[b], np.float64) + 2.0
        for k in range(K):
            p = stats.kstest(pi[:, b, k], stats.beta(a[k], a.sum() - a[k]).cdf).pvalue
            assert p > P_MIN, (b, k, p)
        np.testing.assert_allclose(pi[:, b].sum(axis=1), 1.0, rtol=1e-5)


def test_sampler_cap_reaches_the_caller():
    """Failure detection without a fault: a lowered NB inversion cap is reached
    on the device, the kernel records it, and busseq_run reports it."""
    n_b, G, K, seed = [40, 30], 200, 3, 505
    Y, _, _ = bq.simulate(n_b, G, K, seed)
    s = bq.Sampler(Y, n_b, K, seed=seed, test_nb_inv_cap=1)
    try:
        with pytest.raises(bq.BusseqError) as e:
            s.run(4, 2, 0)
        assert e.value.code == -5  # BUSSEQ_ERR_SAMPLER
        msg = bq.lib().busseq_last_error().decode()
        m = re.search(r"flags 0x([0-9a-f]+)", msg)
        assert "device-side bound" in msg and m and int(m.group(1), 16) & 4, msg  # bit 4: the NB cap
    finally:
        s.close()
    # the context is still usable: the same chain without the lowered cap runs
    with bq.Sampler(Y, n_b, K, seed=seed) as ok:
        ok.run(4, 2, 0)
