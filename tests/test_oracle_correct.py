"""The FP64 oracle of the batch-corrected counts (randomised quantile matching
from NB(mu, phi_b) to NB(exp(alpha + beta_w), phi_1)), pinned three ways on
the CPU:

* without batch or cell effects the map is the identity, entry for entry;
* against scipy.stats.nbinom: the same uniform v gives u = F(x-1) + v P(x)
  and x* = min {k : F*(k) >= u}; disagreements only where the oracle's
  position lies within 1e-9 (relative) of a tail value;
* the corrected counts of one batch with strong effects follow the target
  distribution NB(mu*, phi_1) (mean, variance and a chi-square fit).
"""
import numpy as np
import pytest

from oracle import pyoracle as po

SEED = 77


def _words(seed, entity):
    ctr = [entity & 0xFFFFFFFF, ((entity >> 32) & 0xFFFF) | (17 << 16), 0, 0]
    r = po.philox(ctr, (seed & 0xFFFFFFFF, seed >> 32))
    return r[0], r[1]


def _v(seed, entity):
    w0, w1 = _words(seed, entity)
    m = ((w0 << 32) | w1) >> 12
    return (2 * m + 1) * 2.0 ** -53


def _est(n_b, G, K, rng, effects=True):
    B, N = len(n_b), sum(n_b)
    est = {"alpha": rng.uniform(0.0, 3.0, G), "beta": np.zeros((K, G)), "nu": np.zeros((B, G)),
           "delta": np.zeros(N), "phi": np.repeat(rng.uniform(2.0, 20.0, (1, G)), B, axis=0),
           "W": rng.integers(0, K, N).astype(np.int32)}
    est["beta"][1:] = rng.normal(0.0, 1.0, (K - 1, G))
    if effects:
        est["nu"][1:] = rng.normal(0.5, 0.5, (B - 1, G))
        est["delta"] = rng.normal(0.0, 0.3, N)
        off = np.concatenate([[0], np.cumsum(n_b)])[:-1]
        est["delta"][off] = 0.0
        est["phi"] = rng.uniform(1.0, 30.0, (B, G))
    return est


def _means(n_b, est):
    b_of = np.repeat(np.arange(len(n_b)), n_b)
    ab = est["alpha"][None, :] + est["beta"][est["W"]]
    mu = np.exp(ab + est["nu"][b_of] + est["delta"][:, None])
    return b_of, mu, np.exp(ab)


def _draw(n_b, est, rng):
    b_of, mu, _ = _means(n_b, est)
    ph = est["phi"][b_of]
    return rng.negative_binomial(ph, ph / (ph + mu)).astype(np.int32)


def test_identity_without_batch_effects():
    rng = np.random.default_rng(1)
    n_b, G, K = [40, 30, 30], 50, 3
    est = _est(n_b, G, K, rng, effects=False)
    X = _draw(n_b, est, rng)
    X[0, :4] = [0, 1, 150, 300]  # far tails too (positions down to ~1e-170; below 1e-280 they saturate)
    out, mg = po.corrected_counts(X, n_b, SEED, est)
    assert np.array_equal(out, X)
    assert np.all(mg > 0)


def test_matches_scipy_quantiles():
    stats = pytest.importorskip("scipy.stats")
    rng = np.random.default_rng(2)
    n_b, G, K = [30, 20, 25], 40, 4
    est = _est(n_b, G, K, rng)
    X = _draw(n_b, est, rng)
    out, mg = po.corrected_counts(X, n_b, SEED, est)
    b_of, mu, mus = _means(n_b, est)
    N = sum(n_b)
    checked = 0
    for i in range(N):
        for g in range(G):
            ph, ph1 = est["phi"][b_of[i], g], est["phi"][0, g]
            p, p1 = ph / (ph + mu[i, g]), ph1 / (ph1 + mus[i, g])
            x = int(X[i, g])
            v = _v(SEED, i * G + g)
            u = stats.nbinom.cdf(x - 1, ph, p) + v * stats.nbinom.pmf(x, ph, p)
            if u > 1 - 1e-9:
                continue  # scipy works on the lower tail only
            want = int(stats.nbinom.ppf(u, ph1, p1))
            # ppf may round a hair either way; the exact condition decides
            while want > 0 and stats.nbinom.cdf(want - 1, ph1, p1) >= u:
                want -= 1
            while stats.nbinom.cdf(want, ph1, p1) < u:
                want += 1
            if out[i, g] != want:
                assert abs(int(out[i, g]) - want) == 1 and mg[i, g] < 1e-9, (i, g, out[i, g], want, mg[i, g])
            checked += 1
    assert checked > 0.99 * N * G


def test_corrected_batch_follows_target():
    stats = pytest.importorskip("scipy.stats")
    rng = np.random.default_rng(3)
    n_b, G, K = [50, 20000], 1, 2
    est = {"alpha": np.array([2.0]), "beta": np.zeros((K, G)), "nu": np.array([[0.0], [1.2]]),
           "delta": np.concatenate([[0.0], rng.normal(0, 0.2, 49), [0.0], rng.normal(0, 0.2, 19999)]),
           "phi": np.array([[10.0], [3.0]]), "W": np.zeros(sum(n_b), np.int32)}
    X = _draw(n_b, est, rng)
    out, _ = po.corrected_counts(X, n_b, SEED, est)
    y = out[50:, 0].astype(np.float64)
    mus, ph1 = np.exp(2.0), 10.0
    n = y.size
    assert abs(y.mean() - mus) < 4 * np.sqrt((mus + mus ** 2 / ph1) / n)
    var = mus + mus ** 2 / ph1
    assert abs(y.var() - var) < 0.06 * var
    # chi-square over the bins 0..29 and >= 30
    p1 = ph1 / (ph1 + mus)
    probs = np.append(stats.nbinom.pmf(np.arange(30), ph1, p1), stats.nbinom.sf(29, ph1, p1))
    obs = np.append(np.bincount(np.minimum(y.astype(int), 30), minlength=31)[:30], np.sum(y >= 30))
    chi2 = np.sum((obs - n * probs) ** 2 / (n * probs))
    assert chi2 < stats.chi2.ppf(0.999, 30)
    # before correction the batch is visibly off target
    assert X[50:, 0].mean() > 2 * mus
