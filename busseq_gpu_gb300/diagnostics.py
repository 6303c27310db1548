"""MCMC diagnostics for the sampler's kept draws (host-side, numpy).

* ``ess_geyer``: effective sample size of each coordinate of a chain by Geyer's
  initial monotone sequence estimator (C. J. Geyer, "Practical Markov chain
  Monte Carlo", Statistical Science 7(4), 1992): with autocorrelations rho_t,
  the sums Gamma_k = rho_{2k} + rho_{2k+1} are kept while positive, made
  non-increasing, and tau = -1 + 2 sum_k Gamma_k; ESS = n / tau (at most
  n log10 n, the cap Stan applies to antithetic chains).  Autocovariances come
  from one FFT per block of coordinates.
* ``adjusted_rand_index``: Hubert and Arabie's adjusted Rand index of two
  labelings, from their contingency table.
"""
from __future__ import annotations

import numpy as np


def ess_geyer(draws: np.ndarray, block: int = 4096) -> np.ndarray:
    """ESS of every row of ``draws`` (coordinates x iterations).  Rows that do
    not move (zero variance) get NaN."""
    x = np.asarray(draws, dtype=np.float64)
    if x.ndim == 1:
        x = x[None, :]
    m, n = x.shape
    out = np.full(m, np.nan)
    if n < 4:
        return out
    nfft = 1 << int(np.ceil(np.log2(2 * n)))
    for r0 in range(0, m, block):
        xb = x[r0:r0 + block]
        xc = xb - xb.mean(axis=1, keepdims=True)
        f = np.fft.rfft(xc, n=nfft, axis=1)
        acov = np.fft.irfft(f * np.conj(f), n=nfft, axis=1)[:, :n] / n
        var = acov[:, 0]
        ok = var > 0
        rho = np.zeros_like(acov)
        rho[ok] = acov[ok] / var[ok, None]
        npairs = n // 2
        gam = rho[:, 0:2 * npairs:2] + rho[:, 1:2 * npairs:2]       # Gamma_k, k = 0 .. npairs-1
        pos = np.cumprod(gam > 0, axis=1).astype(bool)              # initial positive sequence
        mono = np.minimum.accumulate(np.where(pos, gam, np.inf), axis=1)
        s = np.where(pos, mono, 0.0).sum(axis=1)
        tau = -1.0 + 2.0 * s
        tau = np.maximum(tau, 1.0 / np.log10(max(n, 10)))           # ESS <= n log10 n
        e = n / tau
        e[~ok] = np.nan
        out[r0:r0 + block] = e
    return out


def adjusted_rand_index(a, b) -> float:
    """Adjusted Rand index of two labelings of the same items."""
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    if a.size != b.size:
        raise ValueError("labelings differ in length")
    _, ia = np.unique(a, return_inverse=True)
    _, ib = np.unique(b, return_inverse=True)
    table = np.zeros((ia.max() + 1, ib.max() + 1), dtype=np.int64)
    np.add.at(table, (ia, ib), 1)

    def c2(v):
        v = np.asarray(v, dtype=np.float64)
        return (v * (v - 1.0) / 2.0).sum()

    s_ij = c2(table)
    s_a = c2(table.sum(axis=1))
    s_b = c2(table.sum(axis=0))
    total = c2([a.size])
    expected = s_a * s_b / total if total > 0 else 0.0
    max_index = 0.5 * (s_a + s_b)
    if max_index == expected:
        return 1.0
    return float((s_ij - expected) / (max_index - expected))
