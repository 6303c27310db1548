"""Batch-corrected counts on the GPU against the FP64 oracle.

The kernel and the oracle evaluate the same mathematical map (randomised
quantile matching of each imputed count onto NB(exp(alpha + beta_w), phi_1))
by different numerical routes (continued fraction of the incomplete beta and
pmf recurrences on the device; term-by-term summation in the oracle), from
the same estimates and the same 53-bit uniforms.  The counts must agree
exactly, except at a certified near-tie: the two differ by one and the
oracle's probability position lies within TIE of the tail value between
them (relative).  Positions below 1e-280 are floored there on both sides.
"""
import numpy as np
import pytest

import busseq_gpu_gb300 as bq
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

TIE = 1e-8
SEED = 4242


def _compare(got, want, mg, max_ties=3):
    diff = got != want
    if diff.any():
        idx = np.argwhere(diff)
        assert len(idx) <= max_ties, (len(idx), idx[:5], got[diff][:5], want[diff][:5], mg[diff][:5])
        assert np.all(np.abs(got[diff].astype(np.int64) - want[diff]) == 1), (got[diff], want[diff])
        assert np.all(np.abs(mg[diff]) < TIE), mg[diff]
    return int(diff.sum())


def _oracle(h, n_b):
    est = h.estimates(with_XZ=True)
    out, mg = po.corrected_counts(est["X"], n_b, h.seed, est)
    return est, out, mg


def test_after_a_run_matches_oracle():
    n_b, G, K = [60, 45, 70], 300, 4
    Y, _, _ = bq.simulate(n_b, G, K, 11)
    h = bq.Sampler(Y, n_b, K, seed=SEED)
    h.run(40, 20, 10)
    got = h.corrected_counts()
    again = h.corrected_counts()
    est, want, mg = _oracle(h, n_b)
    h.close()
    assert np.array_equal(got, again)  # keyed by the seed: reproducible
    _compare(got, want, mg)
    # the first batch keeps its counts where its cells have no size effect
    assert got.shape == Y.shape and got.min() >= 0


def _crafted(rng, n_b, G, K, effects):
    """Estimates over a wide range: means 0.1 .. 1e4, dispersions 0.3 .. 300
    (p^phi below 1e-304 for the largest), counts in both far tails.  The
    dispersions stay above mean / 300 so that the oracle's term-by-term tail
    sums (about 40 (mean / phi) terms each) stay short."""
    B, N = len(n_b), sum(n_b)
    alpha = np.linspace(-2.0, 9.0, G)
    floor = np.exp(alpha + 2.5) / 300.0
    phi1 = np.maximum(np.exp(rng.uniform(np.log(0.3), np.log(300.0), G)), floor)
    phi = np.repeat(phi1[None], B, axis=0)
    beta = np.zeros((K, G))
    beta[1:] = rng.normal(0, 0.5, (K - 1, G))
    nu = np.zeros((B, G))
    delta = np.zeros(N)
    off = np.concatenate([[0], np.cumsum(n_b)])[:-1]
    if effects:
        nu[1:] = rng.normal(0.7, 0.4, (B - 1, G))
        delta = rng.normal(0, 0.3, N)
        delta[off] = 0
        phi[1:] = np.maximum(phi1[None] * np.exp(rng.normal(0, 0.7, (B - 1, G))), floor[None])
    W = rng.integers(0, K, N).astype(np.int32)
    b_of = np.repeat(np.arange(B), n_b)
    mu = np.exp(alpha[None] + beta[W] + nu[b_of] + delta[:, None])
    ph = phi[b_of]
    X = rng.negative_binomial(ph, ph / (ph + mu)).astype(np.int64)
    # far tails: a few cells get counts many standard deviations out, or zero
    sd = np.sqrt(mu + mu * mu / ph)
    for r in range(0, N, 7):
        X[r] = np.minimum(mu[r] + 12 * sd[r] + 3, 2e6).astype(np.int64)
    for r in range(3, N, 11):
        X[r, ::2] = 0  # (every cell keeps some counts: empty cells are refused)
    X = np.minimum(X, 2_000_000).astype(np.int32)
    st = {"alpha": alpha, "beta": beta, "nu": nu, "delta": delta, "phi": phi, "W": W, "X": X}
    return st


def _sampler_with(st, n_b, K):
    X = st["X"]
    h = bq.Sampler(X, n_b, K, seed=SEED)
    cur = h.get_state()
    cur.update({k: np.asarray(v, cur[k].dtype) for k, v in st.items()})
    cur["Z"] = np.zeros_like(cur["Z"])
    h.set_state(cur)
    return h


@pytest.mark.parametrize("effects", [False, True])
def test_wide_range_matches_oracle(effects):
    rng = np.random.default_rng(5 + effects)
    n_b, G, K = [30, 25, 20], 96, 3
    st = _crafted(rng, n_b, G, K, effects)
    h = _sampler_with(st, n_b, K)
    got = h.corrected_counts()
    est, want, mg = _oracle(h, n_b)
    h.close()
    assert np.array_equal(est["X"], st["X"])
    if not effects:
        # no batch or cell effect: the map is the identity, including the tails
        # whose probability positions stay above 1e-280
        assert np.array_equal(want[mg > 0], st["X"][mg > 0])
    _compare(got, want, mg)


def _scattered(rng, n_b, G, K):
    """Means from 1e-2 to 1e5 with strong batch and cell effects, dispersions
    0.05 .. 1000 (at least mean / 1000), counts scattered over both tails
    (including positions below the 1e-280 floor)."""
    B, N = len(n_b), sum(n_b)
    alpha = rng.uniform(-5, 9, G)
    beta = np.zeros((K, G))
    beta[1:] = rng.normal(0, 1, (K - 1, G))
    nu = np.zeros((B, G))
    nu[1:] = rng.normal(0, 1.5, (B - 1, G))
    off = np.concatenate([[0], np.cumsum(n_b)])[:-1]
    delta = rng.normal(0, 0.8, N)
    delta[off] = 0
    W = rng.integers(0, K, N).astype(np.int32)
    b_of = np.repeat(np.arange(B), n_b)
    mu = np.exp(alpha[None] + beta[W] + nu[b_of] + delta[:, None])
    phi = np.maximum(np.exp(rng.uniform(np.log(0.05), np.log(1000), (B, G))), mu.max(axis=0)[None] / 1000 + 1e-9)
    X = np.round(mu * np.exp(rng.normal(0, 1.5, (N, G)))).astype(np.int64)
    X[rng.random((N, G)) < 0.2] = 0
    X[:, 0] = np.maximum(X[:, 0], 1)  # every cell keeps some counts
    X = np.minimum(X, 3_000_000).astype(np.int32)
    return {"alpha": alpha, "beta": beta, "nu": nu, "delta": delta, "phi": phi, "W": W, "X": X}


def test_scattered_counts_match_oracle():
    rng = np.random.default_rng(101)
    n_b, G, K = [70, 60], 80, 4
    st = _scattered(rng, n_b, G, K)
    h = _sampler_with(st, n_b, K)
    got = h.corrected_counts()
    _, want, mg = _oracle(h, n_b)
    h.close()
    assert (mg < 0).sum() > 0  # the floor is exercised
    _compare(got, want, mg)


def test_device_output_and_cli(tmp_path):
    import os
    import subprocess
    torch = pytest.importorskip("torch")
    n_b, G, K = [30, 25, 20], 120, 3
    Y, _, _ = bq.simulate(n_b, G, K, 99)
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand(99)
    p0 = libc.rand() * 0.5 / 2147483647.0  # the command line's initial p (glibc rand)
    h = bq.Sampler(Y, n_b, K, seed=99, p0=p0)
    h.run(30, 15, 8)
    host = h.corrected_counts()
    dev = torch.empty((sum(n_b), G), dtype=torch.int32, device="cuda")
    h.corrected_counts(out=dev)
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)
    h.close()
    cnt, dim = tmp_path / "counts.txt", tmp_path / "dim.txt"
    np.savetxt(cnt, Y, fmt="%d", delimiter=" ")
    dim.write_text("\n".join(str(x) for x in n_b))
    r = subprocess.run([bq.CLI_PATH, "-B", "3", "-N", str(dim), "-G", str(G), "-K", str(K), "-s", "99", "-c",
                        str(cnt), "-i", "30", "-b", "15", "-u", "8", "-o", str(tmp_path / "out"), "--corrected"],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    path = str(tmp_path / "out") + "_corrected_X.txt"
    assert os.path.exists(path)
    cli = np.loadtxt(path, dtype=np.int64).reshape(sum(n_b), G)
    assert np.array_equal(cli, host)
