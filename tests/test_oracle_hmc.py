"""The FP64 oracle's gradient of the block log posterior (the HMC target), pinned
against central finite differences of its own log posterior (h = 1e-3, FP64),
and the metric's sign and scale (CPU only)."""
import numpy as np
import pytest

import busseq_gpu_gb300 as bq
from oracle import pyoracle as po

N_B, G, K, SEED = [14, 11, 9], 24, 3, 5


@pytest.fixture(scope="module")
def warm():
    Y, _, _ = bq.simulate(N_B, G, K, SEED)
    o = po.State(Y, N_B, K, SEED)
    o.init(0.3)
    for it in range(8):
        o.sweep(it, 4)
    return o


def _coords(o, rng, n):
    """(array name, flat index) of n random free coordinates of each block."""
    off = np.concatenate([[0], np.cumsum(N_B)])
    first = set(off[:-1].tolist())
    out = []
    out += [("alpha", g) for g in rng.choice(G, n, replace=False)]
    out += [("beta", int(k) * G + int(g)) for k, g in zip(rng.integers(1, K, n), rng.choice(G, n))]
    out += [("nu", int(b) * G + int(g)) for b, g in zip(rng.integers(1, len(N_B), n), rng.choice(G, n))]
    out += [("delta", int(i)) for i in rng.choice([i for i in range(sum(N_B)) if i not in first], n, replace=False)]
    out += [("psi", int(b) * G + int(g)) for b, g in zip(rng.integers(0, len(N_B), n), rng.choice(G, n))]
    return out


def test_gradient_matches_central_differences(warm):
    o = warm
    gm = o.hmc_grad()
    rng = np.random.default_rng(0)
    h = 1e-3
    for name, j in _coords(o, rng, 6):
        if name == "psi":
            arr = o.phi.reshape(-1)
            base = arr[j]
            arr[j] = base * np.exp(h)
            fp = o.hmc_logpost()
            arr[j] = base * np.exp(-h)
            fm = o.hmc_logpost()
            arr[j] = base
        else:
            arr = getattr(o, name).reshape(-1)
            base = arr[j]
            arr[j] = base + h
            fp = o.hmc_logpost()
            arr[j] = base - h
            fm = o.hmc_logpost()
            arr[j] = base
        fd = (fp - fm) / (2 * h)
        an = gm["grad"][name].reshape(-1)[j]
        assert abs(fd - an) <= 1e-5 * max(1.0, abs(an)) + 1e-6, (name, j, fd, an)


def test_fixed_coordinates_and_metric(warm):
    o = warm
    gm = o.hmc_grad()
    off = np.concatenate([[0], np.cumsum(N_B)])[:-1]
    assert np.all(gm["grad"]["beta"][0] == 0) and np.all(gm["grad"]["nu"][0] == 0)
    assert np.all(gm["grad"]["delta"][off] == 0)
    for k, m in gm["metric"].items():
        assert np.all(np.isfinite(m)), k
    for k in ("alpha", "beta", "nu", "delta"):
        assert np.all(gm["metric"][k] > 0), k


def test_metric_is_the_negative_hessian_diagonal(warm):
    """The eta-coordinates' metric is the observed information: minus the
    diagonal of the log posterior's Hessian, checked by central differences of
    the oracle's own gradient (alpha_g, beta_gk, nu_bg and delta_i each enter
    their own entries only, so a one-coordinate difference is the diagonal)."""
    o = warm
    gm = o.hmc_grad()
    rng = np.random.default_rng(3)
    h = 1e-4
    for name, j in _coords(o, rng, 5):
        if name == "psi":
            continue
        arr = getattr(o, name).reshape(-1)
        base = arr[j]
        arr[j] = base + h
        gp = o.hmc_grad()["grad"][name].reshape(-1)[j]
        arr[j] = base - h
        gmn = o.hmc_grad()["grad"][name].reshape(-1)[j]
        arr[j] = base
        hess = -(gp - gmn) / (2 * h)
        m = gm["metric"][name].reshape(-1)[j]
        assert abs(hess - m) <= 1e-4 * abs(m) + 1e-6, (name, j, hess, m)
